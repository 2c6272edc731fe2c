// Host-visible declarations of the wavefront kernels' launch wrappers and the
// queue / job structures they share with the C ABI layer.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "device.cuh"

namespace turner {

// SoA ray queue (one entry per live path at one depth).
struct RayQueue {
    float4* o;        // origin xyz, chunk-local path index (uint bits) in w
    float4* d;        // direction xyz, job index (uint bits) in w
    float4* T;        // path throughput (RGBA)
    uint2* rng;       // bounce stream state
    uint32_t* count;  // number of valid entries (device)
    uint32_t* rec;    // training record of the bounce that spawned the ray, or kNoRecord (may be null)
};

constexpr uint32_t kNoRecord = 0xFFFFFFFFu;
constexpr int kSamplingGuided = 2;   // TURNER_SAMPLING_GUIDED

// Learned-proposal data per ray-queue slot (guided jobs only).
struct GuideQueue {
    float* feat;      // 9 floats: position in [0,1]^3 (scene box), shading normal, albedo
    float* out;       // 40 floats: mixture parameters from the network
};

// Training samples recorded at guided bounces during a pass.
struct Records {
    float* feat;      // 9 per record (network input)
    float* dir;       // 3 per record (sampled direction)
    float* weight;    // target weight, filled after the pass
    uint32_t* path;   // chunk-local path index
    float* l_before;  // luminance of the path's radiance before the bounce's continuation
    float* t_after;   // luminance of the throughput after the bounce
    float* fcos_pdf;  // luminance of f cos / p for the bounce
    uint32_t* count;
    uint32_t cap;
    uint32_t keep;    // record a bounce when its stream's next 32 bits are below keep
};

// Shadow-ray queue: one entry per hit with the light in front of the surface.
struct ShadowQueue {
    float4* o;        // offset hit point p2, chunk-local path index in w
    float4* d;        // unit light direction, distance to the light in w
    float4* c;        // contribution added to the path if the light is visible
    uint32_t* job;    // job index
    uint32_t* count;
    uint32_t* aux;    // batches with raytracer jobs: kAuxPath, kAuxNoChild or the
                      // queue slot of the mirror ray spawned at the same hit
};

constexpr uint32_t kAuxPath = 0xFFFFFFFEu;      // path-tracer entry: a blocked ray adds nothing
constexpr uint32_t kAuxNoChild = 0xFFFFFFFFu;   // raytracer entry without a mirror ray
constexpr int kRendererPath = 0, kRendererRaytrace = 1, kRendererRaycast = 2;

// One image of a batch, resident in device memory (the job table).
struct JobDesc {
    SceneView sc;
    float cam_pos[3];
    float trafo[9];
    float delta_x, delta_y;
    uint32_t width, height, spp;   // height: the whole image's (the camera's raster)
    uint32_t row0, rows;           // the band rendered: rows [row0, row0 + rows)
    int32_t max_depth, mc;
    float bg[3];
    uint64_t seed;
    int32_t n_lights;
    float light_pos[3];
    float light_col[4];
    int32_t sampling, traversal;
    int32_t guide_depth;     // guided jobs: hits at depth < guide_depth sample from the proposal, deeper ones by cosine
    float exposure, inv_gamma;
    int32_t gamma, tone_map;
    int32_t renderer;
    float shadow_intensity, max_visibility;
    uint64_t pixel_offset;   // first pixel of this job in the batch's pixel space
    uint64_t path_offset;    // first path of this job in the batch's path space
    float4* out;             // output image (device)
};

// A render pass: whole pixels [pixel0, pixel0 + n_pixels) of the batch's
// pixel space, which are paths [path0, path0 + n_paths). With -m = M > 1 a
// path has up to M^max_depth rays at its widest level, so the queues hold
// n_rays entries.
struct Chunk {
    uint64_t pixel0, path0;
    uint32_t n_pixels, n_paths;
    uint32_t n_rays;   // bound on the rays of one level (n_paths unless -m > 1 branches)
};

// How traversal kernels are launched. persistent: one grid of resident
// blocks whose lanes pull rays from `work` (a zeroed device counter) until the
// queue is empty; otherwise one thread per queue slot.
struct TraverseCfg {
    bool persistent = true;
    unsigned blocks_per_sm = 0;   // 0: as many as are resident
    unsigned block = 128;         // threads per block of the persistent kernels: 128 or 256
    unsigned stack = kStackCap;   // traversal stack entries: 64 or kStackCap (128)
    bool mailbox = false;         // skip repeated tests of a triangle (128-thread blocks)
    unsigned min_blocks = 10;     // 10, 12, 16: cap registers so that many blocks fit per SM (128-thread
                                  // blocks); 0: no cap. 10 (48 registers) is fastest on GB300
    unsigned refill = 1;          // persistent: a warp takes new rays once this many lanes are idle (1..32)
    bool packet = false;          // warps of fresh rays with one direction octant traverse as packets
                                  // (128-thread blocks, 10 per SM, no mailbox, not FAST); results unchanged
    bool speculative = false;     // speculative traversal rounds (128-thread blocks, 10 per SM, no mailbox,
                                  // not FAST); results are unchanged
    unsigned ring = 0;            // 4 or 8: the stack's newest entries in shared memory (128-thread blocks,
                                  // 10 per SM, no mailbox); 0: the whole stack in local memory
    uint32_t* work = nullptr;
};

void launch_intersect(const SceneView& sc, const float* ox, const float* oy, const float* oz, const float* dx,
                      const float* dy, const float* dz, uint64_t n, uint32_t* id, float* r, float* s, float* t,
                      int fast, const TraverseCfg& cfg, cudaStream_t stream);

// Any-hit occlusion of SoA rays: blocked[i] = 1 iff some triangle of a leaf the
// ray's traversal visits has a valid intersection with r <= tmax[i]. Persistent
// launch; cfg.work must be a zeroed device counter.
void launch_occluded(const SceneView& sc, const float* ox, const float* oy, const float* oz, const float* dx,
                     const float* dy, const float* dz, const float* tmax, uint32_t n, uint8_t* blocked,
                     const TraverseCfg& cfg, cudaStream_t stream);

// Gather-bandwidth probe: blocks x 256 threads, each making loads_per_thread
// (a multiple of 8) independent loads of load_bytes (8 or 32) at random
// positions in buf (buf_bytes / load_bytes a power of two, buf 32-byte
// aligned); out receives one word per thread.
void launch_gather_probe(const void* buf, uint64_t buf_bytes, int load_bytes, uint32_t loads_per_thread,
                         uint32_t seed, uint32_t* out, unsigned blocks, cudaStream_t stream);

// `single` is the scene of every job when the batch has one scene (rays then
// skip the per-ray job-table lookup); nullptr for multi-scene batches.
void launch_camera(const JobDesc* jobs, uint32_t n_jobs, const Chunk& c, const RayQueue& q, float4* L,
                   cudaStream_t stream);
void launch_trace(const SceneView* single, const JobDesc* jobs, const RayQueue& q, Hit* hits, uint32_t capacity,
                  int fast, const TraverseCfg& cfg, cudaStream_t stream);
// job_counts (optional): per job {traced rays, shadow rays}, 64-bit.
// gq / recs: learned-proposal inputs and training records (null pointers
// when no job of the batch samples with the learned proposal).
void launch_shade(const JobDesc* jobs, int depth, const RayQueue& in, const Hit* hits, const RayQueue& out,
                  const ShadowQueue& sh, float4* L, unsigned long long* job_counts, const GuideQueue& gq,
                  const Records& recs, uint32_t capacity, bool mixed, cudaStream_t stream);
// Network inputs for the hits of guided jobs that will bounce (zeros elsewhere).
// The raytracer's and raycaster's shading (raytracer.cpp:5-67,
// raycaster.cpp:6-24) of the entries of their jobs; k_shade skips those.
void launch_shade_classic(const JobDesc* jobs, int depth, const RayQueue& in, const Hit* hits, const RayQueue& out,
                          const ShadowQueue& sh, float4* L, unsigned long long* job_counts, uint32_t capacity,
                          cudaStream_t stream);
void launch_guide_features(const JobDesc* jobs, int depth, const RayQueue& q, const Hit* hits, float* feat,
                           uint32_t capacity, cudaStream_t stream);
// atomic_l: add to L atomically (batches with -m > 1, where several shadow
// rays of one path are in the queue at once). next_T: throughput of the next
// ray queue, which blocked raytracer shadow rays darken (sh.aux non-null).
void launch_shadow(const SceneView* single, const JobDesc* jobs, const ShadowQueue& sh, float4* L, uint32_t capacity,
                   bool atomic_l, float4* next_T, const TraverseCfg& cfg, cudaStream_t stream);
void launch_resolve(const JobDesc* jobs, uint32_t n_jobs, const Chunk& c, const float4* L, cudaStream_t stream);
// acc[p] += (double) sum of the chunk's sample radiance for pixel p (linear)
void launch_accumulate(const JobDesc* jobs, uint32_t n_jobs, const Chunk& c, const float4* L, double4* acc,
                       cudaStream_t stream);

} // namespace turner

struct turner_guide;
struct turner_ctx;

namespace turner {
namespace guide {
// Host entry points of guide.cu used by the render loop (all asynchronous on
// `stream` except train_device's optional loss readback).
int forward_queue(turner_guide* g, const float* feat, const uint32_t* n_dev, uint32_t cap, float* out,
                  cudaStream_t stream);
int finalize_records(const uint32_t* count, uint32_t cap, const float4* L, const uint32_t* path,
                     const float* l_before, const float* t_after, const float* fcos_pdf, float* weight, int mode,
                     cudaStream_t stream);
// One Adam step on n samples, or on min(n, *n_dev) when n_dev is given; a
// step with fewer than min_n samples changes nothing. Asynchronous unless
// loss_out is given (then it waits and writes the step's mean loss).
int train_device(turner_guide* g, const float* feat, const float* dirs, const float* wts, uint32_t n,
                 const uint32_t* n_dev, uint32_t min_n, float lr, cudaStream_t stream, float* loss_out);
// Adam steps taken and the last step's mean loss (waits for the stream).
int train_state(turner_guide* g, uint64_t* steps, float* last_loss);
// The context a proposal was created on (null once that context is destroyed).
turner_ctx* owner(const turner_guide* g);
// Called by turner_destroy for each proposal still alive: drops the context
// and its stream, so that the proposal accepts turner_guide_destroy only.
void orphan(turner_guide* g);
} // namespace guide
} // namespace turner
