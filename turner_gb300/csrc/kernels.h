// Host-visible declarations of the wavefront kernels' launch wrappers and the
// queue / job structures they share with the C ABI layer.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "device.cuh"

namespace turner {

// SoA ray queue (one entry per live path at one depth).
struct RayQueue {
    float4* o;        // origin xyz, path index (uint bits) in w
    float4* d;        // direction xyz
    float4* T;        // path throughput (RGBA)
    uint2* rng;       // bounce stream state
    uint32_t* count;  // number of valid entries (device)
};

// Shadow-ray queue: one entry per hit with a light in front of the surface.
struct ShadowQueue {
    float4* o;        // offset hit point p2, path index in w
    float4* d;        // unit light direction, distance to the light in w
    float4* c;        // contribution added to the path if the light is visible
    uint32_t* count;
};

// Everything a render pass needs about one job, by value in kernel params.
struct JobDev {
    SceneView sc;
    float cam_pos[3];
    float trafo[9];
    float delta_x, delta_y;
    uint32_t width, height, spp;
    int32_t max_depth, mc;
    float bg[3];
    uint64_t seed;
    int32_t n_lights;
    float light_pos[3];
    float light_col[4];
    int32_t sampling, traversal;
    float exposure, inv_gamma;
    int32_t gamma, tone_map;
};

// How traversal kernels are launched. persistent: one grid of resident
// blocks whose lanes pull rays from `work` (a zeroed device counter) until the
// queue is empty; otherwise one thread per queue slot.
struct TraverseCfg {
    bool persistent = true;
    unsigned blocks_per_sm = 0;   // 0: as many as are resident
    uint32_t* work = nullptr;
};

void launch_intersect(const SceneView& sc, const float* ox, const float* oy, const float* oz, const float* dx,
                      const float* dy, const float* dz, uint64_t n, uint32_t* id, float* r, float* s, float* t,
                      int fast, const TraverseCfg& cfg, cudaStream_t stream);
void launch_camera(const JobDev& job, uint32_t first_pixel, uint32_t n_paths, const RayQueue& q, float4* L,
                   cudaStream_t stream);
void launch_trace(const SceneView& sc, const RayQueue& q, Hit* hits, uint32_t capacity, int fast,
                  const TraverseCfg& cfg, cudaStream_t stream);
void launch_shade(const JobDev& job, int depth, const RayQueue& in, const Hit* hits, const RayQueue& out,
                  const ShadowQueue& sh, float4* L, uint32_t capacity, cudaStream_t stream);
void launch_shadow(const SceneView& sc, const ShadowQueue& sh, float4* L, uint32_t capacity, const TraverseCfg& cfg,
                   cudaStream_t stream);
void launch_resolve(const JobDev& job, uint32_t first_pixel, uint32_t n_pixels, const float4* L, float4* out,
                    cudaStream_t stream);

} // namespace turner
