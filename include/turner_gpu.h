/*
 * turner_gpu.h — C ABI of the GB300 path-tracing core.
 *
 * Plain C: opaque handles, plain pointers and sizes, int status codes, no
 * exceptions and no C++ or torch types cross it. One context owns device
 * memory and one CUDA stream on one GPU; calls on a context come from one
 * host thread at a time.
 *
 * What it replaces in the reference (turner-renderer/turner):
 *   - the render block of main.cpp:181-236 (row thread pool, pixel/sample
 *     loops, per-pixel mean, exposure, gamma) together with the per-ray
 *     renderer plug-in `Color trace(const Ray&, KDTreeIntersection&,
 *     const std::vector<Light>&, int depth, const TracerConfig&)`
 *     (trace.h:23-25, defined in pathtracer.cpp:14-102)   -> turner_render
 *   - `const OptionalId KDTreeIntersection::intersect(const Ray&, float& r,
 *     float& a, float& b)` (lib/kdtree.h:291, lib/kdtree.cpp:516-607),
 *     batched                                             -> turner_intersect
 *   - the kd-tree produced by `KDTree::KDTree(Triangles)` (lib/kdtree.cpp:474-490)
 *     is consumed verbatim: FlatNode words and the precomputed Triangle fields,
 *     in the order KDTree::serialize / Triangle::serialize emit them
 *     (lib/kdtree.h:228-230, lib/triangle.h:89-92)        -> turner_upload_scene
 *   - `KDTree::KDTree(Triangles)` itself, re-implemented on the host with the
 *     same node output                                   -> turner_kdtree_build
 */
#ifndef TURNER_GPU_H
#define TURNER_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
#define TURNER_OK 0
#define TURNER_ERR_INVALID_ARG (-1)   /* null pointer, zero size, bad enum      */
#define TURNER_ERR_CUDA (-2)          /* a CUDA runtime call failed             */
#define TURNER_ERR_OUT_OF_MEMORY (-3) /* device or host allocation failed       */
#define TURNER_ERR_BAD_SCENE (-4)     /* node array fails validation            */
#define TURNER_ERR_TIMEOUT (-5)       /* a bounded device wait gave up          */
#define TURNER_ERR_DEVICE_BOUNDS (-6) /* a device-side index check fired        */
#define TURNER_ERR_UNSUPPORTED (-7)   /* valid but not implemented combination  */
#define TURNER_ERR_NO_DEVICE (-8)     /* no CUDA device / wrong architecture    */
#define TURNER_ERR_TOO_LARGE (-9)     /* request exceeds a documented maximum   */

/* Triangle id returned for a miss: detail::OptionalId's invalid value
 * FlatNode::MAX_TRIANGLE_ID = 1 << 30 (lib/kdtree.h:66,156-160). */
#define TURNER_MISS 0x40000000u

/* Pointer placement flags for turner_intersect / turner_render. */
#define TURNER_HOST_BUFFERS 0u   /* arrays are host memory; copies are made  */
#define TURNER_DEVICE_BUFFERS 1u /* arrays are device memory of this context's GPU */

/* Traversal modes. PARITY reproduces KDTreeIntersection::intersect exactly:
 * every overlapped leaf is visited, first strict minimum kept. FAST stops
 * once no later cell can hold a closer hit (checked against PARITY by the
 * tests). Shadow rays always stop at the first blocker; that is exact. */
#define TURNER_TRAVERSAL_PARITY 0
#define TURNER_TRAVERSAL_FAST 1

/* Bounce sampling. UNIFORM is the reference's sampling::hemisphere
 * (lib/sampling.h:20-32, weight 2*cos); COSINE is cosine-weighted. */
#define TURNER_SAMPLING_UNIFORM 0
#define TURNER_SAMPLING_COSINE 1
/* GUIDED: the context's learned proposal (turner_set_guide), mixed 1/2 with
 * cosine sampling so the pdf stays positive on the hemisphere; estimator
 * f cos / p. No reference counterpart. */
#define TURNER_SAMPLING_GUIDED 2

/* ------------------------------------------------------------- records */

/* One triangle in Triangle::serialize order (lib/triangle.h:89-114):
 * 48 floats = 192 bytes. `u`, `v`, `normal`, `uv`, `vv`, `uu`, `denom` are
 * the constructor's precomputed values (lib/triangle.h:22-39); pass them as
 * the reference computed them for bit-exact hits. */
typedef struct turner_triangle {
    float vertices[3][3];
    float normals[3][3];
    float ambient[4];
    float diffuse[4];
    float emissive[4];
    float reflective[4];
    float reflectivity;
    float u[3];
    float v[3];
    float normal[3];
    float uv, vv, uu, denom;
} turner_triangle;

/* Pinhole camera of lib/types.h:88-123. The camera looks down -z of its node
 * frame; `trafo` is the node's rotation (row-major a1..c3), `position` the
 * node's translation. Primary directions are NOT normalised (raster2cam). */
typedef struct turner_camera {
    float position[3];
    float trafo[9];
    float delta_x; /* tan(aiCamera::mHorizontalFOV), as Camera computes it */
    float aspect;  /* aiCamera::mAspect; delta_y = delta_x / aspect        */
} turner_camera;

/* Point light (lib/types.h:81-84). No distance falloff, as in the reference. */
typedef struct turner_light {
    float position[3];
    float color[4];
} turner_light;

/* One image to render: the TracerConfig fields of config.h:13-165 that the
 * path tracer reads, plus the scene, camera, light and seed. */
typedef struct turner_job {
    uint32_t scene_id;
    uint32_t width;               /* -w                                       */
    uint32_t height;              /* the reference uses int(width / aspect)   */
    uint32_t pixel_samples;       /* -p                                       */
    int32_t max_depth;            /* -d: rays are traced at depths 0..max_depth */
    int32_t monte_carlo_samples;  /* -m: bounce rays per hit (0..TURNER_MAX_MC). With
                                     M > 1 (pathtracer.cpp:72-88) child k of a hit
                                     draws from its own stream, derived from its
                                     parent's (a wavefront cannot follow the
                                     reference's depth-first draws); a path has up
                                     to M^max_depth rays at its widest level, and
                                     passes shrink to fit them (at most 2^26 per
                                     path: TURNER_ERR_TOO_LARGE). Not with GUIDED. */
    float exposure;               /* --exposure                               */
    float inverse_gamma;          /* --inverse-gamma                          */
    int32_t gamma_correction;     /* 0 for --no-gamma-correction              */
    float background[3];          /* --background; alpha is 1                 */
    uint64_t seed;                /* per-(pixel, sample) stream seed base     */
    int32_t n_lights;             /* 0 or 1 (main.cpp:121-136 allows at most 1) */
    turner_light light;
    turner_camera camera;
    int32_t sampling;             /* TURNER_SAMPLING_*                        */
    int32_t traversal;            /* TURNER_TRAVERSAL_* for bounce rays; a batch
                                     uses FAST only if every job asks for it  */
    int32_t linear_output;        /* 1: write the per-pixel mean radiance
                                     without exposure and gamma (for error
                                     measurements against converged images) */
    int32_t renderer;             /* TURNER_RENDERER_*: which trace() plug-in */
    float shadow_intensity;       /* raytracer --shadow (config.h: 0.5)       */
    float max_visibility;         /* raycaster --max-visibility (config.h: 2) */
    /* Image rows [row_begin, row_end) to render; row_end = 0 means height.
     * The reference's unit of work is one image row (main.cpp:193-226); a
     * band is what one GPU of a row-partitioned frame renders. The camera
     * and every (pixel, sample) stream use the pixel's place in the whole
     * image, so a band is bit-identical to the same rows of a full render.
     * The output then holds only the band: width * (row_end - row_begin)
     * pixels, its first row being row_begin. */
    uint32_t row_begin;
    uint32_t row_end;
} turner_job;

/* The reference links one trace() per executable (trace.h:23-25):
 *   PATH      pathtracer.cpp:14-102 (default)
 *   RAYTRACE  raytracer.cpp:5-67: Lambertian direct light, mirror bounces
 *             up to max_depth, shadows darken by shadow_intensity; needs
 *             exactly one light (the reference reads lights.front())
 *   RAYCAST   raycaster.cpp:6-24: diffuse colour, alpha = 1 - r /
 *             max_visibility clamped to [0, 1]; only hits count as rays
 * RAYTRACE and RAYCAST ignore sampling and monte_carlo_samples. */
#define TURNER_RENDERER_PATH 0
#define TURNER_RENDERER_RAYTRACE 1
#define TURNER_RENDERER_RAYCAST 2

/* Largest -m. */
#define TURNER_MAX_MC 64

/* Jobs per turner_render call. */
#define TURNER_MAX_JOBS 4096

typedef struct turner_stats {
    uint64_t rays;          /* reference count: traced rays at depth <= max_depth,
                               misses included, shadow rays excluded (pathtracer.cpp:21) */
    uint64_t primary_rays;  /* main.cpp:211                                */
    uint64_t shadow_rays;   /* one per hit with a light                    */
    double device_ms;       /* device time of the render, CUDA events      */
} turner_stats;

typedef struct turner_ctx turner_ctx;
typedef struct turner_kdtree turner_kdtree;
typedef struct turner_mesh turner_mesh;

/* ------------------------------------------------------------ context */
const char* turner_strerror(int status);
int turner_create(turner_ctx** out, int device);
void turner_destroy(turner_ctx* ctx);
/* Last device-side error word (TURNER_ERR_* or 0) and clears it. */
int turner_last_device_error(turner_ctx* ctx);
/* Text of the last failing CUDA call on this context ("" if none). No
 * reference counterpart: diagnostics of this library. */
const char* turner_last_error_message(turner_ctx* ctx);
/* Number of kernels this context has launched so far. No reference
 * counterpart: lets benchmarks report how much work ran on the GPU. */
uint64_t turner_launch_count(turner_ctx* ctx);
/* Paths in flight per render pass (queue length), >= 1024. Default 2^24.
 * No reference counterpart: the reference renders one row per task. */
int turner_set_chunk_paths(turner_ctx* ctx, uint32_t paths);
/* Traversal launch shape. persistent != 0 (default): resident blocks whose
 * lanes take a new ray as soon as their current one finishes; blocks_per_sm
 * caps the resident blocks (0 = occupancy limit, at most 64). persistent == 0:
 * one thread per ray. No reference counterpart: tuning knob of this library. */
int turner_set_traversal_launch(turner_ctx* ctx, int persistent, uint32_t blocks_per_sm);

/* Gather-bandwidth roof of the traversal: times a kernel that makes
 * independent loads of load_bytes (8: one node word; 32: one half of a
 * triangle record) at random positions in a buffer of buffer_bytes (a power
 * of two, at least 4096; 64 MiB fits in L2 as the large-mesh scene does),
 * best of `repeats` launches after a warm-up launch, CUDA events; *gbs =
 * bytes loaded / time. Allocates and frees its buffer. No reference
 * counterpart: the roof against which traversal throughput is reported. */
int turner_probe_gather(turner_ctx* ctx, uint64_t buffer_bytes, uint32_t load_bytes, uint32_t repeats, double* gbs);

/* Refill threshold of the persistent traversal, per kind of ray: a warp
 * takes new rays only once `lanes` (1..32) of its 32 lanes are idle. 1
 * keeps the most lanes busy; 32 takes rays a whole warp at a time, so that
 * neighbouring rays of a coherent queue stay in one warp and share their
 * node and triangle loads. Defaults: 32 for camera rays and their shadow
 * rays (a warp holds 32 samples of neighbouring pixels), 2 for bounce rays,
 * 4 for their shadow rays, 1 for turner_intersect / turner_occluded.
 * Results do not depend on it. No reference counterpart: tuning knob of
 * this library. */
#define TURNER_RAYS_PRIMARY 0         /* camera rays (depth 0)                  */
#define TURNER_RAYS_BOUNCE 1          /* bounce rays (depth >= 1)               */
#define TURNER_RAYS_SHADOW_PRIMARY 2  /* shadow rays from camera-ray hits       */
#define TURNER_RAYS_SHADOW 3          /* shadow rays from bounce-ray hits       */
#define TURNER_RAYS_INTERSECT 4       /* turner_intersect and turner_occluded   */
#define TURNER_RAYS_KINDS 5
int turner_set_traversal_refill(turner_ctx* ctx, int kind, uint32_t lanes);
/* Where the persistent traversal keeps its stack: entries = 4 or 8 puts each
 * thread's newest entries in shared memory ([slot][thread] words, so lanes
 * at different depths never share a bank) and moves older ones to local
 * memory; 0 (default) keeps the whole stack in local memory. Applies to the
 * default launch shape (128-thread blocks, 10 per SM, no mailbox). Results
 * do not depend on it. No reference counterpart: the reference's stack is a
 * heap std::stack (lib/kdtree.cpp:522-560). */
int turner_set_traversal_ring(turner_ctx* ctx, uint32_t entries);
/* on != 0: speculative traversal rounds (Aila & Laine 2009): a lane that has
 * found a leaf sets its triangle run aside and descends on toward the next
 * leaf while other lanes of its warp are still searching, then the warp tests
 * the runs set aside together. Leaf runs are still tested in the reference's
 * order, so results do not change. Applies to the default launch shape and
 * PARITY / shadow traversal (not FAST). Default off. No reference
 * counterpart: tuning knob of this library. */
int turner_set_traversal_speculative(turner_ctx* ctx, int on);
/* Packet traversal: a warp whose rays were all just taken, share their
 * direction signs and their scene walks the tree as one: a cell is entered
 * when some lane's interval overlaps it, each lane tests exactly the leaf
 * runs its own traversal would, in the same order, and node words and
 * triangle records are loaded once for the warp. Results do not change.
 * mode is a mask: TURNER_PACKET_CAMERA (default) for the camera rays of
 * renders (warps of neighbouring samples), TURNER_PACKET_BATCHED for every
 * qualifying warp of turner_intersect, turner_occluded and
 * turner_intersect_noalloc; 0 turns packets off. No reference counterpart:
 * tuning knob of this library. */
#define TURNER_PACKET_CAMERA 1
#define TURNER_PACKET_BATCHED 2
int turner_set_traversal_packet(turner_ctx* ctx, int mode);

/* Per-kernel device time, measured with CUDA events on the context stream
 * around every launch while profiling is on. No reference counterpart: the
 * reference only has Runtime wall-clock timers (lib/runtime.h). */
#define TURNER_KERNEL_CAMERA 0
#define TURNER_KERNEL_TRACE 1     /* closest-hit traversal of a ray queue  */
#define TURNER_KERNEL_SHADE 2
#define TURNER_KERNEL_SHADOW 3    /* any-hit traversal of the shadow queue */
#define TURNER_KERNEL_RESOLVE 4
#define TURNER_KERNEL_INTERSECT 5
#define TURNER_KERNEL_GUIDE_FEATURES 6   /* network inputs of guided hits */
#define TURNER_KERNEL_MLP_FORWARD 7      /* tcgen05 inference of the learned proposal */
#define TURNER_KERNEL_GUIDE_TRAIN 8      /* record weights + one training step (timed always) */
#define TURNER_KERNEL_KINDS 9
int turner_set_profiling(turner_ctx* ctx, int on);
/* Copies the accumulated milliseconds and launch counts per kind (arrays of
 * TURNER_KERNEL_KINDS; either may be NULL) and optionally resets them. */
int turner_kernel_times(turner_ctx* ctx, double* ms, uint64_t* launches, int reset);

/* --------------------------------------------------------------- scene */
/* Copies a flattened kd-tree to the device. `nodes` are FlatNode::data_
 * words (lib/kdtree.h:136-153) in the reference's DFS order; `box` is
 * KDTree::box() as {min x,y,z, max x,y,z}. The node array is validated on
 * the host (child indices forward and in range, leaf ids < n_tris, every
 * leaf run terminated inside the array) so that device traversal is in
 * bounds by construction; a failing array returns TURNER_ERR_BAD_SCENE. */
int turner_upload_scene(turner_ctx* ctx, const uint64_t* nodes, uint32_t n_nodes, const turner_triangle* tris,
                        uint32_t n_tris, const float box[6], uint32_t* scene_id);
int turner_free_scene(turner_ctx* ctx, uint32_t scene_id);
/* The host-side check turner_upload_scene applies, without a device:
 * TURNER_OK and the traversal stack depth the tree needs (the largest number
 * of inner nodes on a root-to-leaf path), TURNER_ERR_BAD_SCENE, or
 * TURNER_ERR_TOO_LARGE when that depth exceeds the kernels' stack (128).
 * No reference counterpart: the reference trusts its own builder's output. */
int turner_validate_nodes(const uint64_t* nodes, uint32_t n_nodes, uint32_t n_tris, uint32_t* stack_depth);

/* ---------------------------------------------------------- intersect */
/* Batched KDTreeIntersection::intersect. Rays are SoA (ox, oy, oz, dx, dy,
 * dz), each of n floats; directions need not be normalised. For each ray:
 * hit_id = triangle index or TURNER_MISS; r = parametric distance (FLT_MAX on
 * a miss); s, t = barycentric coordinates (0 on a miss). `flags` selects
 * host or device buffers. `mode` is TURNER_TRAVERSAL_*. Synchronous. */
int turner_intersect(turner_ctx* ctx, uint32_t scene_id, const float* ox, const float* oy, const float* oz,
                     const float* dx, const float* dy, const float* dz, uint64_t n, uint32_t* hit_id, float* r,
                     float* s, float* t, int mode, uint32_t flags);

/* Batched shadow-ray test of the path tracer (pathtracer.cpp:44-58): the
 * reference traces the closest hit from p2 toward the light and calls the
 * point lit when there is no hit or r_closest > |light - p2|. Here
 * blocked[i] = 1 iff the ray (SoA as in turner_intersect) has a valid
 * triangle intersection with r <= tmax[i] in a leaf its traversal visits,
 * else 0: the same predicate, so blocked == !(miss || r_closest > tmax)
 * for the reference's closest hit, decided without finding the closest hit
 * (traversal stops at the first such triangle). The renders use the same
 * test for their shadow rays. `flags` selects host or device buffers.
 * Synchronous. */
int turner_occluded(turner_ctx* ctx, uint32_t scene_id, const float* ox, const float* oy, const float* oz,
                    const float* dx, const float* dy, const float* dz, const float* tmax, uint64_t n,
                    uint8_t* blocked, uint32_t flags);

/* Batched intersect that allocates nothing. No counterpart in the reference.
 * For callers that must not allocate device memory while they run: a
 * renderer's per-frame loop (cudaMalloc can synchronize the whole device and
 * stall the frame) or a host framework whose own pool owns every device
 * allocation. They upload the scene once at load time, then pass rays and
 * outputs in device memory they own (SoA as in turner_intersect with
 * TURNER_DEVICE_BUFFERS); results are identical to turner_intersect.
 * The traversal's scratch (its work counter) lives in a static device array
 * of TURNER_NOALLOC_SCRATCH_WORDS 32-bit words that every GPU loading this
 * library holds until exit; no cudaMalloc, cudaFree or allocating library
 * call is made. The first call on a device looks up that array's device
 * address (cudaGetSymbolAddress), so make the first call before any stream
 * capture. All calls on a device share the array: calls that overlap on the
 * GPU (other streams, other contexts) race and must be serialized by the
 * caller. At most TURNER_NOALLOC_MAX_RAYS rays per call (the counter is 32
 * bits); more return TURNER_ERR_TOO_LARGE. Synchronous on the context stream. */
#define TURNER_NOALLOC_SCRATCH_WORDS 64
#define TURNER_NOALLOC_MAX_RAYS (1ull << 30)
int turner_intersect_noalloc(turner_ctx* ctx, uint32_t scene_id, const float* ox, const float* oy, const float* oz,
                             const float* dx, const float* dy, const float* dz, uint64_t n, uint32_t* hit_id,
                             float* r, float* s, float* t, int mode);

/* -------------------------------------------------------------- render */
/* Renders each job into out_rgba[j] (width*height*4 floats, row-major RGBA
 * after the per-pixel mean, exposure and gamma of main.cpp:216-223), host or
 * device memory per `flags`. All jobs of a call form one batch: their pixels
 * are laid end to end and traced in passes of up to the chunk length (a pass
 * may hold pixels of several jobs of different scenes, sizes, sample counts
 * and depths); a batch of more than one job is captured into one CUDA graph
 * and launched once. stats may be NULL; otherwise it receives one
 * turner_stats per job (device_ms is the whole batch's). Synchronous. */
int turner_render(turner_ctx* ctx, const turner_job* jobs, uint32_t n_jobs, float* const* out_rgba,
                  turner_stats* stats, uint32_t flags);
/* Launch configuration picked by turner_autotune. No reference counterpart.
 *   persistent     1: persistent traversal with ray replacement, 0: one thread per ray
 *   blocks_per_sm  resident traversal blocks per SM (0 = occupancy limit)
 *   block          threads per traversal block (128 or 256)
 *   stack          traversal stack entries (64 or 128; 64 only if every scene fits)
 *   chunk_paths    paths in flight per render pass (queue length)
 *   mailbox        1: skip a triangle this ray tested in the last four tests
 *                  (exact: a repeat cannot change the answer; 128-thread blocks)
 *   min_blocks     10, 12 or 16: cap traversal registers so that many 128-thread
 *                  blocks fit per SM (48, 40, 32 registers), 0: no cap.
 *                  Default 10: the traversal is latency-bound and 10 blocks
 *                  beat the uncapped 9 (56 registers) and the 12 at 40
 *                  registers, which spill more
 *   refill_camera, refill_bounce, packets: the warp refill thresholds of
 *                  camera and bounce rays and camera-ray packets (see
 *                  turner_set_traversal_refill / _packet) */
typedef struct turner_tuning {
    int32_t persistent;
    uint32_t blocks_per_sm;
    uint32_t block;
    uint32_t stack;
    uint32_t chunk_paths;
    uint32_t mailbox;
    uint32_t min_blocks;
    double ms;             /* device time of the batch with this configuration */
    uint32_t candidates;   /* configurations timed (0: taken from the cache)  */
    uint32_t refill_camera;   /* turner_set_traversal_refill for camera rays (1..32) */
    uint32_t refill_bounce;   /* and for bounce rays (1..32)                         */
    uint32_t packets;         /* 1: camera-ray warps as packets (turner_set_traversal_packet) */
} turner_tuning;
/* Times configurations on the given batch (coordinate descent over the
 * fields above, two renders each, CUDA events) and applies the fastest to the
 * context. Results are cached per GPU model and batch shape in the file named
 * by TURNER_TUNE_CACHE (default ~/.cache/turner_gb300_tuning.txt); force != 0
 * ignores the cache. */
int turner_autotune(turner_ctx* ctx, const turner_job* jobs, uint32_t n_jobs, int force, turner_tuning* out);
int turner_set_tuning(turner_ctx* ctx, const turner_tuning* tuning);
int turner_get_tuning(turner_ctx* ctx, turner_tuning* tuning);

/* When renders are captured into a CUDA graph. AUTO (default): batches of
 * more than one job; ALWAYS: every render and accumulate pass; NEVER: no
 * capture (per-kernel timing with turner_set_profiling needs it). A batch of
 * the same shape as the previous one updates the instantiated graph in place
 * (cudaGraphExecUpdate) instead of instantiating a new one. Renders that
 * train the learned proposal are never captured. No reference counterpart. */
#define TURNER_GRAPH_AUTO 0
#define TURNER_GRAPH_ALWAYS 1
#define TURNER_GRAPH_NEVER 2
int turner_set_graph_mode(turner_ctx* ctx, int mode);
/* Number of CUDA graphs launched by this context. No reference counterpart. */
uint64_t turner_graph_launch_count(turner_ctx* ctx);

/* Progressive FP64 accumulation for converged reference images: adds
 * `passes` further sample passes of pixel_samples each to a double-precision
 * per-pixel sum held by the context (keyed by job seed and size) and writes
 * the running mean (linear radiance, no tone map) to out_rgba_mean. With
 * out_rgba_mean NULL the sum stays on the device (nothing is copied back;
 * a later call with passes = 0 reads the mean). */
int turner_render_accumulate(turner_ctx* ctx, const turner_job* job, uint32_t passes, double* out_rgba_mean,
                             uint64_t* total_samples, uint32_t flags);

/* ------------------------------------------------- learned proposal */
/* A small MLP predicting, per hit point, an 8-lobe von Mises-Fisher mixture
 * over bounce directions (no counterpart in the reference, whose bounces are
 * uniform on the hemisphere). BF16 weights on tcgen05 tensor cores with FP32
 * accumulation; trained with Adam on (features, direction, weight) samples.
 *   features  9 floats per sample: position in [0,1]^3 (scene box), shading
 *             normal, albedo
 *   output    40 floats per sample: 8 x (direction, log concentration, logit)
 *   loss      mean over samples of -weight * log q(direction) (the KL
 *             objective; turner_guide_set_objective below)
 * Parameters: TURNER_GUIDE_PARAMS floats, W1 b1 ... W5 b5 (W row-major
 * [out x in]; layers 80->64->64->64->64->40). */
#define TURNER_GUIDE_PARAMS 20264
typedef struct turner_guide turner_guide;
/* A proposal runs on the stream of the context it was created on. Destroying
 * it unbinds it from that context (turner_set_guide). Destroying the context
 * first is allowed: the proposal then accepts turner_guide_destroy only, and
 * its other calls return TURNER_ERR_INVALID_ARG. */
int turner_guide_create(turner_ctx* ctx, uint64_t seed, turner_guide** out);
void turner_guide_destroy(turner_guide* guide);
/* set != 0: load params (host, TURNER_GUIDE_PARAMS floats); 0: read them. */
int turner_guide_params(turner_guide* guide, float* params, int set);
/* Host buffers: features n*9 in, out n*40 out. */
int turner_guide_forward(turner_guide* guide, const float* features, uint32_t n, float* out);
/* Sum over samples of d(-w log q)/d params into grad (host), and the summed loss. */
int turner_guide_gradient(turner_guide* guide, const float* features, const float* dirs, const float* weights,
                          uint32_t n, float* grad, float* loss);
/* Training objective of the proposal, for turner_guide_gradient, _train and
 * online training. KL (default): loss -c log q(w) per sample, the gradient
 * averaged over the samples. VARIANCE: the second moment of the estimator
 * that samples the mixture p = q/2 + max(0, n.w)/(2 pi): per sample the
 * gradient of -c' log q with c' = c^2 q(w) / (2 p(w)) held constant (n the
 * normal of the sample's features), the step's gradient divided by the sum
 * of its weights c'. */
#define TURNER_GUIDE_OBJECTIVE_KL 0
#define TURNER_GUIDE_OBJECTIVE_VARIANCE 1
int turner_guide_set_objective(turner_guide* guide, int objective);
/* `steps` Adam steps (learning rate lr) on one batch; *loss = mean loss of the last. */
int turner_guide_train(turner_guide* guide, const float* features, const float* dirs, const float* weights,
                       uint32_t n, float lr, uint32_t steps, float* loss);

/* Binds a proposal to the context for jobs with TURNER_SAMPLING_GUIDED
 * (guide may be NULL to unbind; a proposal created on another context is
 * rejected with TURNER_ERR_INVALID_ARG). train != 0: online training during
 * turner_render / turner_render_accumulate: after every pass (chunk), the
 * pass's recorded bounces (about records_per_pass of them, >= 128; 0 keeps
 * the current value, default 2^18) get their target weight (incident
 * radiance times f cos / p, from the rest of the path) and one Adam step with
 * learning rate lr runs, on the context's stream without a host
 * synchronisation. Training renders are not captured into graphs. */
int turner_set_guide(turner_ctx* ctx, turner_guide* guide, int train, float lr, uint32_t records_per_pass);
/* Guided jobs sample from the proposal at hits of depth < depth (1..64,
 * default 64: every bounce) and by cosine below; network inputs and
 * inference run only for the guided depths. No reference counterpart. */
int turner_set_guide_depth(turner_ctx* ctx, uint32_t depth);
/* Weights of the online training records: 0 (default) the incident radiance
 * times f cos / p, the target of the proposal's own distribution; 1 also
 * times the path throughput that reached the bounce (the luminance the path
 * gained after it), so the shared network favours the bounces that carry
 * most of the pixels' radiance; 2 times the square root of that throughput.
 * No reference counterpart. */
int turner_set_guide_weighting(turner_ctx* ctx, int mode);
/* Adam steps per training pass (1..64, default 16), each over all of the
 * pass's records: more steps per pass learn faster from the same samples
 * (16 gave the best equal-time result on the baffled room; each step takes
 * about 0.4 ms for 2^16 records). */
int turner_set_guide_steps(turner_ctx* ctx, uint32_t steps_per_pass);
/* Adam steps the bound proposal has taken (in renders and turner_guide_train),
 * its last mean loss (both 0 when no proposal is bound; waits for the
 * context's stream), and the device time of training during renders. */
int turner_guide_stats(turner_ctx* ctx, uint64_t* steps, float* last_loss, double* train_ms);

/* ---------------------------------------------------------- host tree */
/* SAH kd-tree of [WH06] Algorithm 4 with the reference's constants and
 * tie-breaking (lib/kdtree.cpp:124-467): the node words and triangle records
 * are identical to KDTree's. vertices: n*9 floats (v0, v1, v2); normals: n*9
 * or NULL (zero normals); diffuse: n*4 or NULL. Subtrees are built on
 * `threads` host threads (0 = all cores). */
int turner_kdtree_build(const float* vertices, const float* normals, const float* diffuse, uint32_t n_tris,
                        int threads, turner_kdtree** out);
uint32_t turner_kdtree_num_nodes(const turner_kdtree* tree);
uint32_t turner_kdtree_num_triangles(const turner_kdtree* tree);
uint32_t turner_kdtree_height(const turner_kdtree* tree);
/* Copies nodes (num_nodes words), triangle records and box out; any may be NULL. */
int turner_kdtree_export(const turner_kdtree* tree, uint64_t* nodes, turner_triangle* tris, float box[6]);
int turner_upload_kdtree(turner_ctx* ctx, const turner_kdtree* tree, uint32_t* scene_id);
void turner_kdtree_free(turner_kdtree* tree);
/* Sets the reflective colour and reflectivity of every triangle record
 * (n_tris * 5 floats: r, g, b, a, reflectivity), the material fields the
 * Whitted raytracer reads (raytracer.cpp:46-55). They do not change the tree. */
int turner_kdtree_set_reflective(turner_kdtree* tree, const float* reflective);

/* Builds a kd-tree on the context's GPU, level by level: SAH with the
 * reference's cost constants and termination test over 32 bins per axis in
 * cells of more than 8192 triangles and over every clipped-box bound in
 * smaller cells, triangles classified by their polygons clipped to each cell,
 * and no empty-space splits (the flattened tree could not keep them). No counterpart
 * for the build itself: the reference builds on the host
 * (lib/kdtree.cpp:124-412), and its node words depend on std::sort's order
 * among equal events, so this tree is not the reference's. It is in the same
 * FlatNode format with the same triangle records, and every leaf lists every
 * triangle whose box meets its cell, so closest hits agree with the
 * reference's tree except where the reference's own thick-plane clipping
 * leaves a triangle out. Synchronous; allocates device memory while it runs. */
int turner_kdtree_build_gpu(turner_ctx* ctx, const float* vertices, const float* normals, const float* diffuse,
                            uint32_t n_tris, turner_kdtree** out);

/* ---------------------------------------------------------- tree files */
/* A binary file holding one kd-tree (node words, triangle records, box),
 * keyed by the content of the triangles it was built from. Replaces the
 * reference's fixed-name cereal cache ./kdtree.cache (main.cpp:142-167),
 * which is not keyed by the scene. Layout: a 128-byte header ("TRNKDT01",
 * key, counts, box, height, payload checksum), then the node words (8 bytes
 * each), then the triangle records (192 bytes each), all little-endian. */
typedef struct turner_tree_file turner_tree_file;
/* 64-bit content key of a triangle set (the arrays turner_kdtree_build takes). */
uint64_t turner_mesh_key(const float* vertices, const float* normals, const float* diffuse, uint32_t n_tris);
/* Writes the tree under a temporary name and renames it to `path`. */
int turner_kdtree_save(const turner_kdtree* tree, uint64_t key, const char* path);
/* Reads a tree file; key != 0 must match the stored key. A bad magic, size,
 * key or checksum is TURNER_ERR_BAD_SCENE. */
int turner_kdtree_load(const char* path, uint64_t key, turner_kdtree** out);
/* turner_kdtree_build through a cache directory: loads <dir>/<key>.tkd when
 * it is valid for these triangles, else builds and writes it. cache_dir NULL
 * builds without a cache. *from_cache (may be NULL) tells which happened. */
int turner_kdtree_build_cached(const float* vertices, const float* normals, const float* diffuse, uint32_t n_tris,
                               int threads, const char* cache_dir, turner_kdtree** out, int* from_cache);
/* Maps a tree file read-only (no copy); the arrays can go straight to
 * turner_upload_scene. verify != 0 checks the payload checksum. */
int turner_tree_file_map(const char* path, uint64_t key, int verify, turner_tree_file** out);
const uint64_t* turner_tree_file_nodes(const turner_tree_file* file, uint32_t* n_nodes);
const turner_triangle* turner_tree_file_triangles(const turner_tree_file* file, uint32_t* n_tris);
const float* turner_tree_file_box(const turner_tree_file* file);
uint64_t turner_tree_file_key(const turner_tree_file* file);
void turner_tree_file_unmap(turner_tree_file* file);

/* ------------------------------------------------------------ scenes */
/* Seeded synthetic scenes (the reference loads .blend files through assimp,
 * which this build does not ship):
 *   0 ROOM         36-triangle box room: 5 walls, two boxes rotated +-17 deg,
 *                  a 2-triangle ceiling quad, point light below the ceiling
 *   1 SPHERE_ROOM  room shell + icosphere subdivided `detail` times (7 ->
 *                  327,680 triangles), displaced by 5-octave value noise
 *   2 SOUP         clustered triangle soup of `count` triangles in the room
 *   3 BAFFLE_ROOM  walls tessellated detail x detail quads, a 1.5x1.5 baffle
 *                  0.3 below the light
 *   4 BAFFLE_SPHERE the SPHERE_ROOM sphere inside the BAFFLE_ROOM room
 *   5 MIRROR_ROOM  the ROOM with reflective boxes (reflectivity 0.3 and 0.85),
 *                  for the raytracer */
#define TURNER_SCENE_ROOM 0
#define TURNER_SCENE_SPHERE_ROOM 1
#define TURNER_SCENE_SOUP 2
#define TURNER_SCENE_BAFFLE_ROOM 3
#define TURNER_SCENE_BAFFLE_SPHERE 4
#define TURNER_SCENE_MIRROR_ROOM 5

int turner_scene_make(int kind, uint32_t detail, uint32_t count, uint64_t seed, float aspect, turner_mesh** out);
uint32_t turner_mesh_num_triangles(const turner_mesh* mesh);
const float* turner_mesh_vertices(const turner_mesh* mesh); /* n*9 */
const float* turner_mesh_normals(const turner_mesh* mesh);  /* n*9 */
const float* turner_mesh_diffuse(const turner_mesh* mesh);  /* n*4 */
/* n*5: reflective colour (rgba) and reflectivity per triangle (zeros where a
 * scene has no mirrors); give it to turner_kdtree_set_reflective. */
const float* turner_mesh_reflective(const turner_mesh* mesh);
/* Camera as the scene defines it; *hfov receives aiCamera::mHorizontalFOV. */
void turner_mesh_camera(const turner_mesh* mesh, turner_camera* cam, float* hfov);
/* Returns the number of lights (0 or 1) and copies the first. */
int turner_mesh_light(const turner_mesh* mesh, turner_light* light);
void turner_mesh_free(turner_mesh* mesh);

/* Hit-test ray set: n rays, origins uniform in box, directions uniform on
 * the sphere (Marsaglia 1972), seeded; SoA outputs of n floats each. */
int turner_make_rays(uint64_t n, const float box[6], uint64_t seed, float* ox, float* oy, float* oz, float* dx,
                     float* dy, float* dz);

/* --------------------------------------------------------------- output */
/* P3 writer of lib/raster.h:79-100. Returns the byte length of the full
 * text; writes at most `cap` bytes to `out` (which may be NULL). */
uint64_t turner_write_p3(const float* rgba, uint32_t width, uint32_t height, char* out, uint64_t cap);

#ifdef __cplusplus
}
#endif

#endif /* TURNER_GPU_H */
