// C ABI of the GB300 path-tracing core: contexts, scene upload with
// validation, batched intersection and the wavefront render loop.
#include "guide.cuh"
#include "kernels.h"
#include "turner_gpu.h"

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <future>
#include <memory>
#include <thread>
#include <mutex>
#include <new>
#include <string>
#include <vector>

namespace {

using namespace turner;

struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    ~DevBuf() { release(); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    // grows, never shrinks; contents are not preserved
    cudaError_t ensure(size_t n) {
        if (n <= bytes) return cudaSuccess;
        release();
        cudaError_t e = cudaMalloc(&p, n);
        if (e != cudaSuccess) {
            p = nullptr;
            return e;
        }
        bytes = n;
        return cudaSuccess;
    }
    template <class T> T* as() const { return static_cast<T*>(p); }
};

// Page-locked host memory, grown on demand: uploads stage through it so that
// their copies run asynchronously at full link speed.
struct PinnedBuf {
    void* p = nullptr;
    size_t bytes = 0;
    ~PinnedBuf() { release(); }
    void release() {
        if (p) cudaFreeHost(p);
        p = nullptr;
        bytes = 0;
    }
    cudaError_t ensure(size_t n) {
        if (n <= bytes) return cudaSuccess;
        release();
        cudaError_t e = cudaMallocHost(&p, n);
        if (e != cudaSuccess) {
            p = nullptr;
            return e;
        }
        bytes = n;
        return cudaSuccess;
    }
};

struct SceneStore {
    bool live = false;
    DevBuf nodes, tri, shade, refl;
    SceneView view{};
};

int map_cuda(cudaError_t e) {
    if (e == cudaSuccess) return TURNER_OK;
    if (e == cudaErrorMemoryAllocation) return TURNER_ERR_OUT_OF_MEMORY;
    return TURNER_ERR_CUDA;
}

} // namespace

struct turner_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::vector<std::unique_ptr<SceneStore>> scenes;
    std::vector<uint32_t> validate_scratch;   // node-check depths of the last upload, kept for the next
    // render workspace
    PinnedBuf staging;                 // upload staging (scene records)
    DevBuf L, qa[4], qb[4], hits, shq[3], shjob, shaux, counters, image, rays_in, rays_out, work, jobtab, jobcnt, acc, tune_out;
    uint64_t acc_key[7] = {};          // what the FP64 running sum belongs to
    uint64_t acc_samples = 0, acc_passes = 0;
    int graph_mode = TURNER_GRAPH_AUTO;
    cudaGraphExec_t graph_exec = nullptr;   // last instantiated batch graph, updated in place when it can be
    uint64_t graph_updates = 0;
    // learned proposal used by jobs with TURNER_SAMPLING_GUIDED, and every
    // live proposal created on this context (they share its stream)
    turner_guide* guide = nullptr;
    std::vector<turner_guide*> guides;
    bool guide_train = false;
    float guide_lr = 1e-3f;
    uint32_t guide_records = 1u << 18;   // training samples per pass
    uint32_t guide_steps_per_pass = 16;   // Adam steps on each pass's samples
    int32_t guide_depth = 64;             // hits below this depth sample by cosine
    int32_t guide_weighting = 0;          // training targets: 0 incident radiance, 1 / 2 also by path throughput
    DevBuf gfeat, gout, qa_rec, qb_rec, r_feat, r_dir, r_weight, r_path, r_lbefore, r_tafter, r_fcp, r_count;
    double guide_train_ms = 0.0;
    uint64_t graph_launches = 0;
    TraverseCfg traverse;              // persistent traversal on by default
    // refill threshold of the persistent traversal per ray kind (TURNER_RAYS_*).
    // Measured on the 327,692-triangle frame (1920x1080x16, depth 3): whole-warp
    // refills keep a camera-ray warp's 2 pixels x 16 samples together (closest
    // hit 173.7 -> 143.1 ms, their shadow rays 74.8 -> 60.0 ms in total);
    // incoherent bounce and shadow rays want nearly every idle lane refilled
    uint32_t refill[TURNER_RAYS_KINDS] = {32, 2, 32, 4, 1};
    int packet_mode = TURNER_PACKET_CAMERA;   // where warps of coherent fresh rays traverse as packets
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    uint32_t chunk_paths = 1u << 24;   // paths in flight per render pass
    uint64_t launches = 0;
    std::string last_error;
    // optional per-kernel timing: event pairs around launches, summed per kind
    bool profiling = false;
    std::vector<cudaEvent_t> ev_pool;
    std::vector<std::pair<int, size_t>> ev_used;   // (kernel kind, first event index)
    double kernel_ms[TURNER_KERNEL_KINDS] = {};
    uint64_t kernel_launches[TURNER_KERNEL_KINDS] = {};
};

#define TURNER_CK(call)                                                                      \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess) {                                                             \
            ctx->last_error = std::string(#call) + ": " + cudaGetErrorString(e_);            \
            return map_cuda(e_);                                                             \
        }                                                                                    \
    } while (0)

namespace {

// Brackets one kernel launch with an event pair when profiling is on.
struct KernelTimer {
    turner_ctx* ctx;
    int kind;
    size_t first = 0;
    bool on = false;
    KernelTimer(turner_ctx* c, int k, bool always = false) : ctx(c), kind(k) {
        ctx->launches += 1;
        if (!ctx->profiling && !always) return;
        first = ctx->ev_used.size() * 2;
        while (ctx->ev_pool.size() < first + 2) {
            cudaEvent_t e;
            if (cudaEventCreate(&e) != cudaSuccess) return;
            ctx->ev_pool.push_back(e);
        }
        cudaEventRecord(ctx->ev_pool[first], ctx->stream);
        on = true;
    }
    ~KernelTimer() {
        if (!on) return;
        cudaEventRecord(ctx->ev_pool[first + 1], ctx->stream);
        ctx->ev_used.emplace_back(kind, first);
    }
};

// After a stream synchronize: folds the recorded event pairs into the totals.
void collect_kernel_times(turner_ctx* ctx) {
    for (const auto& u : ctx->ev_used) {
        float ms = 0;
        if (cudaEventElapsedTime(&ms, ctx->ev_pool[u.second], ctx->ev_pool[u.second + 1]) == cudaSuccess) {
            ctx->kernel_ms[u.first] += ms;
            ctx->kernel_launches[u.first] += 1;
            if (u.first == TURNER_KERNEL_GUIDE_TRAIN) ctx->guide_train_ms += ms;
        }
    }
    ctx->ev_used.clear();
}

// Checks that traversal stays inside the arrays: child indices point forward
// and in range, leaf ids are valid triangles, every leaf run ends (half-empty
// leaf or inner node) before the end of the array. Returns the stack depth
// traversal needs (the largest number of inner nodes on a root-to-leaf path),
// or -1. Every edge of the flattened tree points forward (left child i + 1,
// right child > i, next leaf of a run i + 1), so one forward pass that only
// looks at nodes reached from the root visits them after all their parents.
long validate_nodes(const uint64_t* nodes, uint32_t n_nodes, uint32_t n_tris, std::vector<uint32_t>& depth) {
    if (n_nodes == 0) return -1;
    depth.assign(n_nodes, 0);    // inner nodes above, +1 (0: not reached); reused, so no fresh pages per call
    depth[0] = 1;
    uint32_t height = 0;
    for (uint32_t i = 0; i < n_nodes; ++i) {
        const uint32_t di = depth[i];
        if (di == 0) continue;
        const uint64_t w = nodes[i];
        const uint32_t lo = static_cast<uint32_t>(w);
        if ((lo & 3u) != 3u) {
            const uint32_t right = lo >> 2;
            if (i + 1 >= n_nodes || right <= i || right >= n_nodes) return -1;
            const uint32_t dc = std::min<uint32_t>(di + 1, 1u << 30);
            depth[i + 1] = std::max(depth[i + 1], dc);
            depth[right] = std::max(depth[right], dc);
            height = std::max(height, di);
        } else {
            if (static_cast<uint32_t>(w >> 32) >= n_tris) return -1;
            if (lo == 0xFFFFFFFFu) continue;         // half-empty leaf: the run ends
            if ((lo >> 2) >= n_tris) return -1;
            if (i + 1 >= n_nodes) return -1;
            if ((static_cast<uint32_t>(nodes[i + 1]) & 3u) == 3u) depth[i + 1] = std::max(depth[i + 1], di);
        }
    }
    return static_cast<long>(height);
}

// Rows of the band a job renders ([row_begin, row_end), row_end 0 = height).
uint32_t job_rows(const turner_job& j) { return (j.row_end ? j.row_end : j.height) - j.row_begin; }

// Pixels a job renders (and holds in its output).
uint64_t job_pixels(const turner_job& j) { return uint64_t(j.width) * job_rows(j); }

void fill_job(const turner_job& j, const SceneView& sc, JobDesc& d) {
    std::memset(&d, 0, sizeof(d));
    d.sc = sc;
    std::memcpy(d.cam_pos, j.camera.position, sizeof(d.cam_pos));
    std::memcpy(d.trafo, j.camera.trafo, sizeof(d.trafo));
    d.delta_x = j.camera.delta_x;
    d.delta_y = j.camera.delta_x / j.camera.aspect;   // lib/types.h:104
    d.width = j.width;
    d.height = j.height;
    d.row0 = j.row_begin;
    d.rows = job_rows(j);
    d.spp = j.pixel_samples;
    d.max_depth = j.max_depth;
    d.mc = j.monte_carlo_samples;
    std::memcpy(d.bg, j.background, sizeof(d.bg));
    d.seed = j.seed;
    d.n_lights = j.n_lights;
    std::memcpy(d.light_pos, j.light.position, sizeof(d.light_pos));
    std::memcpy(d.light_col, j.light.color, sizeof(d.light_col));
    d.sampling = j.sampling;
    d.traversal = j.traversal;
    d.exposure = j.exposure;
    d.inv_gamma = j.inverse_gamma;
    d.gamma = j.gamma_correction;
    d.tone_map = 1;
    d.renderer = j.renderer;
    d.shadow_intensity = j.shadow_intensity;
    d.max_visibility = j.max_visibility;
}

// Rays of one path at its widest level: M^max_depth for the branching
// estimator (-m M > 1), else 1; 0 if that exceeds 2^26.
uint64_t branch_width(const turner_job& j) {
    if (j.monte_carlo_samples <= 1 || j.renderer != TURNER_RENDERER_PATH) return 1;
    uint64_t w = 1;
    for (int d = 0; d < j.max_depth; ++d) {
        w *= static_cast<uint64_t>(j.monte_carlo_samples);
        if (w > (1ull << 26)) return 0;
    }
    return w;
}

int check_job(turner_ctx* ctx, const turner_job& j) {
    if (j.scene_id >= ctx->scenes.size() || !ctx->scenes[j.scene_id]->live) return TURNER_ERR_INVALID_ARG;
    if (j.width == 0 || j.height == 0 || j.pixel_samples == 0 || j.max_depth < 0) return TURNER_ERR_INVALID_ARG;
    if (j.row_end > j.height || j.row_begin >= (j.row_end ? j.row_end : j.height)) return TURNER_ERR_INVALID_ARG;
    if (!(j.camera.aspect > 0)) return TURNER_ERR_INVALID_ARG;
    if (j.monte_carlo_samples < 0 || j.n_lights < 0 || j.n_lights > 1) return TURNER_ERR_INVALID_ARG;
    if (j.monte_carlo_samples > TURNER_MAX_MC) return TURNER_ERR_TOO_LARGE;
    if (j.monte_carlo_samples > 1 && j.sampling == TURNER_SAMPLING_GUIDED) return TURNER_ERR_UNSUPPORTED;
    if (branch_width(j) == 0) return TURNER_ERR_TOO_LARGE;
    if (j.sampling != TURNER_SAMPLING_UNIFORM && j.sampling != TURNER_SAMPLING_COSINE &&
        j.sampling != TURNER_SAMPLING_GUIDED)
        return TURNER_ERR_INVALID_ARG;
    if (j.sampling == TURNER_SAMPLING_GUIDED && !ctx->guide) return TURNER_ERR_INVALID_ARG;
    if (j.traversal != TURNER_TRAVERSAL_PARITY && j.traversal != TURNER_TRAVERSAL_FAST) return TURNER_ERR_INVALID_ARG;
    if (j.renderer < TURNER_RENDERER_PATH || j.renderer > TURNER_RENDERER_RAYCAST) return TURNER_ERR_INVALID_ARG;
    if (j.renderer != TURNER_RENDERER_PATH) {
        // TracerConfig::check (config.h:125-132); the raytracer reads lights.front()
        if (!(j.shadow_intensity >= 0.f && j.shadow_intensity <= 1.f) || !(j.max_visibility >= 0.f))
            return TURNER_ERR_INVALID_ARG;
        if (j.renderer == TURNER_RENDERER_RAYTRACE && j.n_lights != 1) return TURNER_ERR_INVALID_ARG;
        if (j.sampling == TURNER_SAMPLING_GUIDED) return TURNER_ERR_INVALID_ARG;
    }
    if (uint64_t(j.width) * j.height > (1ull << 31)) return TURNER_ERR_TOO_LARGE;
    if (j.max_depth > 64) return TURNER_ERR_TOO_LARGE;
    return TURNER_OK;
}

} // namespace

extern "C" {

const char* turner_strerror(int status) {
    switch (status) {
    case TURNER_OK: return "ok";
    case TURNER_ERR_INVALID_ARG: return "invalid argument";
    case TURNER_ERR_CUDA: return "CUDA runtime error";
    case TURNER_ERR_OUT_OF_MEMORY: return "out of memory";
    case TURNER_ERR_BAD_SCENE: return "node array failed validation";
    case TURNER_ERR_TIMEOUT: return "bounded device wait timed out";
    case TURNER_ERR_DEVICE_BOUNDS: return "device-side index check failed";
    case TURNER_ERR_UNSUPPORTED: return "unsupported parameter combination";
    case TURNER_ERR_NO_DEVICE: return "no suitable CUDA device";
    case TURNER_ERR_TOO_LARGE: return "request exceeds a documented maximum";
    default: return "unknown status";
    }
}

int turner_create(turner_ctx** out, int device) {
    if (!out) return TURNER_ERR_INVALID_ARG;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) return TURNER_ERR_NO_DEVICE;
    cudaDeviceProp prop{};
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return TURNER_ERR_NO_DEVICE;
    if (prop.major * 10 + prop.minor != 103) return TURNER_ERR_NO_DEVICE;   // built for sm_103a only
    auto* ctx = new (std::nothrow) turner_ctx;
    if (!ctx) return TURNER_ERR_OUT_OF_MEMORY;
    ctx->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev1);
    if (e != cudaSuccess) {
        delete ctx;
        return map_cuda(e);
    }
    *out = ctx;
    return TURNER_OK;
}

void turner_destroy(turner_ctx* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    // proposals that outlive their context lose its stream: afterwards they
    // accept turner_guide_destroy only
    for (turner_guide* g : ctx->guides) turner::guide::orphan(g);
    ctx->guides.clear();
    ctx->guide = nullptr;
    if (ctx->graph_exec) cudaGraphExecDestroy(ctx->graph_exec);
    ctx->scenes.clear();
    for (cudaEvent_t e : ctx->ev_pool) cudaEventDestroy(e);
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

int turner_last_device_error(turner_ctx* ctx) { return ctx ? TURNER_OK : TURNER_ERR_INVALID_ARG; }

} // extern "C"

namespace turner {
cudaStream_t ctx_stream(turner_ctx* ctx) { return ctx->stream; }
int ctx_device(turner_ctx* ctx) { return ctx->device; }
void ctx_add_guide(turner_ctx* ctx, turner_guide* g) { ctx->guides.push_back(g); }
void ctx_remove_guide(turner_ctx* ctx, turner_guide* g) {
    ctx->guides.erase(std::remove(ctx->guides.begin(), ctx->guides.end(), g), ctx->guides.end());
    if (ctx->guide == g) {
        ctx->guide = nullptr;
        ctx->guide_train = false;
    }
}
} // namespace turner

extern "C" {

uint64_t turner_launch_count(turner_ctx* ctx) { return ctx ? ctx->launches : 0; }

const char* turner_last_error_message(turner_ctx* ctx) { return ctx ? ctx->last_error.c_str() : ""; }

int turner_validate_nodes(const uint64_t* nodes, uint32_t n_nodes, uint32_t n_tris, uint32_t* stack_depth) {
    if (!nodes || n_nodes == 0 || n_tris == 0) return TURNER_ERR_INVALID_ARG;
    std::vector<uint32_t> scratch;
    const long depth = validate_nodes(nodes, n_nodes, n_tris, scratch);
    if (depth < 0) return TURNER_ERR_BAD_SCENE;
    if (stack_depth) *stack_depth = static_cast<uint32_t>(depth);
    return depth > kStackCap ? TURNER_ERR_TOO_LARGE : TURNER_OK;
}

int turner_upload_scene(turner_ctx* ctx, const uint64_t* nodes, uint32_t n_nodes, const turner_triangle* tris,
                        uint32_t n_tris, const float box[6], uint32_t* scene_id) {
    if (!ctx || !nodes || !tris || !box || !scene_id || n_nodes == 0 || n_tris == 0) return TURNER_ERR_INVALID_ARG;
    if (n_tris >= TURNER_MISS || n_nodes >= TURNER_MISS) return TURNER_ERR_TOO_LARGE;
    TURNER_CK(cudaSetDevice(ctx->device));
    // the node check runs on its own thread while the records are converted
    std::vector<uint32_t>& scratch = ctx->validate_scratch;
    auto checked = std::async(std::launch::async,
                              [=, &scratch]() { return validate_nodes(nodes, n_nodes, n_tris, scratch); });
    auto fail = [&](int status) {
        checked.wait();
        return status;
    };

    auto sc = std::unique_ptr<SceneStore>(new (std::nothrow) SceneStore);
    if (!sc) return fail(TURNER_ERR_OUT_OF_MEMORY);
    bool any_reflective = false;
    for (uint32_t i = 0; i < n_tris && !any_reflective; ++i) any_reflective = tris[i].reflectivity > 0.f;
    // staging layout: node words | intersection records | shading records | reflective colours
    const size_t node_bytes = sizeof(uint64_t) * n_nodes, rec_bytes = sizeof(float4) * 4 * size_t(n_tris);
    const size_t refl_bytes = any_reflective ? sizeof(float4) * size_t(n_tris) : 0;
    const size_t off_tri = (node_bytes + 255) & ~size_t(255), off_shade = off_tri + rec_bytes,
                 off_refl = off_shade + rec_bytes;
    cudaError_t e = cudaStreamSynchronize(ctx->stream);   // the staging buffer may still feed a copy
    if (e == cudaSuccess) e = ctx->staging.ensure(off_refl + refl_bytes);
    if (e != cudaSuccess) return fail(map_cuda(e));
    char* stage = static_cast<char*>(ctx->staging.p);
    float4* tri = reinterpret_cast<float4*>(stage + off_tri);
    float4* shade = reinterpret_cast<float4*>(stage + off_shade);
    float4* refl = reinterpret_cast<float4*>(stage + off_refl);
    auto convert = [&](uint32_t b, uint32_t e2) {
        for (uint32_t i = b; i < e2; ++i) {
            const turner_triangle& t = tris[i];
            tri[4 * size_t(i) + 0] = make_float4(t.vertices[0][0], t.vertices[0][1], t.vertices[0][2], t.uv);
            tri[4 * size_t(i) + 1] = make_float4(t.normal[0], t.normal[1], t.normal[2], t.vv);
            tri[4 * size_t(i) + 2] = make_float4(t.u[0], t.u[1], t.u[2], t.uu);
            tri[4 * size_t(i) + 3] = make_float4(t.v[0], t.v[1], t.v[2], t.denom);
            shade[4 * size_t(i) + 0] = make_float4(t.normals[0][0], t.normals[0][1], t.normals[0][2], t.diffuse[0]);
            shade[4 * size_t(i) + 1] = make_float4(t.normals[1][0], t.normals[1][1], t.normals[1][2], t.diffuse[1]);
            shade[4 * size_t(i) + 2] = make_float4(t.normals[2][0], t.normals[2][1], t.normals[2][2], t.diffuse[2]);
            shade[4 * size_t(i) + 3] = make_float4(t.diffuse[3], t.reflectivity, 0.f, 0.f);
            if (any_reflective)
                refl[i] = make_float4(t.reflective[0], t.reflective[1], t.reflective[2], t.reflective[3]);
        }
    };
    {
        const unsigned hw = std::max(1u, std::min(8u, std::thread::hardware_concurrency()));
        const uint32_t per = std::max<uint32_t>(16384, (n_tris + hw - 1) / hw);
        std::vector<std::thread> pool;
        for (uint32_t b = per; b < n_tris; b += per) pool.emplace_back(convert, b, std::min(n_tris, b + per));
        std::memcpy(stage, nodes, node_bytes);
        convert(0, std::min(n_tris, per));
        for (auto& th : pool) th.join();
    }
    e = sc->nodes.ensure(node_bytes);
    if (e == cudaSuccess) e = sc->tri.ensure(rec_bytes);
    if (e == cudaSuccess) e = sc->shade.ensure(rec_bytes);
    if (e == cudaSuccess && any_reflective) e = sc->refl.ensure(refl_bytes);
    if (e == cudaSuccess) e = cudaMemcpyAsync(sc->nodes.p, stage, node_bytes, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(sc->tri.p, tri, rec_bytes, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(sc->shade.p, shade, rec_bytes, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess && any_reflective)
        e = cudaMemcpyAsync(sc->refl.p, refl, refl_bytes, cudaMemcpyHostToDevice, ctx->stream);
    const long depth = checked.get();
    const cudaError_t es = cudaStreamSynchronize(ctx->stream);
    if (e == cudaSuccess) e = es;
    if (e != cudaSuccess) return map_cuda(e);
    if (depth < 0) return TURNER_ERR_BAD_SCENE;
    if (depth > kStackCap) return TURNER_ERR_TOO_LARGE;
    SceneView& v = sc->view;
    v.nodes = sc->nodes.as<uint2>();
    v.tri = sc->tri.as<float4>();
    v.shade = sc->shade.as<float4>();
    v.refl = any_reflective ? sc->refl.as<float4>() : nullptr;
    for (int k = 0; k < 3; ++k) {
        v.lo[k] = box[k];
        v.hi[k] = box[3 + k];
    }
    v.n_nodes = n_nodes;
    v.n_tris = n_tris;
    v.height = static_cast<uint32_t>(depth);
    sc->live = true;
    ctx->scenes.push_back(std::move(sc));
    *scene_id = static_cast<uint32_t>(ctx->scenes.size() - 1);
    return TURNER_OK;
}

int turner_free_scene(turner_ctx* ctx, uint32_t scene_id) {
    if (!ctx || scene_id >= ctx->scenes.size() || !ctx->scenes[scene_id]->live) return TURNER_ERR_INVALID_ARG;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    auto& sc = *ctx->scenes[scene_id];
    sc.nodes.release();
    sc.tri.release();
    sc.shade.release();
    sc.refl.release();
    sc.live = false;
    return TURNER_OK;
}

int turner_upload_kdtree(turner_ctx* ctx, const turner_kdtree* tree, uint32_t* scene_id) {
    if (!ctx || !tree) return TURNER_ERR_INVALID_ARG;
    const uint32_t nn = turner_kdtree_num_nodes(tree), nt = turner_kdtree_num_triangles(tree);
    std::vector<uint64_t> nodes(nn);
    std::vector<turner_triangle> tris(nt);
    float box[6];
    int st = turner_kdtree_export(tree, nodes.data(), tris.data(), box);
    if (st != TURNER_OK) return st;
    return turner_upload_scene(ctx, nodes.data(), nn, tris.data(), nt, box, scene_id);
}

int turner_intersect(turner_ctx* ctx, uint32_t scene_id, const float* ox, const float* oy, const float* oz,
                     const float* dx, const float* dy, const float* dz, uint64_t n, uint32_t* hit_id, float* r,
                     float* s, float* t, int mode, uint32_t flags) {
    if (!ctx || scene_id >= ctx->scenes.size() || !ctx->scenes[scene_id]->live) return TURNER_ERR_INVALID_ARG;
    if (!ox || !oy || !oz || !dx || !dy || !dz || !hit_id || !r || !s || !t) return TURNER_ERR_INVALID_ARG;
    if (mode != TURNER_TRAVERSAL_PARITY && mode != TURNER_TRAVERSAL_FAST) return TURNER_ERR_INVALID_ARG;
    if (flags > TURNER_DEVICE_BUFFERS) return TURNER_ERR_INVALID_ARG;
    if (n == 0) return TURNER_OK;
    TURNER_CK(cudaSetDevice(ctx->device));
    const SceneView& sc = ctx->scenes[scene_id]->view;
    const int fast = mode == TURNER_TRAVERSAL_FAST;
    TURNER_CK(ctx->work.ensure(sizeof(uint32_t) * 64));
    TraverseCfg cfg = ctx->traverse;
    if (sc.height > 64) cfg.stack = kStackCap;
    cfg.work = ctx->work.as<uint32_t>();
    cfg.refill = ctx->refill[TURNER_RAYS_INTERSECT];
    cfg.packet = (ctx->packet_mode & TURNER_PACKET_BATCHED) != 0;
    if (flags == TURNER_DEVICE_BUFFERS) {
        for (uint64_t b = 0; b < n; b += (1ull << 30)) {
            const uint64_t m = std::min<uint64_t>(n - b, 1ull << 30);
            TURNER_CK(cudaMemsetAsync(cfg.work, 0, sizeof(uint32_t), ctx->stream));
            KernelTimer kt(ctx, TURNER_KERNEL_INTERSECT);
            launch_intersect(sc, ox + b, oy + b, oz + b, dx + b, dy + b, dz + b, m, hit_id + b, r + b, s + b, t + b,
                             fast, cfg, ctx->stream);
        }
        TURNER_CK(cudaGetLastError());
        TURNER_CK(cudaStreamSynchronize(ctx->stream));
        collect_kernel_times(ctx);
        return TURNER_OK;
    }
    // host buffers: stage through device memory in slices
    const uint64_t slice = std::min<uint64_t>(n, 1ull << 24);
    TURNER_CK(ctx->rays_in.ensure(6 * sizeof(float) * slice));
    TURNER_CK(ctx->rays_out.ensure(4 * sizeof(float) * slice));
    float* din = ctx->rays_in.as<float>();
    float* dout = ctx->rays_out.as<float>();
    const float* src[6] = {ox, oy, oz, dx, dy, dz};
    for (uint64_t b = 0; b < n; b += slice) {
        const uint64_t m = std::min(slice, n - b);
        for (int k = 0; k < 6; ++k) {
            TURNER_CK(cudaMemcpyAsync(din + k * slice, src[k] + b, m * sizeof(float), cudaMemcpyHostToDevice,
                                      ctx->stream));
        }
        TURNER_CK(cudaMemsetAsync(cfg.work, 0, sizeof(uint32_t), ctx->stream));
        {
            KernelTimer kt(ctx, TURNER_KERNEL_INTERSECT);
            launch_intersect(sc, din, din + slice, din + 2 * slice, din + 3 * slice, din + 4 * slice,
                             din + 5 * slice, m, reinterpret_cast<uint32_t*>(dout), dout + slice, dout + 2 * slice,
                             dout + 3 * slice, fast, cfg, ctx->stream);
        }
        TURNER_CK(cudaGetLastError());
        TURNER_CK(cudaMemcpyAsync(hit_id + b, dout, m * sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream));
        TURNER_CK(cudaMemcpyAsync(r + b, dout + slice, m * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
        TURNER_CK(cudaMemcpyAsync(s + b, dout + 2 * slice, m * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
        TURNER_CK(cudaMemcpyAsync(t + b, dout + 3 * slice, m * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    }
    TURNER_CK(cudaStreamSynchronize(ctx->stream));
    collect_kernel_times(ctx);
    return TURNER_OK;
}

int turner_occluded(turner_ctx* ctx, uint32_t scene_id, const float* ox, const float* oy, const float* oz,
                    const float* dx, const float* dy, const float* dz, const float* tmax, uint64_t n,
                    uint8_t* blocked, uint32_t flags) {
    if (!ctx || scene_id >= ctx->scenes.size() || !ctx->scenes[scene_id]->live) return TURNER_ERR_INVALID_ARG;
    if (!ox || !oy || !oz || !dx || !dy || !dz || !tmax || !blocked) return TURNER_ERR_INVALID_ARG;
    if (flags > TURNER_DEVICE_BUFFERS) return TURNER_ERR_INVALID_ARG;
    if (n == 0) return TURNER_OK;
    TURNER_CK(cudaSetDevice(ctx->device));
    const SceneView& sc = ctx->scenes[scene_id]->view;
    TURNER_CK(ctx->work.ensure(sizeof(uint32_t) * 64));
    TraverseCfg cfg = ctx->traverse;
    cfg.work = ctx->work.as<uint32_t>();
    cfg.refill = ctx->refill[TURNER_RAYS_INTERSECT];
    cfg.packet = (ctx->packet_mode & TURNER_PACKET_BATCHED) != 0;
    // slices of at most 2^30 rays (the work counter is 32 bits)
    const uint64_t slice = flags == TURNER_DEVICE_BUFFERS ? std::min<uint64_t>(n, 1ull << 30)
                                                          : std::min<uint64_t>(n, 1ull << 24);
    float* din = nullptr;
    uint8_t* dout = nullptr;
    if (flags == TURNER_HOST_BUFFERS) {
        TURNER_CK(ctx->rays_in.ensure(7 * sizeof(float) * slice));
        TURNER_CK(ctx->rays_out.ensure(slice));
        din = ctx->rays_in.as<float>();
        dout = ctx->rays_out.as<uint8_t>();
    }
    const float* src[7] = {ox, oy, oz, dx, dy, dz, tmax};
    for (uint64_t b = 0; b < n; b += slice) {
        const uint32_t m = static_cast<uint32_t>(std::min(slice, n - b));
        const float* a[7];
        uint8_t* out = blocked + b;
        if (flags == TURNER_HOST_BUFFERS) {
            for (int k = 0; k < 7; ++k) {
                TURNER_CK(cudaMemcpyAsync(din + k * slice, src[k] + b, m * sizeof(float), cudaMemcpyHostToDevice,
                                          ctx->stream));
                a[k] = din + k * slice;
            }
            out = dout;
        } else {
            for (int k = 0; k < 7; ++k) a[k] = src[k] + b;
        }
        TURNER_CK(cudaMemsetAsync(cfg.work, 0, sizeof(uint32_t), ctx->stream));
        {
            KernelTimer kt(ctx, TURNER_KERNEL_INTERSECT);
            launch_occluded(sc, a[0], a[1], a[2], a[3], a[4], a[5], a[6], m, out, cfg, ctx->stream);
        }
        TURNER_CK(cudaGetLastError());
        if (flags == TURNER_HOST_BUFFERS) {
            TURNER_CK(cudaMemcpyAsync(blocked + b, dout, m, cudaMemcpyDeviceToHost, ctx->stream));
        }
    }
    TURNER_CK(cudaStreamSynchronize(ctx->stream));
    collect_kernel_times(ctx);
    return TURNER_OK;
}

int turner_probe_gather(turner_ctx* ctx, uint64_t buffer_bytes, uint32_t load_bytes, uint32_t repeats,
                        double* gbs) {
    if (!ctx || !gbs || (load_bytes != 8 && load_bytes != 32) || repeats == 0) return TURNER_ERR_INVALID_ARG;
    if (buffer_bytes < 4096 || (buffer_bytes & (buffer_bytes - 1)) || buffer_bytes > (1ull << 34))
        return TURNER_ERR_INVALID_ARG;
    TURNER_CK(cudaSetDevice(ctx->device));
    int sms = 0;
    TURNER_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
    const unsigned blocks = static_cast<unsigned>(sms) * 8;   // 8 x 256 threads per SM
    const uint32_t loads = 2048;                               // per thread
    DevBuf buf, out;
    TURNER_CK(buf.ensure(buffer_bytes));
    TURNER_CK(out.ensure(sizeof(uint32_t) * blocks * 256));
    TURNER_CK(cudaMemsetAsync(buf.p, 0x3c, buffer_bytes, ctx->stream));
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    TURNER_CK(cudaEventCreate(&e0));
    cudaError_t err = cudaEventCreate(&e1);
    double best = 0.0;
    // the first launch warms L2 with the buffer; the best of the rest is kept
    for (uint32_t r = 0; r <= repeats && err == cudaSuccess; ++r) {
        cudaEventRecord(e0, ctx->stream);
        launch_gather_probe(buf.p, buffer_bytes, static_cast<int>(load_bytes), loads, r, out.as<uint32_t>(), blocks,
                            ctx->stream);
        cudaEventRecord(e1, ctx->stream);
        err = cudaEventSynchronize(e1);
        float ms = 0;
        if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, e0, e1);
        if (err == cudaSuccess && r > 0 && ms > 0) {
            const double bytes = double(blocks) * 256.0 * loads * load_bytes;
            best = std::max(best, bytes / (ms * 1e-3) / 1e9);
        }
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    ctx->launches += repeats + 1;
    TURNER_CK(err);
    *gbs = best;
    return TURNER_OK;
}

int turner_set_chunk_paths(turner_ctx* ctx, uint32_t paths) {
    if (!ctx || paths < 1024) return TURNER_ERR_INVALID_ARG;
    ctx->chunk_paths = paths;
    return TURNER_OK;
}

int turner_set_traversal_packet(turner_ctx* ctx, int mode) {
    if (!ctx || mode < 0 || mode > (TURNER_PACKET_CAMERA | TURNER_PACKET_BATCHED)) return TURNER_ERR_INVALID_ARG;
    ctx->packet_mode = mode;
    return TURNER_OK;
}

int turner_set_traversal_speculative(turner_ctx* ctx, int on) {
    if (!ctx) return TURNER_ERR_INVALID_ARG;
    ctx->traverse.speculative = on != 0;
    return TURNER_OK;
}

int turner_set_traversal_ring(turner_ctx* ctx, uint32_t entries) {
    if (!ctx || (entries != 0 && entries != 4 && entries != 8)) return TURNER_ERR_INVALID_ARG;
    ctx->traverse.ring = entries;
    return TURNER_OK;
}

int turner_set_traversal_refill(turner_ctx* ctx, int kind, uint32_t lanes) {
    if (!ctx || kind < 0 || kind >= TURNER_RAYS_KINDS || lanes < 1 || lanes > 32) return TURNER_ERR_INVALID_ARG;
    ctx->refill[kind] = lanes;
    return TURNER_OK;
}

int turner_set_traversal_launch(turner_ctx* ctx, int persistent, uint32_t blocks_per_sm) {
    if (!ctx || blocks_per_sm > 64) return TURNER_ERR_INVALID_ARG;
    ctx->traverse.persistent = persistent != 0;
    ctx->traverse.blocks_per_sm = blocks_per_sm;
    return TURNER_OK;
}

} // extern "C"

namespace {

// A batch of jobs laid out for one launch sequence: the device job table,
// the pixel chunks (passes) and the workspace size.
struct Batch {
    std::vector<JobDesc> table;
    std::vector<Chunk> chunks;
    uint64_t total_pixels = 0;
    uint32_t cap = 0;                // queue entries per pass (paths, or rays of a level with -m > 1)
    int levels = 0;                  // largest max_depth + 1
    bool single_scene = true;
    SceneView single{};
    uint32_t max_height = 0;         // deepest traversal stack any scene needs
    bool guided = false;             // some job samples with the learned proposal
    bool branching = false;          // some job has -m > 1 (radiance is added atomically)
    bool has_path = false;           // some job uses the path tracer
    bool has_classic = false;        // some job uses the raytracer or the raycaster
};

int plan_batch(turner_ctx* ctx, const turner_job* jobs, uint32_t n_jobs, float4* const* outs, bool tone_map,
               Batch& b) {
    b.table.resize(n_jobs);
    uint64_t pixels = 0, paths = 0, load = 0, max_load = 1;
    std::vector<uint64_t> width(n_jobs);
    for (uint32_t j = 0; j < n_jobs; ++j) {
        fill_job(jobs[j], ctx->scenes[jobs[j].scene_id]->view, b.table[j]);
        JobDesc& d = b.table[j];
        d.tone_map = tone_map ? 1 : 0;
        d.guide_depth = ctx->guide_depth;
        d.pixel_offset = pixels;
        d.path_offset = paths;
        d.out = outs ? outs[j] : nullptr;
        pixels += uint64_t(d.width) * d.rows;
        paths += uint64_t(d.width) * d.rows * d.spp;
        width[j] = branch_width(jobs[j]);
        load += uint64_t(d.width) * d.rows * d.spp * width[j];
        max_load = std::max<uint64_t>(max_load, uint64_t(d.spp) * width[j]);
        if (width[j] > 1) b.branching = true;
        if (d.renderer == TURNER_RENDERER_PATH) b.has_path = true;
        else b.has_classic = true;
        b.levels = std::max(b.levels, d.max_depth + 1);
        if (jobs[j].scene_id != jobs[0].scene_id) b.single_scene = false;
        b.max_height = std::max(b.max_height, d.sc.height);
        if (d.sampling == TURNER_SAMPLING_GUIDED) b.guided = true;
    }
    b.total_pixels = pixels;
    b.single = b.table[0].sc;
    if (max_load > (1ull << 30)) return TURNER_ERR_TOO_LARGE;   // one pixel must fit a pass
    b.cap = static_cast<uint32_t>(std::min<uint64_t>(load, std::max<uint64_t>(ctx->chunk_paths, max_load)));
    (void)paths;
    // whole pixels, at most cap queue entries per level per chunk; a chunk
    // may span several jobs
    Chunk c{0, 0, 0, 0, 0};
    for (uint32_t j = 0; j < n_jobs; ++j) {
        const JobDesc& d = b.table[j];
        const uint64_t per_pixel = uint64_t(d.spp) * width[j];
        uint64_t left = uint64_t(d.width) * d.rows;
        while (left > 0) {
            const uint64_t room = (b.cap - c.n_rays) / per_pixel;
            if (room == 0) {
                b.chunks.push_back(c);
                c = Chunk{c.pixel0 + c.n_pixels, c.path0 + c.n_paths, 0, 0, 0};
                continue;
            }
            const uint64_t take = std::min(room, left);
            c.n_pixels += static_cast<uint32_t>(take);
            c.n_paths += static_cast<uint32_t>(take * d.spp);
            c.n_rays += static_cast<uint32_t>(take * per_pixel);
            left -= take;
        }
    }
    if (c.n_pixels) b.chunks.push_back(c);
    return TURNER_OK;
}

int ensure_workspace(turner_ctx* ctx, const Batch& b) {
    const uint32_t cap = b.cap;
    TURNER_CK(ctx->L.ensure(sizeof(float4) * cap));
    for (int k = 0; k < 3; ++k) {
        TURNER_CK(ctx->qa[k].ensure(sizeof(float4) * cap));
        TURNER_CK(ctx->qb[k].ensure(sizeof(float4) * cap));
        TURNER_CK(ctx->shq[k].ensure(sizeof(float4) * cap));
    }
    TURNER_CK(ctx->qa[3].ensure(sizeof(uint2) * cap));
    TURNER_CK(ctx->qb[3].ensure(sizeof(uint2) * cap));
    TURNER_CK(ctx->shjob.ensure(sizeof(uint32_t) * cap));
    if (b.has_classic) TURNER_CK(ctx->shaux.ensure(sizeof(uint32_t) * cap));
    TURNER_CK(ctx->hits.ensure(sizeof(Hit) * cap));
    TURNER_CK(ctx->counters.ensure(sizeof(uint32_t) * 4 * size_t(b.levels + 1) * b.chunks.size()));
    TURNER_CK(ctx->jobtab.ensure(sizeof(JobDesc) * b.table.size()));
    TURNER_CK(ctx->jobcnt.ensure(sizeof(unsigned long long) * 2 * b.table.size()));
    if (b.guided) {
        TURNER_CK(ctx->gfeat.ensure(sizeof(float) * 9 * size_t(cap)));
        TURNER_CK(ctx->gout.ensure(sizeof(float) * guide::kOut * size_t(cap)));
        if (ctx->guide_train) {
            const size_t rc = ctx->guide_records;
            TURNER_CK(ctx->qa_rec.ensure(sizeof(uint32_t) * cap));
            TURNER_CK(ctx->qb_rec.ensure(sizeof(uint32_t) * cap));
            TURNER_CK(ctx->r_feat.ensure(sizeof(float) * 9 * rc));
            TURNER_CK(ctx->r_dir.ensure(sizeof(float) * 3 * rc));
            TURNER_CK(ctx->r_weight.ensure(sizeof(float) * rc));
            TURNER_CK(ctx->r_path.ensure(sizeof(uint32_t) * rc));
            TURNER_CK(ctx->r_lbefore.ensure(sizeof(float) * rc));
            TURNER_CK(ctx->r_tafter.ensure(sizeof(float) * rc));
            TURNER_CK(ctx->r_fcp.ensure(sizeof(float) * rc));
            TURNER_CK(ctx->r_count.ensure(sizeof(uint32_t)));
        }
    }
    return TURNER_OK;
}

// Every launch of the batch on ctx->stream, no host synchronization (so the
// sequence can be captured into a CUDA graph). acc != nullptr: accumulate
// linear radiance in FP64 instead of resolving images.
int launch_batch(turner_ctx* ctx, const Batch& b, double4* acc) {
    const size_t stride = 4 * size_t(b.levels + 1);
    uint32_t* counters = ctx->counters.as<uint32_t>();
    const JobDesc* jobs = ctx->jobtab.as<JobDesc>();
    const uint32_t n_jobs = static_cast<uint32_t>(b.table.size());
    unsigned long long* job_counts = ctx->jobcnt.as<unsigned long long>();
    TURNER_CK(cudaMemsetAsync(counters, 0, sizeof(uint32_t) * stride * b.chunks.size(), ctx->stream));
    TURNER_CK(cudaMemsetAsync(job_counts, 0, sizeof(unsigned long long) * 2 * n_jobs, ctx->stream));
    const SceneView* single = b.single_scene ? &b.single : nullptr;
    int fast = 1;
    for (const JobDesc& d : b.table) fast &= d.traversal == TURNER_TRAVERSAL_FAST ? 1 : 0;
    const bool train = b.guided && ctx->guide_train;
    const RayQueue qa{ctx->qa[0].as<float4>(), ctx->qa[1].as<float4>(), ctx->qa[2].as<float4>(),
                      ctx->qa[3].as<uint2>(), nullptr, train ? ctx->qa_rec.as<uint32_t>() : nullptr};
    const RayQueue qb{ctx->qb[0].as<float4>(), ctx->qb[1].as<float4>(), ctx->qb[2].as<float4>(),
                      ctx->qb[3].as<uint2>(), nullptr, train ? ctx->qb_rec.as<uint32_t>() : nullptr};
    const GuideQueue gq{b.guided ? ctx->gfeat.as<float>() : nullptr, b.guided ? ctx->gout.as<float>() : nullptr};
    Records recs{};
    if (train) {
        recs = Records{ctx->r_feat.as<float>(), ctx->r_dir.as<float>(), ctx->r_weight.as<float>(),
                       ctx->r_path.as<uint32_t>(), ctx->r_lbefore.as<float>(), ctx->r_tafter.as<float>(),
                       ctx->r_fcp.as<float>(), ctx->r_count.as<uint32_t>(), ctx->guide_records, 0};
    }
    ShadowQueue sh{ctx->shq[0].as<float4>(), ctx->shq[1].as<float4>(), ctx->shq[2].as<float4>(),
                   ctx->shjob.as<uint32_t>(), nullptr, b.has_classic ? ctx->shaux.as<uint32_t>() : nullptr};
    for (size_t ci = 0; ci < b.chunks.size(); ++ci) {
        const Chunk& c = b.chunks[ci];
        uint32_t* cnt = counters + stride * ci;   // [queued rays | shadow rays | trace work | shadow work]
        RayQueue cur = qa, nxt = qb;
        cur.count = cnt;
        if (train) {
            // keep about guide_records of this pass's bounces, spread over all paths
            const double bounces = double(c.n_paths) * std::max(1, std::min(b.levels - 1, ctx->guide_depth));
            recs.keep = static_cast<uint32_t>(std::min(16777216.0, 16777216.0 * ctx->guide_records / bounces));
            TURNER_CK(cudaMemsetAsync(recs.count, 0, sizeof(uint32_t), ctx->stream));
        }
        {
            KernelTimer kt(ctx, TURNER_KERNEL_CAMERA);
            launch_camera(jobs, n_jobs, c, cur, ctx->L.as<float4>(), ctx->stream);
        }
        for (int depth = 0; depth < b.levels; ++depth) {
            nxt.count = cnt + depth + 1;
            sh.count = cnt + (b.levels + 1) + depth;
            TraverseCfg trace_cfg = ctx->traverse;
            if (b.max_height > 64) trace_cfg.stack = kStackCap;   // the short stack only where every scene fits
            TraverseCfg shadow_cfg = trace_cfg;
            trace_cfg.work = cnt + 2 * (b.levels + 1) + depth;
            shadow_cfg.work = cnt + 3 * (b.levels + 1) + depth;
            trace_cfg.refill = ctx->refill[depth == 0 ? TURNER_RAYS_PRIMARY : TURNER_RAYS_BOUNCE];
            shadow_cfg.refill = ctx->refill[depth == 0 ? TURNER_RAYS_SHADOW_PRIMARY : TURNER_RAYS_SHADOW];
            // packets where whole warps of coherent rays arrive: camera rays (their
            // shadow rays measured slower as packets)
            trace_cfg.packet = (ctx->packet_mode & TURNER_PACKET_CAMERA) && depth == 0;
            shadow_cfg.packet = false;
            {
                KernelTimer kt(ctx, TURNER_KERNEL_TRACE);
                launch_trace(single, jobs, cur, ctx->hits.as<Hit>(), c.n_rays, fast, trace_cfg, ctx->stream);
            }
            if (b.guided && depth + 1 < b.levels && depth < ctx->guide_depth) {
                {
                    KernelTimer kt(ctx, TURNER_KERNEL_GUIDE_FEATURES);
                    launch_guide_features(jobs, depth, cur, ctx->hits.as<Hit>(), gq.feat, c.n_paths, ctx->stream);
                }
                int gs;
                {
                    KernelTimer kt(ctx, TURNER_KERNEL_MLP_FORWARD);
                    gs = guide::forward_queue(ctx->guide, gq.feat, cur.count, c.n_paths, gq.out, ctx->stream);
                }
                if (gs != TURNER_OK) return gs;
            }
            if (b.has_path) {
                KernelTimer kt(ctx, TURNER_KERNEL_SHADE);
                launch_shade(jobs, depth, cur, ctx->hits.as<Hit>(), nxt, sh, ctx->L.as<float4>(), job_counts, gq,
                             recs, c.n_rays, b.has_classic, ctx->stream);
            }
            if (b.has_classic) {
                KernelTimer kt(ctx, TURNER_KERNEL_SHADE);
                launch_shade_classic(jobs, depth, cur, ctx->hits.as<Hit>(), nxt, sh, ctx->L.as<float4>(), job_counts,
                                     c.n_rays, ctx->stream);
            }
            {
                KernelTimer kt(ctx, TURNER_KERNEL_SHADOW);
                launch_shadow(single, jobs, sh, ctx->L.as<float4>(), c.n_rays, b.branching, nxt.T, shadow_cfg,
                              ctx->stream);
            }
            std::swap(cur, nxt);
        }
        {
            KernelTimer kt(ctx, TURNER_KERNEL_RESOLVE);
            if (acc) launch_accumulate(jobs, n_jobs, c, ctx->L.as<float4>(), acc, ctx->stream);
            else launch_resolve(jobs, n_jobs, c, ctx->L.as<float4>(), ctx->stream);
        }
        TURNER_CK(cudaGetLastError());
        if (train) {
            // online training: this pass's bounces, weighted by the radiance they brought back
            // (no host synchronisation: the step reads the record count on the device and
            // skips itself when fewer than 128 bounces were recorded)
            KernelTimer kt(ctx, TURNER_KERNEL_GUIDE_TRAIN, true);
            int gs = guide::finalize_records(recs.count, recs.cap, ctx->L.as<float4>(), recs.path, recs.l_before,
                                             recs.t_after, recs.fcos_pdf, recs.weight, ctx->guide_weighting,
                                             ctx->stream);
            if (gs != TURNER_OK) return gs;
            for (uint32_t k = 0; k < ctx->guide_steps_per_pass; ++k) {
                gs = guide::train_device(ctx->guide, recs.feat, recs.dir, recs.weight, recs.cap, recs.count, 128,
                                         ctx->guide_lr, ctx->stream, nullptr);
                if (gs != TURNER_OK) return gs;
                ctx->launches += 3;   // prep, forward, backward (with the Adam step and the repack)
            }
        }
    }
    return TURNER_OK;
}

// Runs a planned batch: uploads the job table, launches (through a CUDA graph
// for multi-job batches), synchronizes and fills per-job statistics.
int run_batch(turner_ctx* ctx, const Batch& b, double4* acc, turner_stats* stats, bool use_graph) {
    int st = ensure_workspace(ctx, b);
    if (st != TURNER_OK) return st;
    TURNER_CK(cudaMemcpyAsync(ctx->jobtab.p, b.table.data(), sizeof(JobDesc) * b.table.size(),
                              cudaMemcpyHostToDevice, ctx->stream));
    TURNER_CK(cudaEventRecord(ctx->ev0, ctx->stream));
    if (use_graph) {
        cudaGraph_t graph = nullptr;
        cudaGraphExec_t exec = nullptr;
        const bool prof = ctx->profiling;
        ctx->profiling = false;   // no per-kernel event pairs inside a captured graph
        TURNER_CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
        st = launch_batch(ctx, b, acc);
        const cudaError_t ec = cudaStreamEndCapture(ctx->stream, &graph);
        ctx->profiling = prof;
        if (st != TURNER_OK) {
            if (graph) cudaGraphDestroy(graph);
            return st;
        }
        TURNER_CK(ec);
        // A batch of the same shape captures the same topology with new
        // parameters: update the previous executable instead of
        // instantiating a new one (instantiation costs milliseconds).
        cudaError_t e = cudaSuccess;
        if (ctx->graph_exec) {
            cudaGraphExecUpdateResultInfo info{};
            if (cudaGraphExecUpdate(ctx->graph_exec, graph, &info) == cudaSuccess) {
                exec = ctx->graph_exec;
                ctx->graph_updates += 1;
            } else {
                cudaGetLastError();   // clear the update's error; instantiate below
                cudaGraphExecDestroy(ctx->graph_exec);
                ctx->graph_exec = nullptr;
            }
        }
        if (!exec) {
            e = cudaGraphInstantiate(&exec, graph, 0);
            if (e == cudaSuccess) ctx->graph_exec = exec;
        }
        if (e == cudaSuccess) e = cudaGraphLaunch(exec, ctx->stream);
        ctx->graph_launches += e == cudaSuccess ? 1 : 0;
        cudaGraphDestroy(graph);
        TURNER_CK(e);
    } else {
        st = launch_batch(ctx, b, acc);
        if (st != TURNER_OK) return st;
    }
    TURNER_CK(cudaEventRecord(ctx->ev1, ctx->stream));
    std::vector<unsigned long long> counts(2 * b.table.size());
    TURNER_CK(cudaMemcpyAsync(counts.data(), ctx->jobcnt.p, sizeof(unsigned long long) * counts.size(),
                              cudaMemcpyDeviceToHost, ctx->stream));
    TURNER_CK(cudaStreamSynchronize(ctx->stream));
    collect_kernel_times(ctx);
    if (stats) {
        float ms = 0;
        cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
        for (size_t j = 0; j < b.table.size(); ++j) {
            const JobDesc& d = b.table[j];
            stats[j].rays = counts[2 * j];
            stats[j].shadow_rays = counts[2 * j + 1];
            stats[j].primary_rays = uint64_t(d.width) * d.rows * d.spp;
            stats[j].device_ms = ms;
        }
    }
    return TURNER_OK;
}

} // namespace

extern "C" {

int turner_render(turner_ctx* ctx, const turner_job* jobs, uint32_t n_jobs, float* const* out_rgba,
                  turner_stats* stats, uint32_t flags) {
    if (!ctx || !jobs || !out_rgba || n_jobs == 0 || flags > TURNER_DEVICE_BUFFERS) return TURNER_ERR_INVALID_ARG;
    if (n_jobs > TURNER_MAX_JOBS) return TURNER_ERR_TOO_LARGE;
    for (uint32_t j = 0; j < n_jobs; ++j) {
        if (!out_rgba[j]) return TURNER_ERR_INVALID_ARG;
        const int st = check_job(ctx, jobs[j]);
        if (st != TURNER_OK) return st;
    }
    TURNER_CK(cudaSetDevice(ctx->device));
    std::vector<float4*> outs(n_jobs);
    uint64_t total = 0;
    for (uint32_t j = 0; j < n_jobs; ++j) total += job_pixels(jobs[j]);
    if (flags == TURNER_HOST_BUFFERS) {
        TURNER_CK(ctx->image.ensure(sizeof(float4) * total));
        uint64_t off = 0;
        for (uint32_t j = 0; j < n_jobs; ++j) {
            outs[j] = ctx->image.as<float4>() + off;
            off += job_pixels(jobs[j]);
        }
    } else {
        for (uint32_t j = 0; j < n_jobs; ++j) outs[j] = reinterpret_cast<float4*>(out_rgba[j]);
    }
    Batch b;
    int st = plan_batch(ctx, jobs, n_jobs, outs.data(), true, b);
    if (st != TURNER_OK) return st;
    for (uint32_t j = 0; j < n_jobs; ++j) b.table[j].tone_map = jobs[j].linear_output ? 0 : 1;
    const bool graph = ctx->graph_mode == TURNER_GRAPH_ALWAYS || (ctx->graph_mode == TURNER_GRAPH_AUTO && n_jobs > 1);
    st = run_batch(ctx, b, nullptr, stats, graph && !(b.guided && ctx->guide_train));
    if (st != TURNER_OK) return st;
    if (flags == TURNER_HOST_BUFFERS) {
        for (uint32_t j = 0; j < n_jobs; ++j) {
            TURNER_CK(cudaMemcpyAsync(out_rgba[j], outs[j], sizeof(float4) * job_pixels(jobs[j]),
                                      cudaMemcpyDeviceToHost, ctx->stream));
        }
        TURNER_CK(cudaStreamSynchronize(ctx->stream));
    }
    return TURNER_OK;
}

int turner_render_accumulate(turner_ctx* ctx, const turner_job* job, uint32_t passes, double* out_rgba_mean,
                             uint64_t* total_samples, uint32_t flags) {
    if (!ctx || !job || flags > TURNER_DEVICE_BUFFERS) return TURNER_ERR_INVALID_ARG;
    int st = check_job(ctx, *job);
    if (st != TURNER_OK) return st;
    TURNER_CK(cudaSetDevice(ctx->device));
    const uint64_t n = job_pixels(*job);
    // the running sum is keyed by what the image depends on; anything else resets it
    const uint64_t key[7] = {job->scene_id, job->width, job->height, job->seed,
                             uint64_t(uint32_t(job->max_depth)) << 32 | uint32_t(job->sampling),
                             uint64_t(uint32_t(job->monte_carlo_samples)),
                             uint64_t(job->row_begin) << 32 | job->row_end};
    if (std::memcmp(key, ctx->acc_key, sizeof(key)) != 0 || ctx->acc_samples == 0) {
        TURNER_CK(ctx->acc.ensure(sizeof(double4) * n));
        TURNER_CK(cudaMemsetAsync(ctx->acc.p, 0, sizeof(double4) * n, ctx->stream));
        std::memcpy(ctx->acc_key, key, sizeof(key));
        ctx->acc_samples = 0;
        ctx->acc_passes = 0;
    }
    for (uint32_t p = 0; p < passes; ++p) {
        turner_job jp = *job;
        // each pass draws fresh streams: a distinct seed base per pass
        jp.seed = job->seed ^ (0x9E3779B97F4A7C15ULL * (ctx->acc_passes + 1));
        Batch b;
        st = plan_batch(ctx, &jp, 1, nullptr, false, b);
        if (st != TURNER_OK) return st;
        st = run_batch(ctx, b, ctx->acc.as<double4>(), nullptr,
                       ctx->graph_mode == TURNER_GRAPH_ALWAYS && !(b.guided && ctx->guide_train));
        if (st != TURNER_OK) return st;
        ctx->acc_passes += 1;
        ctx->acc_samples += job->pixel_samples;
    }
    if (!out_rgba_mean) {   // the sum stays on the device
        if (total_samples) *total_samples = ctx->acc_samples;
        return TURNER_OK;
    }
    std::vector<double> sums(4 * n);
    TURNER_CK(cudaMemcpyAsync(sums.data(), ctx->acc.p, sizeof(double) * sums.size(), cudaMemcpyDeviceToHost,
                              ctx->stream));
    TURNER_CK(cudaStreamSynchronize(ctx->stream));
    const double inv = ctx->acc_samples ? 1.0 / static_cast<double>(ctx->acc_samples) : 0.0;
    for (double& v : sums) v *= inv;
    if (flags == TURNER_HOST_BUFFERS) {
        std::memcpy(out_rgba_mean, sums.data(), sizeof(double) * sums.size());
    } else {
        TURNER_CK(cudaMemcpyAsync(out_rgba_mean, sums.data(), sizeof(double) * sums.size(), cudaMemcpyHostToDevice,
                                  ctx->stream));
        TURNER_CK(cudaStreamSynchronize(ctx->stream));
    }
    if (total_samples) *total_samples = ctx->acc_samples;
    return TURNER_OK;
}

} // extern "C"

// ------------------------------------------------------------------ tuning
namespace {

uint64_t fnv1a(uint64_t h, const void* p, size_t n) {
    const unsigned char* c = static_cast<const unsigned char*>(p);
    for (size_t i = 0; i < n; ++i) h = (h ^ c[i]) * 0x100000001B3ULL;
    return h;
}

// What a tuning result depends on: the GPU and the shape of the batch.
std::string tuning_key(turner_ctx* ctx, const turner_job* jobs, uint32_t n_jobs) {
    cudaDeviceProp prop{};
    cudaGetDeviceProperties(&prop, ctx->device);
    uint64_t h = 0xCBF29CE484222325ULL;
    for (uint32_t j = 0; j < n_jobs; ++j) {
        const SceneView& v = ctx->scenes[jobs[j].scene_id]->view;
        const uint64_t f[9] = {v.n_tris, v.n_nodes, v.height, jobs[j].width, job_rows(jobs[j]),
                               jobs[j].pixel_samples, uint64_t(uint32_t(jobs[j].max_depth)),
                               uint64_t(uint32_t(jobs[j].sampling)), uint64_t(uint32_t(jobs[j].traversal))};
        h = fnv1a(h, f, sizeof(f));
    }
    char buf[64];
    std::snprintf(buf, sizeof(buf), "%016llx", static_cast<unsigned long long>(h));
    std::string name(prop.name);
    for (char& c : name) if (c == ' ' || c == '|') c = '_';
    return name + "|sm" + std::to_string(prop.multiProcessorCount) + "|" + buf;
}

std::string tuning_cache_path() {
    if (const char* p = std::getenv("TURNER_TUNE_CACHE")) return p;
    const char* home = std::getenv("HOME");
    return std::string(home ? home : "/tmp") + "/.cache/turner_gb300_tuning.txt";
}

bool tuning_lookup(const std::string& key, turner_tuning& t) {
    FILE* f = std::fopen(tuning_cache_path().c_str(), "r");
    if (!f) return false;
    char line[512];
    bool found = false;
    while (std::fgets(line, sizeof(line), f)) {
        char k[256];
        turner_tuning r{};
        if (std::sscanf(line, "%255s %d %u %u %u %u %u %u %lf %u %u %u", k, &r.persistent, &r.blocks_per_sm, &r.block,
                        &r.stack, &r.chunk_paths, &r.mailbox, &r.min_blocks, &r.ms, &r.refill_camera,
                        &r.refill_bounce, &r.packets) == 12 && key == k) {
            t = r;
            found = true;   // the last entry for a key wins
        }
    }
    std::fclose(f);
    return found;
}

void tuning_store(const std::string& key, const turner_tuning& t) {
    FILE* f = std::fopen(tuning_cache_path().c_str(), "a");
    if (!f) return;
    std::fprintf(f, "%s %d %u %u %u %u %u %u %.4f %u %u %u\n", key.c_str(), t.persistent, t.blocks_per_sm, t.block,
                 t.stack, t.chunk_paths, t.mailbox, t.min_blocks, t.ms, t.refill_camera, t.refill_bounce, t.packets);
    std::fclose(f);
}

bool valid_min_blocks(uint32_t v) { return v == 0 || v == 10 || v == 12 || v == 16; }

void apply_tuning(turner_ctx* ctx, const turner_tuning& t) {
    ctx->traverse.persistent = t.persistent != 0;
    ctx->traverse.blocks_per_sm = t.blocks_per_sm;
    ctx->traverse.block = t.block == 256 ? 256 : 128;
    ctx->traverse.stack = t.stack == 64 ? 64 : kStackCap;
    ctx->traverse.mailbox = t.mailbox != 0;
    ctx->traverse.min_blocks = valid_min_blocks(t.min_blocks) ? t.min_blocks : 0;
    ctx->chunk_paths = std::max<uint32_t>(1024, t.chunk_paths);
    if (t.refill_camera >= 1 && t.refill_camera <= 32) ctx->refill[TURNER_RAYS_PRIMARY] = t.refill_camera;
    if (t.refill_bounce >= 1 && t.refill_bounce <= 32) ctx->refill[TURNER_RAYS_BOUNCE] = t.refill_bounce;
    ctx->packet_mode = (ctx->packet_mode & ~TURNER_PACKET_CAMERA) | (t.packets ? TURNER_PACKET_CAMERA : 0);
}

} // namespace

extern "C" {

int turner_set_tuning(turner_ctx* ctx, const turner_tuning* t) {
    if (!ctx || !t) return TURNER_ERR_INVALID_ARG;
    if ((t->block != 128 && t->block != 256) || (t->stack != 64 && t->stack != kStackCap) || t->blocks_per_sm > 64 ||
        t->chunk_paths < 1024 || t->mailbox > 1 || !valid_min_blocks(t->min_blocks) || t->refill_camera < 1 ||
        t->refill_camera > 32 || t->refill_bounce < 1 || t->refill_bounce > 32 || t->packets > 1)
        return TURNER_ERR_INVALID_ARG;
    apply_tuning(ctx, *t);
    return TURNER_OK;
}

int turner_get_tuning(turner_ctx* ctx, turner_tuning* t) {
    if (!ctx || !t) return TURNER_ERR_INVALID_ARG;
    t->persistent = ctx->traverse.persistent ? 1 : 0;
    t->blocks_per_sm = ctx->traverse.blocks_per_sm;
    t->block = ctx->traverse.block;
    t->stack = ctx->traverse.stack;
    t->chunk_paths = ctx->chunk_paths;
    t->mailbox = ctx->traverse.mailbox ? 1 : 0;
    t->min_blocks = ctx->traverse.min_blocks;
    t->ms = 0;
    t->candidates = 0;
    t->refill_camera = ctx->refill[TURNER_RAYS_PRIMARY];
    t->refill_bounce = ctx->refill[TURNER_RAYS_BOUNCE];
    t->packets = (ctx->packet_mode & TURNER_PACKET_CAMERA) ? 1 : 0;
    return TURNER_OK;
}

int turner_autotune(turner_ctx* ctx, const turner_job* jobs, uint32_t n_jobs, int force, turner_tuning* out) {
    if (!ctx || !jobs || n_jobs == 0 || n_jobs > TURNER_MAX_JOBS) return TURNER_ERR_INVALID_ARG;
    for (uint32_t j = 0; j < n_jobs; ++j) {
        const int st = check_job(ctx, jobs[j]);
        if (st != TURNER_OK) return st;
    }
    TURNER_CK(cudaSetDevice(ctx->device));
    const std::string key = tuning_key(ctx, jobs, n_jobs);
    turner_tuning best{};
    if (!force && tuning_lookup(key, best)) {
        apply_tuning(ctx, best);
        best.candidates = 0;
        if (out) *out = best;
        return TURNER_OK;
    }
    uint32_t max_height = 0;
    uint64_t total_paths = 0, total_pixels = 0;
    for (uint32_t j = 0; j < n_jobs; ++j) {
        max_height = std::max(max_height, ctx->scenes[jobs[j].scene_id]->view.height);
        total_pixels += job_pixels(jobs[j]);
        total_paths += job_pixels(jobs[j]) * jobs[j].pixel_samples;
    }
    TURNER_CK(ctx->tune_out.ensure(sizeof(float4) * total_pixels));
    std::vector<float*> outs(n_jobs);
    uint64_t off = 0;
    for (uint32_t j = 0; j < n_jobs; ++j) {
        outs[j] = reinterpret_cast<float*>(ctx->tune_out.as<float4>() + off);
        off += job_pixels(jobs[j]);
    }
    std::vector<turner_stats> st(n_jobs);
    uint32_t tried = 0;
    auto measure = [&](const turner_tuning& t, double& ms) -> int {
        apply_tuning(ctx, t);
        double best_ms = 1e300;
        for (int rep = 0; rep < 2; ++rep) {   // the first run warms caches and allocates the workspace
            const int s = turner_render(ctx, jobs, n_jobs, outs.data(), st.data(), TURNER_DEVICE_BUFFERS);
            if (s != TURNER_OK) return s;
            if (rep) best_ms = st[0].device_ms;
        }
        ms = best_ms;
        ++tried;
        return TURNER_OK;
    };
    // coordinate descent from the defaults, one knob at a time
    turner_tuning cur{1, 0, 128, kStackCap, 1u << 24, 0, 10, 0, 0, 32, 2, 1};
    int s = measure(cur, cur.ms);
    if (s != TURNER_OK) return s;
    const uint32_t blocks[] = {128, 256};
    const uint32_t per_sm[] = {0, 8, 6, 4};
    const uint32_t stacks[] = {kStackCap, 64};
    const uint32_t chunks[] = {1u << 24, 1u << 22, 1u << 20};
    auto try_value = [&](auto setter, const auto& values) -> int {
        for (const auto v : values) {
            turner_tuning cand = cur;
            if (!setter(cand, v)) continue;
            double ms = 0;
            const int r = measure(cand, ms);
            if (r != TURNER_OK) return r;
            if (ms < cur.ms * 0.99) {
                cur = cand;
                cur.ms = ms;
            }
        }
        return TURNER_OK;
    };
    s = try_value([&](turner_tuning& t, uint32_t v) { if (t.block == v) return false; t.block = v; return true; }, blocks);
    if (s == TURNER_OK)
        s = try_value([&](turner_tuning& t, uint32_t v) { if (t.blocks_per_sm == v) return false; t.blocks_per_sm = v; return true; },
                      per_sm);
    if (s == TURNER_OK)
        s = try_value([&](turner_tuning& t, uint32_t v) {
                if (t.stack == v || v < max_height) return false;
                t.stack = v;
                return true;
            }, stacks);
    if (s == TURNER_OK)
        s = try_value([&](turner_tuning& t, uint32_t v) {
                if (t.chunk_paths == v || (v > total_paths && t.chunk_paths >= total_paths)) return false;
                t.chunk_paths = v;
                return true;
            }, chunks);
    if (s == TURNER_OK)
        s = try_value([&](turner_tuning& t, uint32_t v) {
                if (t.mailbox == v || t.block != 128) return false;
                t.mailbox = v;
                return true;
            }, std::vector<uint32_t>{1});
    if (s == TURNER_OK)
        s = try_value([&](turner_tuning& t, uint32_t v) {
                if (t.min_blocks == v || t.block != 128) return false;
                t.min_blocks = v;
                return true;
            }, std::vector<uint32_t>{0, 12, 16});
    if (s == TURNER_OK)
        s = try_value([&](turner_tuning& t, uint32_t v) {
                if (t.refill_camera == v) return false;
                t.refill_camera = v;
                return true;
            }, std::vector<uint32_t>{16, 8});
    if (s == TURNER_OK)
        s = try_value([&](turner_tuning& t, uint32_t v) {
                if (t.refill_bounce == v) return false;
                t.refill_bounce = v;
                return true;
            }, std::vector<uint32_t>{1, 4});
    if (s == TURNER_OK)
        s = try_value([&](turner_tuning& t, uint32_t v) { if (t.packets == v) return false; t.packets = v; return true; },
                      std::vector<uint32_t>{0});
    if (s == TURNER_OK)
        s = try_value([&](turner_tuning& t, int v) { if (t.persistent == v) return false; t.persistent = v; return true; },
                      std::vector<int>{0});
    if (s != TURNER_OK) return s;
    cur.candidates = tried;
    apply_tuning(ctx, cur);
    tuning_store(key, cur);
    if (out) *out = cur;
    return TURNER_OK;
}

int turner_set_guide(turner_ctx* ctx, turner_guide* guide, int train, float lr, uint32_t records_per_pass) {
    if (!ctx || (train && !guide) || !(lr >= 0.f) || (train && records_per_pass < 128)) return TURNER_ERR_INVALID_ARG;
    if (guide && turner::guide::owner(guide) != ctx) return TURNER_ERR_INVALID_ARG;
    ctx->guide = guide;
    ctx->guide_train = train != 0 && guide;
    ctx->guide_lr = lr;
    if (records_per_pass) ctx->guide_records = records_per_pass;
    return TURNER_OK;
}

int turner_set_guide_weighting(turner_ctx* ctx, int mode) {
    if (!ctx || mode < 0 || mode > 2) return TURNER_ERR_INVALID_ARG;
    ctx->guide_weighting = mode;
    return TURNER_OK;
}

int turner_set_guide_depth(turner_ctx* ctx, uint32_t depth) {
    if (!ctx || depth < 1 || depth > 64) return TURNER_ERR_INVALID_ARG;
    ctx->guide_depth = static_cast<int32_t>(depth);
    return TURNER_OK;
}

int turner_set_guide_steps(turner_ctx* ctx, uint32_t steps_per_pass) {
    if (!ctx || steps_per_pass == 0 || steps_per_pass > 64) return TURNER_ERR_INVALID_ARG;
    ctx->guide_steps_per_pass = steps_per_pass;
    return TURNER_OK;
}

int turner_guide_stats(turner_ctx* ctx, uint64_t* steps, float* last_loss, double* train_ms) {
    if (!ctx) return TURNER_ERR_INVALID_ARG;
    if (steps) *steps = 0;
    if (last_loss) *last_loss = 0.f;
    if (ctx->guide) {
        TURNER_CK(cudaSetDevice(ctx->device));
        const int st = guide::train_state(ctx->guide, steps, last_loss);
        if (st != TURNER_OK) return st;
    }
    if (train_ms) *train_ms = ctx->guide_train_ms;
    return TURNER_OK;
}

int turner_set_graph_mode(turner_ctx* ctx, int mode) {
    if (!ctx) return TURNER_ERR_INVALID_ARG;
    if (mode < TURNER_GRAPH_AUTO || mode > TURNER_GRAPH_NEVER) return TURNER_ERR_INVALID_ARG;
    ctx->graph_mode = mode;
    return TURNER_OK;
}

uint64_t turner_graph_launch_count(turner_ctx* ctx) { return ctx ? ctx->graph_launches : 0; }

int turner_set_profiling(turner_ctx* ctx, int on) {
    if (!ctx) return TURNER_ERR_INVALID_ARG;
    ctx->profiling = on != 0;
    return TURNER_OK;
}

int turner_kernel_times(turner_ctx* ctx, double* ms, uint64_t* launches, int reset) {
    if (!ctx) return TURNER_ERR_INVALID_ARG;
    for (int k = 0; k < TURNER_KERNEL_KINDS; ++k) {
        if (ms) ms[k] = ctx->kernel_ms[k];
        if (launches) launches[k] = ctx->kernel_launches[k];
        if (reset) {
            ctx->kernel_ms[k] = 0;
            ctx->kernel_launches[k] = 0;
        }
    }
    return TURNER_OK;
}

} // extern "C"

// ------------------------------------------------ no-allocation intersect
// Scratch of turner_intersect_noalloc: word 0 is the work counter from which
// the persistent traversal's lanes claim rays. The array fills one 256-byte
// segment so that no other variable shares the cache lines of that heavily
// contended atomic. Every GPU that loads this library holds these 256 bytes
// until the process exits.
static __device__ __align__(256) uint32_t g_noalloc_scratch[TURNER_NOALLOC_SCRATCH_WORDS];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
uint32_t* g_noalloc_ptr[kMaxDevices] = {};

// Device address of g_noalloc_scratch on `device`, looked up once per device
// with that device current. In host code the array's name only stands in for
// the symbol; a kernel must be given this address instead.
int noalloc_scratch(int device, uint32_t** out) {
    if (device < 0 || device >= kMaxDevices) return TURNER_ERR_NO_DEVICE;
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ptr[device]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) return e != cudaSuccess ? map_cuda(e) : TURNER_ERR_CUDA;
        g_noalloc_ptr[device] = static_cast<uint32_t*>(p);
    }
    *out = g_noalloc_ptr[device];
    return TURNER_OK;
}

} // namespace

extern "C" {

int turner_intersect_noalloc(turner_ctx* ctx, uint32_t scene_id, const float* ox, const float* oy, const float* oz,
                             const float* dx, const float* dy, const float* dz, uint64_t n, uint32_t* hit_id,
                             float* r, float* s, float* t, int mode) {
    if (!ctx || scene_id >= ctx->scenes.size() || !ctx->scenes[scene_id]->live) return TURNER_ERR_INVALID_ARG;
    if (!ox || !oy || !oz || !dx || !dy || !dz || !hit_id || !r || !s || !t) return TURNER_ERR_INVALID_ARG;
    if (mode != TURNER_TRAVERSAL_PARITY && mode != TURNER_TRAVERSAL_FAST) return TURNER_ERR_INVALID_ARG;
    if (n > TURNER_NOALLOC_MAX_RAYS) return TURNER_ERR_TOO_LARGE;
    if (n == 0) return TURNER_OK;
    TURNER_CK(cudaSetDevice(ctx->device));
    uint32_t* scratch = nullptr;
    const int st = noalloc_scratch(ctx->device, &scratch);
    if (st != TURNER_OK) {
        ctx->last_error = "cudaGetSymbolAddress(g_noalloc_scratch) failed";
        return st;
    }
    // the array keeps the previous call's counter: it must start at zero
    TURNER_CK(cudaMemsetAsync(scratch, 0, sizeof(uint32_t), ctx->stream));
    // the context's launch configuration, as turner_intersect uses it
    const SceneView& sc = ctx->scenes[scene_id]->view;
    TraverseCfg cfg = ctx->traverse;
    if (sc.height > 64) cfg.stack = kStackCap;
    cfg.refill = ctx->refill[TURNER_RAYS_INTERSECT];
    cfg.packet = (ctx->packet_mode & TURNER_PACKET_BATCHED) != 0;
    cfg.work = scratch;
    {
        KernelTimer kt(ctx, TURNER_KERNEL_INTERSECT);
        launch_intersect(sc, ox, oy, oz, dx, dy, dz, n, hit_id, r, s, t, mode == TURNER_TRAVERSAL_FAST, cfg,
                         ctx->stream);
    }
    TURNER_CK(cudaGetLastError());
    TURNER_CK(cudaStreamSynchronize(ctx->stream));
    collect_kernel_times(ctx);
    return TURNER_OK;
}


} // extern "C"
