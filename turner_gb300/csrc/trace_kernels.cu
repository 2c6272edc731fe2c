// Wavefront path-tracing kernels for sm_103a (compiled with -fmad=false).
//
// One render pass over a chunk of whole pixels of a batch of images (the job
// table, `JobDesc`, lives in device memory):
//   k_camera   primary rays for every (pixel, sample) path        main.cpp:200-214
//   per depth 0..max depth of the batch:
//     k_traverse<QueueSrc>   closest hit of every queued ray     kdtree.cpp:516-607
//     k_shade   hit point, interpolated normal, offset, next-event
//               shadow ray, bounce direction; appends live paths to
//               the next queue (warp ballot + one atomic per warp)  pathtracer.cpp:14-102
//     k_traverse<ShadowSrc>  any-hit occlusion; adds the direct term   pathtracer.cpp:44-58
//   k_resolve  per-pixel mean over samples in sample order, then exposure and
//              gamma                                              main.cpp:216-223
// The radiance of a path is accumulated forward: L += T * diffuse *
// direct / pi at every hit (when the light is visible) and L += T * bg on a
// miss, with T *= diffuse * 2 cos(theta) per uniform bounce (diffuse for a
// cosine bounce). This is the reference's recursion
// L_k = diffuse * (direct / pi + 2 cos L_{k+1}) unrolled.
#include <algorithm>
#include <map>
#include <mutex>

#include "device.cuh"
#include "guide.cuh"
#include "kernels.h"

namespace turner {

namespace {

constexpr int kBlock = 128;

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31u; }

// Warp-aggregated append: one atomicAdd per warp, slots in lane order. Must
// be reached by every lane of the warp.
__device__ __forceinline__ uint32_t warp_append(uint32_t* counter, bool pred) {
    const unsigned mask = __ballot_sync(0xFFFFFFFFu, pred);
    if (mask == 0) return 0;
    const int leader = __ffs(mask) - 1;
    uint32_t base = 0;
    if (static_cast<int>(lane_id()) == leader) base = atomicAdd(counter, static_cast<uint32_t>(__popc(mask)));
    base = __shfl_sync(0xFFFFFFFFu, base, leader);
    return base + static_cast<uint32_t>(__popc(mask & ((1u << lane_id()) - 1u)));
}

// Appends `cnt` entries per lane (one atomic per warp); returns this lane's
// first slot. Every lane of the warp must call it.
__device__ __forceinline__ uint32_t warp_append_n(uint32_t* counter, uint32_t cnt) {
    const uint32_t lane = lane_id();
    uint32_t x = cnt;   // inclusive prefix sum over the warp
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, off);
        if (lane >= static_cast<uint32_t>(off)) x += y;
    }
    const uint32_t total = __shfl_sync(0xFFFFFFFFu, x, 31);
    if (total == 0) return 0;
    uint32_t base = 0;
    if (lane == 31) base = atomicAdd(counter, total);
    base = __shfl_sync(0xFFFFFFFFu, base, 31);
    return base + x - cnt;
}

__device__ __forceinline__ void atomic_add4(float4* p, float4 v) {
    atomicAdd(&p->x, v.x);
    atomicAdd(&p->y, v.y);
    atomicAdd(&p->z, v.z);
    atomicAdd(&p->w, v.w);
}

// Job owning global path g / global pixel p (job offsets ascend).
__device__ __forceinline__ uint32_t job_of_path(const JobDesc* jobs, uint32_t n_jobs, uint64_t g) {
    uint32_t lo = 0, hi = n_jobs;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (jobs[mid].path_offset <= g) lo = mid;
        else hi = mid;
    }
    return lo;
}

__device__ __forceinline__ uint32_t job_of_pixel(const JobDesc* jobs, uint32_t n_jobs, uint64_t p) {
    uint32_t lo = 0, hi = n_jobs;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (jobs[mid].pixel_offset <= p) lo = mid;
        else hi = mid;
    }
    return lo;
}

__global__ void __launch_bounds__(kBlock) k_intersect(SceneView sc, const float* __restrict__ ox,
                                                      const float* __restrict__ oy, const float* __restrict__ oz,
                                                      const float* __restrict__ dx, const float* __restrict__ dy,
                                                      const float* __restrict__ dz, uint64_t n,
                                                      uint32_t* __restrict__ hit_id, float* __restrict__ hr,
                                                      float* __restrict__ hs, float* __restrict__ ht, int fast) {
    const uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float3 o = make_float3(ox[i], oy[i], oz[i]);
    const float3 d = make_float3(dx[i], dy[i], dz[i]);
    const Hit h = fast ? traverse<false, true>(sc, o, d, 0.f) : traverse<false, false>(sc, o, d, 0.f);
    hit_id[i] = h.id;
    hr[i] = h.id < kMiss ? h.r : kFltMax;
    hs[i] = h.id < kMiss ? h.s : 0.f;
    ht[i] = h.id < kMiss ? h.t : 0.f;
}

// Camera::raster2cam (lib/types.h:117-123) with jitter from the path's own
// xorshift stream; the direction is not normalised.
__global__ void __launch_bounds__(kBlock) k_camera(const JobDesc* __restrict__ jobs, uint32_t n_jobs, Chunk c,
                                                   RayQueue q, float4* __restrict__ L) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) *q.count = c.n_paths;
    if (i >= c.n_paths) return;
    const uint64_t g = c.path0 + i;
    const uint32_t j = job_of_path(jobs, n_jobs, g);
    const JobDesc& job = jobs[j];
    const uint64_t local = g - job.path_offset;
    const uint64_t band_pixel = local / job.spp;
    const uint32_t sample = static_cast<uint32_t>(local - band_pixel * job.spp);
    // the pixel's index in the whole image: a band of rows draws the same
    // streams and rays as those rows of a full render
    const uint64_t pixel = uint64_t(job.row0) * job.width + band_pixel;
    const uint32_t y = static_cast<uint32_t>(pixel / job.width);
    const uint32_t x = static_cast<uint32_t>(pixel - uint64_t(y) * job.width);
    uint64_t js, bs;
    path_seeds(job.seed, pixel * job.spp + sample, js, bs);
    const float jx = xorshift_float(js);
    const float jy = xorshift_float(js);
    const float px = static_cast<float>(x) + jx, py = static_cast<float>(y) + jy;
    const float w = static_cast<float>(job.width), h = static_cast<float>(job.height);
    const float vx = -job.delta_x * (1 - 2 * px / w);
    const float vy = job.delta_y * (1 - 2 * py / h);
    const float vz = -1;
    const float* m = job.trafo;
    const float3 d = make_float3(m[0] * vx + m[1] * vy + m[2] * vz, m[3] * vx + m[4] * vy + m[5] * vz,
                                 m[6] * vx + m[7] * vy + m[8] * vz);
    q.o[i] = make_float4(job.cam_pos[0], job.cam_pos[1], job.cam_pos[2], __uint_as_float(i));
    q.d[i] = make_float4(d.x, d.y, d.z, __uint_as_float(j));
    q.T[i] = make_float4(1.f, 1.f, 1.f, 1.f);
    q.rng[i] = make_uint2(static_cast<uint32_t>(bs), static_cast<uint32_t>(bs >> 32));
    if (q.rec) q.rec[i] = kNoRecord;
    L[i] = make_float4(0.f, 0.f, 0.f, 0.f);
}

__device__ __forceinline__ float luminance(float4 c) { return 0.2126f * c.x + 0.7152f * c.y + 0.0722f * c.z; }

// Shading normal of a hit: Triangle::interpolate_normal(1 - s - t, s, t)
// (lib/triangle.h:54-56). Shared by k_shade and the network inputs.
__device__ __forceinline__ float3 shading_normal(const float4& s0, const float4& s1, const float4& s2, const Hit& h) {
    const float w0 = 1.f - h.s - h.t;
    const float nx = w0 * s0.x + h.s * s1.x + h.t * s2.x;
    const float ny = w0 * s0.y + h.s * s1.y + h.t * s2.y;
    const float nz = w0 * s0.z + h.s * s1.z + h.t * s2.z;
    const float inv_len = 1 / sqrtf(nx * nx + ny * ny + nz * nz);
    return make_float3(inv_len * nx, inv_len * ny, inv_len * nz);
}

__global__ void __launch_bounds__(kBlock) k_guide_features(const JobDesc* __restrict__ jobs, int depth, RayQueue q,
                                                           const Hit* __restrict__ hits, float* __restrict__ feat) {
    const uint32_t n = *q.count;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float f[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        const float4 d4 = q.d[i];
        const JobDesc& job = jobs[__float_as_uint(d4.w)];
        const Hit h = hits[i];
        if (job.sampling == kSamplingGuided && depth < job.guide_depth && depth < job.max_depth && job.mc > 0 &&
            h.id < kMiss) {
            const float4 o4 = q.o[i];
            const float3 p = make_float3(o4.x + h.r * d4.x, o4.y + h.r * d4.y, o4.z + h.r * d4.z);
            const float4* rec = job.sc.shade + 4 * size_t(h.id);
            const float4 s0 = __ldg(rec), s1 = __ldg(rec + 1), s2 = __ldg(rec + 2);
            const float3 nrm = shading_normal(s0, s1, s2, h);
            const float pp[3] = {p.x, p.y, p.z};
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const float ext = job.sc.hi[k] - job.sc.lo[k];
                f[k] = ext > 0.f ? fminf(fmaxf((pp[k] - job.sc.lo[k]) / ext, 0.f), 1.f) : 0.5f;
            }
            f[3] = nrm.x;
            f[4] = nrm.y;
            f[5] = nrm.z;
            f[6] = s0.w;
            f[7] = s1.w;
            f[8] = s2.w;
        }
#pragma unroll
        for (int k = 0; k < 9; ++k) feat[9 * size_t(i) + k] = f[k];
    }
}

__device__ __forceinline__ float4 mul4(float4 a, float4 b) { return make_float4(a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w); }
__device__ __forceinline__ float4 scale4(float s, float4 a) { return make_float4(s * a.x, s * a.y, s * a.z, s * a.w); }
__device__ __forceinline__ float4 add4(float4 a, float4 b) { return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
__device__ __forceinline__ float4 sub4(float4 a, float4 b) { return make_float4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }

__global__ void __launch_bounds__(kBlock) k_shade(const JobDesc* __restrict__ jobs, int depth, RayQueue in,
                                                  const Hit* __restrict__ hits, RayQueue out, ShadowQueue sh,
                                                  float4* __restrict__ L, unsigned long long* __restrict__ job_counts,
                                                  GuideQueue gq, Records recs, bool mixed) {
    const uint32_t n = *in.count;
    const uint32_t stride = gridDim.x * blockDim.x;
    // warp-uniform loop so every lane reaches the ballots
    for (uint32_t base = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); base < n; base += stride) {
        const uint32_t i = base + lane_id();
        // mixed: the batch also holds raytracer / raycaster jobs, whose entries
        // k_shade_classic shades
        const bool valid = i < n && (!mixed || jobs[__float_as_uint(in.d[i].w)].renderer == kRendererPath);
        bool emit_shadow = false, emit_bounce = false;
        float4 sh_o, sh_d, sh_c, b_o, b_d, b_T;
        uint2 b_rng;
        // -m > 1: n_branch children, each on its own stream derived from br_state
        uint32_t n_branch = 0, br_path = 0;
        uint64_t br_state = 0;
        float3 br_nrm = make_float3(0.f, 0.f, 0.f), br_p2 = br_nrm;
        float4 br_Td = make_float4(0.f, 0.f, 0.f, 0.f);
        uint32_t jidx = 0;
        bool emit_record = false;
        float rec_dir[3] = {0.f, 0.f, 0.f}, rec_t = 0.f, rec_fcp = 0.f;
        uint32_t rec_path = 0;
        if (valid) {
            const Hit h = hits[i];
            const float4 o4 = in.o[i];
            const float4 d4 = in.d[i];
            jidx = __float_as_uint(d4.w);
            const JobDesc& job = jobs[jidx];
            const uint32_t path = __float_as_uint(o4.w);
            const float4 T = in.T[i];
            if (in.rec) {
                // the bounce that spawned this ray: radiance of the path before its continuation
                const uint32_t r = in.rec[i];
                if (r != kNoRecord) recs.l_before[r] = luminance(L[path]);
            }
            if (h.id >= kMiss) {
                // miss: trace() returns conf.bg_color (alpha 1); with -m > 1 several rays
                // of one path are live at a time, so they add atomically
                const float4 add = mul4(T, make_float4(job.bg[0], job.bg[1], job.bg[2], 1.f));
                if (job.mc > 1) atomic_add4(L + path, add);
                else L[path] = add4(L[path], add);
            } else {
                const float3 p = make_float3(o4.x + h.r * d4.x, o4.y + h.r * d4.y, o4.z + h.r * d4.z);
                const float4* rec = job.sc.shade + 4 * size_t(h.id);
                const float4 s0 = __ldg(rec), s1 = __ldg(rec + 1), s2 = __ldg(rec + 2), s3 = __ldg(rec + 3);
                const float4 diffuse = make_float4(s0.w, s1.w, s2.w, s3.x);
                const float3 nrm = shading_normal(s0, s1, s2, h);
                const float3 p2 = make_float3(p.x + 0.0001f * nrm.x, p.y + 0.0001f * nrm.y, p.z + 0.0001f * nrm.z);
                const float4 Td = mul4(T, diffuse);
                if (job.n_lights > 0) {
                    const float lx = job.light_pos[0] - p.x, ly = job.light_pos[1] - p.y, lz = job.light_pos[2] - p.z;
                    const float inv_l = 1 / sqrtf(lx * lx + ly * ly + lz * lz);
                    const float3 ld = make_float3(inv_l * lx, inv_l * ly, inv_l * lz);
                    const float qx = job.light_pos[0] - p2.x, qy = job.light_pos[1] - p2.y, qz = job.light_pos[2] - p2.z;
                    const float dist = sqrtf(qx * qx + qy * qy + qz * qz);
                    const float c = fmaxf(0.f, ld.x * nrm.x + ld.y * nrm.y + ld.z * nrm.z);
                    if (c > 0.f) {
                        // a zero cosine contributes nothing whether or not the light is blocked
                        const float4 direct = scale4(c, make_float4(job.light_col[0], job.light_col[1],
                                                                    job.light_col[2], job.light_col[3]));
                        sh_c = mul4(Td, scale4(0.318309886183790671538f, direct));
                        sh_o = make_float4(p2.x, p2.y, p2.z, __uint_as_float(path));
                        sh_d = make_float4(ld.x, ld.y, ld.z, dist);
                        emit_shadow = true;
                    }
                }
                if (depth < job.max_depth && job.mc > 1) {
                    const uint2 r2 = in.rng[i];
                    n_branch = static_cast<uint32_t>(job.mc);
                    br_state = uint64_t(r2.x) | (uint64_t(r2.y) << 32);
                    br_nrm = nrm;
                    br_p2 = p2;
                    br_Td = Td;
                    br_path = path;
                } else if (depth < job.max_depth && job.mc > 0) {
                    float m[9];
                    from_to_z(nrm, m);
                    const uint2 r2 = in.rng[i];
                    uint64_t rs = uint64_t(r2.x) | (uint64_t(r2.y) << 32);
                    const float u1 = xorshift_float(rs);
                    const float u2 = xorshift_float(rs);
                    float x, y, z, weight;
                    float3 dir;
                    bool bounce = true;
                    // guided jobs sample from the proposal up to guide_depth, by cosine below
                    const bool guided = job.sampling == kSamplingGuided && depth < job.guide_depth;
                    if (guided) {
                        // learned proposal: 1/2 cosine about the normal, 1/2 the vMF mixture
                        // the network's 40 outputs of this hit: 160 bytes, read once as float4
                        float raw[guide::kOut];
                        const float4* o4 = reinterpret_cast<const float4*>(gq.out + guide::kOut * size_t(i));
#pragma unroll
                        for (int k = 0; k < guide::kOut / 4; ++k) {
                            const float4 v = __ldcs(o4 + k);
                            raw[4 * k] = v.x;
                            raw[4 * k + 1] = v.y;
                            raw[4 * k + 2] = v.z;
                            raw[4 * k + 3] = v.w;
                        }
                        guide::Mixture mix;
                        guide::decode(raw, mix);
                        const float u_sel = xorshift_float(rs);
                        const float ua = xorshift_float(rs);
                        const float ub = xorshift_float(rs);
                        const float uc = xorshift_float(rs);
                        float w3[3];
                        if (u_sel < 0.5f) {
                            const float rr = sqrtf(ua);
                            const float zz = sqrtf(fmaxf(0.f, 1.f - ua));
                            const float phi = 6.28318548202514648438f * ub;
                            const float xx = rr * cosf(phi), yy = rr * sinf(phi);
                            w3[0] = m[0] * xx + m[1] * yy + m[2] * zz;
                            w3[1] = m[3] * xx + m[4] * yy + m[5] * zz;
                            w3[2] = m[6] * xx + m[7] * yy + m[8] * zz;
                        } else {
                            // the first lobe whose cumulative weight reaches uc (the
                            // last one if rounding leaves the sum short), picked with
                            // static indices so that the mixture stays in registers
                            float sel[3] = {0.f, 0.f, 1.f}, sel_kappa = 1.f, acc = 0.f;
                            bool found = false;
#pragma unroll
                            for (int l = 0; l < guide::kLobes; ++l) {
                                acc += mix.w[l];
                                if (!found && (uc <= acc || l == guide::kLobes - 1)) {
                                    sel[0] = mix.mu[l][0];
                                    sel[1] = mix.mu[l][1];
                                    sel[2] = mix.mu[l][2];
                                    sel_kappa = mix.kappa[l];
                                    found = true;
                                }
                            }
                            float rot[9];
                            from_to_z(make_float3(sel[0], sel[1], sel[2]), rot);
                            guide::vmf_sample(sel, sel_kappa, ua, ub, rot, w3);
                        }
                        const float cw = nrm.x * w3[0] + nrm.y * w3[1] + nrm.z * w3[2];
                        const float pdf = 0.5f * guide::mixture_pdf(mix, w3) + 0.5f * fmaxf(cw, 0.f) * guide::kInvPi;
                        bounce = cw > 0.f && pdf > 0.f;   // below the surface the integrand is 0
                        weight = bounce ? cw * guide::kInvPi / pdf : 0.f;
                        dir = make_float3(w3[0], w3[1], w3[2]);
                        x = y = z = 0.f;
                        if (bounce && recs.count) {
                            const float u_keep = xorshift_float(rs);
                            emit_record = u_keep * 16777216.f < static_cast<float>(recs.keep);
                            rec_dir[0] = w3[0];
                            rec_dir[1] = w3[1];
                            rec_dir[2] = w3[2];
                            rec_path = path;
                            rec_fcp = luminance(diffuse) * weight;
                        }
                    } else if (job.sampling == 0) {
                        // sampling::hemisphere (lib/sampling.h:20-32)
                        z = u1;
                        const float rr = sqrtf(fmaxf(0.f, 1.f - z * z));
                        const float phi = 6.28318548202514648438f * u2;
                        x = rr * cosf(phi);
                        y = rr * sinf(phi);
                        weight = 2.f * u1;
                    } else {
                        const float rr = sqrtf(u1);
                        z = sqrtf(fmaxf(0.f, 1.f - u1));
                        const float phi = 6.28318548202514648438f * u2;
                        x = rr * cosf(phi);
                        y = rr * sinf(phi);
                        weight = 1.f;
                    }
                    if (!guided) {
                        dir = make_float3(m[0] * x + m[1] * y + m[2] * z, m[3] * x + m[4] * y + m[5] * z,
                                          m[6] * x + m[7] * y + m[8] * z);
                    }
                    b_o = make_float4(p2.x, p2.y, p2.z, __uint_as_float(path));
                    b_d = make_float4(dir.x, dir.y, dir.z, __uint_as_float(jidx));
                    b_T = scale4(weight, Td);
                    b_rng = make_uint2(static_cast<uint32_t>(rs), static_cast<uint32_t>(rs >> 32));
                    emit_bounce = bounce;
                    rec_t = luminance(b_T);
                }
            }
        }
        // per-job statistics: this queue entry is one traced ray of job jidx
        // (pathtracer.cpp:21); lanes of the same job add with one atomic
        if (job_counts) {
            const unsigned peers = __match_any_sync(0xFFFFFFFFu, valid ? jidx : 0xFFFFFFFFu);
            const unsigned shadow_peers = __ballot_sync(0xFFFFFFFFu, emit_shadow) & peers;
            if (valid && static_cast<int>(lane_id()) == __ffs(peers) - 1) {
                atomicAdd(job_counts + 2 * jidx, static_cast<unsigned long long>(__popc(peers)));
                if (shadow_peers) atomicAdd(job_counts + 2 * jidx + 1, static_cast<unsigned long long>(__popc(shadow_peers)));
            }
        }
        const uint32_t si = warp_append(sh.count, emit_shadow);
        if (emit_shadow) {
            sh.o[si] = sh_o;
            sh.d[si] = sh_d;
            sh.c[si] = sh_c;
            sh.job[si] = jidx;
            if (sh.aux) sh.aux[si] = kAuxPath;
        }
        uint32_t b_rec = kNoRecord;
        if (recs.count) {
            const uint32_t ri = warp_append(recs.count, emit_record);
            if (emit_record && ri < recs.cap) {
                b_rec = ri;
                const float* f = gq.feat + 9 * size_t(i);
#pragma unroll
                for (int k = 0; k < 9; ++k) recs.feat[9 * size_t(ri) + k] = f[k];
#pragma unroll
                for (int k = 0; k < 3; ++k) recs.dir[3 * size_t(ri) + k] = rec_dir[k];
                recs.path[ri] = rec_path;
                recs.t_after[ri] = rec_t;
                recs.fcos_pdf[ri] = rec_fcp;
                recs.l_before[ri] = 0.f;
            }
        }
        const uint32_t bi = warp_append(out.count, emit_bounce);
        if (emit_bounce) {
            out.o[bi] = b_o;
            out.d[bi] = b_d;
            out.T[bi] = b_T;
            out.rng[bi] = b_rng;
            if (out.rec) out.rec[bi] = b_rec;
        }
        // the branching estimator (pathtracer.cpp:72-88 with M > 1): indirect is
        // the mean over M children, so each carries 1/M of the weight
        const uint32_t bb = warp_append_n(out.count, n_branch);
        if (n_branch) {
            const JobDesc& job = jobs[jidx];
            float m[9];
            from_to_z(br_nrm, m);
            const float inv_m = 1.f / static_cast<float>(n_branch);
            for (uint32_t k = 0; k < n_branch; ++k) {
                uint64_t cs = branch_seed(br_state, k);
                const float u1 = xorshift_float(cs);
                const float u2 = xorshift_float(cs);
                float x, y, z, weight;
                if (job.sampling == 0) {
                    z = u1;
                    const float rr = sqrtf(fmaxf(0.f, 1.f - z * z));
                    const float phi = 6.28318548202514648438f * u2;
                    x = rr * cosf(phi);
                    y = rr * sinf(phi);
                    weight = 2.f * u1;
                } else {
                    const float rr = sqrtf(u1);
                    z = sqrtf(fmaxf(0.f, 1.f - u1));
                    const float phi = 6.28318548202514648438f * u2;
                    x = rr * cosf(phi);
                    y = rr * sinf(phi);
                    weight = 1.f;
                }
                const uint32_t slot = bb + k;
                out.o[slot] = make_float4(br_p2.x, br_p2.y, br_p2.z, __uint_as_float(br_path));
                out.d[slot] = make_float4(m[0] * x + m[1] * y + m[2] * z, m[3] * x + m[4] * y + m[5] * z,
                                          m[6] * x + m[7] * y + m[8] * z, __uint_as_float(jidx));
                out.T[slot] = scale4(weight * inv_m, br_Td);
                out.rng[slot] = make_uint2(static_cast<uint32_t>(cs), static_cast<uint32_t>(cs >> 32));
                if (out.rec) out.rec[slot] = kNoRecord;
            }
        }
    }
}

// The other two trace() plug-ins on the same queues.
//   raycaster.cpp:6-24   hit: the diffuse colour with alpha 1 - r / max_visibility
//                        clamped to [0, 1], counted as a ray; miss: background
//   raytracer.cpp:5-67   every call is a ray (also the mirror call one past max
//                        depth, which returns 0); hit: Lambertian direct light
//                        cos * C * I (lib/lambertian.h:15-19) weighted by 1 -
//                        reflectivity when the triangle reflects, plus a mirror
//                        ray d - 2 (n.d) n with throughput reflectivity *
//                        reflective colour; then a shadow ray toward the light.
// In this forward form the shadow ray of a hit carries the hit's direct
// contribution and the queue slot of its mirror ray: when it is blocked
// (a hit with r < |light - p2|), the shadow kernel adds the contribution
// darkened as c - c * shadow_intensity and darkens the mirror ray's
// throughput the same way (the reference's color -= color * shadow_intensity
// on the whole colour, mirror part included).
__global__ void __launch_bounds__(kBlock) k_shade_classic(const JobDesc* __restrict__ jobs, int depth, RayQueue in,
                                                          const Hit* __restrict__ hits, RayQueue out, ShadowQueue sh,
                                                          float4* __restrict__ L,
                                                          unsigned long long* __restrict__ job_counts) {
    const uint32_t n = *in.count;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); base < n; base += stride) {
        const uint32_t i = base + lane_id();
        bool mine = false, emit_shadow = false, emit_child = false;
        uint32_t jidx = 0, counted = 0;
        float4 sh_o, sh_d, sh_c, c_o, c_d, c_T;
        if (i < n) {
            const float4 d4 = in.d[i];
            jidx = __float_as_uint(d4.w);
            mine = jobs[jidx].renderer != kRendererPath;
            if (mine) {
                const JobDesc& job = jobs[jidx];
                const Hit h = hits[i];
                const float4 o4 = in.o[i];
                const float4 T = in.T[i];
                const uint32_t path = __float_as_uint(o4.w);
                const float4 bg = make_float4(job.bg[0], job.bg[1], job.bg[2], 1.f);
                if (job.renderer == kRendererRaycast) {
                    if (h.id >= kMiss) {
                        L[path] = add4(L[path], mul4(T, bg));
                    } else {
                        counted = 1;
                        const float4* rec = job.sc.shade + 4 * size_t(h.id);
                        const float4 s0 = __ldg(rec), s1 = __ldg(rec + 1), s2 = __ldg(rec + 2);
                        const float a = 1.f - (h.r / job.max_visibility);
                        const float alpha = a < 0.f ? 0.f : (a > 1.f ? 1.f : a);
                        L[path] = add4(L[path], mul4(T, make_float4(s0.w, s1.w, s2.w, alpha)));
                    }
                } else {
                    counted = 1;
                    if (h.id >= kMiss) {
                        L[path] = add4(L[path], mul4(T, bg));
                    } else {
                        const float3 p = make_float3(o4.x + h.r * d4.x, o4.y + h.r * d4.y, o4.z + h.r * d4.z);
                        const float4* rec = job.sc.shade + 4 * size_t(h.id);
                        const float4 s0 = __ldg(rec), s1 = __ldg(rec + 1), s2 = __ldg(rec + 2), s3 = __ldg(rec + 3);
                        const float4 diffuse = make_float4(s0.w, s1.w, s2.w, s3.x);
                        const float rho = s3.y;
                        const float3 nrm = shading_normal(s0, s1, s2, h);
                        const float lx = job.light_pos[0] - p.x, ly = job.light_pos[1] - p.y,
                                    lz = job.light_pos[2] - p.z;
                        const float inv_l = 1 / sqrtf(lx * lx + ly * ly + lz * lz);
                        const float cos_a =
                            fmaxf(0.f, inv_l * lx * nrm.x + inv_l * ly * nrm.y + inv_l * lz * nrm.z);
                        const float4 direct = mul4(scale4(cos_a, diffuse), make_float4(job.light_col[0],
                                                                                       job.light_col[1],
                                                                                       job.light_col[2],
                                                                                       job.light_col[3]));
                        const float3 p2 =
                            make_float3(p.x + nrm.x * 0.0001f, p.y + nrm.y * 0.0001f, p.z + nrm.z * 0.0001f);
                        float4 f = direct;
                        if (rho > 0.f) {
                            f = scale4(1.f - rho, direct);
                            if (depth < job.max_depth) {
                                const float4 rc = job.sc.refl ? __ldg(job.sc.refl + h.id)
                                                              : make_float4(0.f, 0.f, 0.f, 0.f);
                                const float dn = 2.f * (nrm.x * d4.x + nrm.y * d4.y + nrm.z * d4.z);
                                c_o = make_float4(p2.x, p2.y, p2.z, __uint_as_float(path));
                                c_d = make_float4(d4.x - dn * nrm.x, d4.y - dn * nrm.y, d4.z - dn * nrm.z,
                                                  __uint_as_float(jidx));
                                c_T = mul4(T, scale4(rho, rc));
                                emit_child = true;
                            } else {
                                counted = 2;   // trace(depth + 1) is called and returns 0
                            }
                        }
                        const float qx = job.light_pos[0] - p2.x, qy = job.light_pos[1] - p2.y,
                                    qz = job.light_pos[2] - p2.z;
                        const float dist = sqrtf(qx * qx + qy * qy + qz * qz);
                        const float inv_q = 1 / dist;
                        sh_o = make_float4(p2.x, p2.y, p2.z, __uint_as_float(path));
                        // blocked iff some hit has r < dist: the any-hit test keeps r <= tmax
                        sh_d = make_float4(inv_q * qx, inv_q * qy, inv_q * qz, nextafterf(dist, 0.f));
                        sh_c = mul4(T, f);
                        emit_shadow = true;
                    }
                }
            }
        }
        if (job_counts) {
            const unsigned peers = __match_any_sync(0xFFFFFFFFu, mine ? jidx : 0xFFFFFFFFu);
            const unsigned one = __ballot_sync(0xFFFFFFFFu, counted >= 1) & peers;
            const unsigned two = __ballot_sync(0xFFFFFFFFu, counted == 2) & peers;
            const unsigned shadow_peers = __ballot_sync(0xFFFFFFFFu, emit_shadow) & peers;
            if (mine && static_cast<int>(lane_id()) == __ffs(peers) - 1) {
                const unsigned c = __popc(one) + __popc(two);
                if (c) atomicAdd(job_counts + 2 * jidx, static_cast<unsigned long long>(c));
                if (shadow_peers) atomicAdd(job_counts + 2 * jidx + 1, static_cast<unsigned long long>(__popc(shadow_peers)));
            }
        }
        const uint32_t ci = warp_append(out.count, emit_child);
        if (emit_child) {
            out.o[ci] = c_o;
            out.d[ci] = c_d;
            out.T[ci] = c_T;
            out.rng[ci] = make_uint2(1u, 0u);
            if (out.rec) out.rec[ci] = kNoRecord;
        }
        const uint32_t si = warp_append(sh.count, emit_shadow);
        if (emit_shadow) {
            sh.o[si] = sh_o;
            sh.d[si] = sh_d;
            sh.c[si] = sh_c;
            sh.job[si] = jidx;
            sh.aux[si] = emit_child ? ci : kAuxNoChild;
        }
    }
}

// ---------------------------------------------------------------- persistent
// Ray sources for the persistent traversal kernel: where rays come from, which
// scene they are traced in, and where the answer goes.
struct QueueSrc {           // closest hit of a ray queue -> hit array
    const float4* o;
    const float4* d;
    const uint32_t* cnt;
    Hit* hits;
    __device__ uint32_t count() const { return *cnt; }
    __device__ void load(uint32_t i, float3& o3, float3& d3, float& tmax, uint32_t& job) const {
        const float4 a = o[i], b = d[i];
        o3 = make_float3(a.x, a.y, a.z);
        d3 = make_float3(b.x, b.y, b.z);
        tmax = 0.f;
        job = __float_as_uint(b.w);
    }
    __device__ void store(uint32_t i, const Hit& h) const { hits[i] = h; }
};

struct ShadowSrc {          // any hit of a shadow queue -> direct light if unblocked
    const float4* o;
    const float4* d;
    const float4* c;
    const uint32_t* jobs;
    const uint32_t* cnt;
    float4* L;
    bool atomic_l;          // -m > 1 in the batch: several shadow rays of one path per level
    const uint32_t* aux;    // raytracer jobs in the batch (see ShadowQueue::aux), else null
    const JobDesc* table;
    float4* next_T;
    __device__ uint32_t count() const { return *cnt; }
    __device__ void load(uint32_t i, float3& o3, float3& d3, float& tmax, uint32_t& job) const {
        const float4 a = o[i], b = d[i];
        o3 = make_float3(a.x, a.y, a.z);
        d3 = make_float3(b.x, b.y, b.z);
        tmax = b.w;
        job = jobs[i];
    }
    __device__ void add(uint32_t path, float4 ci) const {
        if (atomic_l) {
            atomic_add4(L + path, ci);
        } else {
            const float4 l = L[path];
            L[path] = make_float4(l.x + ci.x, l.y + ci.y, l.z + ci.z, l.w + ci.w);
        }
    }
    __device__ void store(uint32_t i, const Hit& h) const {
        if (h.id >= kMiss) {
            add(__float_as_uint(o[i].w), c[i]);
        } else if (aux) {
            const uint32_t a = aux[i];
            if (a == kAuxPath) return;
            // a raytracer hit in shadow: color -= color * shadow_intensity
            const float si = table[jobs[i]].shadow_intensity;
            const float4 ci = c[i];
            add(__float_as_uint(o[i].w), sub4(ci, scale4(si, ci)));
            if (a != kAuxNoChild) {
                const float4 t = next_T[a];
                next_T[a] = sub4(t, scale4(si, t));
            }
        }
    }
};

struct SoaSrc {             // turner_intersect batches
    const float *ox, *oy, *oz, *dx, *dy, *dz;
    uint32_t n;
    uint32_t* id;
    float *r, *s, *t;
    __device__ uint32_t count() const { return n; }
    __device__ void load(uint32_t i, float3& o3, float3& d3, float& tmax, uint32_t& job) const {
        o3 = make_float3(ox[i], oy[i], oz[i]);
        d3 = make_float3(dx[i], dy[i], dz[i]);
        tmax = 0.f;
        job = 0;
    }
    __device__ void store(uint32_t i, const Hit& h) const {
        const bool hit = h.id < kMiss;
        id[i] = h.id;
        r[i] = hit ? h.r : kFltMax;
        s[i] = hit ? h.s : 0.f;
        t[i] = hit ? h.t : 0.f;
    }
};

struct OccSrc {             // turner_occluded batches: any hit with r <= tmax[i]
    const float *ox, *oy, *oz, *dx, *dy, *dz, *tmax;
    uint32_t n;
    uint8_t* blocked;
    __device__ uint32_t count() const { return n; }
    __device__ void load(uint32_t i, float3& o3, float3& d3, float& tm, uint32_t& job) const {
        o3 = make_float3(ox[i], oy[i], oz[i]);
        d3 = make_float3(dx[i], dy[i], dz[i]);
        tm = tmax[i];
        job = 0;
    }
    __device__ void store(uint32_t i, const Hit& h) const { blocked[i] = h.id < kMiss ? 1 : 0; }
};

// Persistent traversal: each lane holds one ray; lanes whose ray is finished
// take the next unclaimed rays (one atomicAdd per warp), so warps stay full
// while rays of very different lengths are traversed. A warp refills only
// once at least `refill` of its lanes are idle (or none is active): 1 refills
// every round and keeps the most lanes busy; 32 refills whole warps, so
// neighbouring rays of a coherent queue (camera rays) stay together and share
// node and record loads. MULTI: every ray names its job and is traced in
// that job's scene.
template <class Src, bool ANY, bool FAST, bool MULTI, int STACK, bool MAILBOX, bool SPEC = false,
          bool PACKET = false, class Stack>
__device__ __forceinline__ void traverse_persistent(const SceneView& single, const JobDesc* __restrict__ jobs,
                                                    Src& src, uint32_t* __restrict__ work, uint32_t refill,
                                                    Stack& st) {
    const uint32_t n = src.count();
    TravState s;
    uint32_t cur = 0;
    bool active = false, exhausted = false;
    bool fresh = false;   // PACKET: the lane's ray has not been advanced yet
    float tmax = 0.f;
    for (;;) {
        const unsigned idle = __ballot_sync(0xFFFFFFFFu, !active && !exhausted);
        if (idle && (static_cast<uint32_t>(__popc(idle)) >= refill || __ballot_sync(0xFFFFFFFFu, active) == 0)) {
            for (;;) {
                const bool need = !active && !exhausted;
                const unsigned mask = __ballot_sync(0xFFFFFFFFu, need);
                if (mask == 0) break;
                const int leader = __ffs(mask) - 1;
                uint32_t base = 0;
                if (static_cast<int>(lane_id()) == leader) base = atomicAdd(work, static_cast<uint32_t>(__popc(mask)));
                base = __shfl_sync(0xFFFFFFFFu, base, leader);
                if (need) {
                    const uint32_t idx = base + static_cast<uint32_t>(__popc(mask & ((1u << lane_id()) - 1u)));
                    if (idx >= n) {
                        exhausted = true;
                    } else {
                        float3 o, d;
                        uint32_t job;
                        src.load(idx, o, d, tmax, job);
                        const bool in_box = MULTI ? trav_begin(jobs[job].sc, o, d, s) : trav_begin(single, o, d, s);
                        if (in_box) {
                            cur = idx;
                            active = true;
                            fresh = true;
                            st.reset();
                        } else {
                            src.store(idx, s.best);   // misses the scene box
                        }
                    }
                }
            }
        }
        const unsigned act = __ballot_sync(0xFFFFFFFFu, active);
        if (act == 0) break;
        if constexpr (PACKET && !FAST) {
            // a warp of fresh rays with the same direction signs and scene
            // walks the tree as a packet (same answers as the lanes alone)
            if (__ballot_sync(0xFFFFFFFFu, active && fresh) == act && __popc(act) >= 8) {
                const int lead = __ffs(act) - 1;
                const uint32_t neg0 = __shfl_sync(0xFFFFFFFFu, s.neg, lead);
                const unsigned long long n0 =
                    __shfl_sync(0xFFFFFFFFu, reinterpret_cast<unsigned long long>(s.nodes), lead);
                const unsigned long long t0 =
                    __shfl_sync(0xFFFFFFFFu, reinterpret_cast<unsigned long long>(s.tri), lead);
                const bool same = !active || (s.neg == neg0 && reinterpret_cast<unsigned long long>(s.nodes) == n0);
                if (__all_sync(0xFFFFFFFFu, same)) {
                    trav_packet<ANY>(s, active, tmax, neg0, reinterpret_cast<const uint2*>(n0),
                                     reinterpret_cast<const float4*>(t0));
                    if (active) {
                        src.store(cur, s.best);
                        active = false;
                    }
                    continue;
                }
            }
            fresh = false;
        }
        if constexpr (SPEC) {
            // every lane takes part in the speculative round's warp votes
            const bool done = trav_round_spec<ANY, MAILBOX>(s, active, tmax, st);
            if (active && done) {
                src.store(cur, s.best);
                active = false;
            }
        } else if (active && trav_round<ANY, FAST, MAILBOX>(s, tmax, st)) {
            src.store(cur, s.best);
            active = false;
        }
    }
}

// Two kernels over the same body: naming a minimum of one resident block in
// __launch_bounds__ changes ptxas's register budget (61 instead of 56
// registers for the closest-hit kernel, 8 instead of 9 resident blocks), so
// the uncapped kernel gives only the block size.
// RING > 0: the stack's newest RING entries in shared memory (RingStack,
// 8 * RING bytes per thread of dynamic shared memory), else all in local memory.
// RING == -1: the local-memory stack with speculative rounds (trav_round_spec);
// RING == -2: the local-memory stack, warps of coherent fresh rays as packets (trav_packet).
template <class Src, bool ANY, bool FAST, bool MULTI, int BLOCK, int STACK, bool MAILBOX, int RING>
__device__ __forceinline__ void traverse_body(const SceneView& single, const JobDesc* __restrict__ jobs, Src& src,
                                              uint32_t* __restrict__ work, uint32_t refill) {
    if constexpr (RING == -2) {
        LocalStack<STACK> st;
        traverse_persistent<Src, ANY, FAST, MULTI, STACK, MAILBOX, false, true>(single, jobs, src, work, refill, st);
    } else if constexpr (RING < 0) {
        LocalStack<STACK> st;
        traverse_persistent<Src, ANY, FAST, MULTI, STACK, MAILBOX, true>(single, jobs, src, work, refill, st);
    } else if constexpr (RING > 0) {
        RingStack<RING, BLOCK, STACK> st;
        st.init();
        traverse_persistent<Src, ANY, FAST, MULTI, STACK, MAILBOX>(single, jobs, src, work, refill, st);
    } else {
        LocalStack<STACK> st;
        traverse_persistent<Src, ANY, FAST, MULTI, STACK, MAILBOX>(single, jobs, src, work, refill, st);
    }
}

template <class Src, bool ANY, bool FAST, bool MULTI, int BLOCK, int STACK, bool MAILBOX, int RING>
__global__ void __launch_bounds__(BLOCK) k_traverse(SceneView single, const JobDesc* __restrict__ jobs, Src src,
                                                     uint32_t* __restrict__ work, uint32_t refill) {
    traverse_body<Src, ANY, FAST, MULTI, BLOCK, STACK, MAILBOX, RING>(single, jobs, src, work, refill);
}

template <class Src, bool ANY, bool FAST, bool MULTI, int BLOCK, int STACK, bool MAILBOX, int MINB, int RING>
__global__ void __launch_bounds__(BLOCK, MINB) k_traverse_capped(SceneView single, const JobDesc* __restrict__ jobs,
                                                                  Src src, uint32_t* __restrict__ work,
                                                                  uint32_t refill) {
    traverse_body<Src, ANY, FAST, MULTI, BLOCK, STACK, MAILBOX, RING>(single, jobs, src, work, refill);
}

// Per-pixel mean in sample order, exposure (1 - exp(-x e)) and gamma (x^g)
// on RGB; alpha is kept (lib/effects.h:15-49).
__global__ void __launch_bounds__(kBlock) k_resolve(const JobDesc* __restrict__ jobs, uint32_t n_jobs, Chunk c,
                                                    const float4* __restrict__ L) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n_pixels) return;
    const uint64_t gp = c.pixel0 + i;
    const uint32_t j = job_of_pixel(jobs, n_jobs, gp);
    const JobDesc& job = jobs[j];
    const uint64_t local = gp - job.pixel_offset;
    const float4* l = L + (job.path_offset + local * job.spp - c.path0);
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    for (uint32_t k = 0; k < job.spp; ++k) acc = add4(acc, l[k]);
    const float fs = static_cast<float>(job.spp);
    acc = make_float4(acc.x / fs, acc.y / fs, acc.z / fs, acc.w / fs);
    if (job.tone_map) {
        acc.x = 1 - expf(-acc.x * job.exposure);
        acc.y = 1 - expf(-acc.y * job.exposure);
        acc.z = 1 - expf(-acc.z * job.exposure);
        if (job.gamma) {
            acc.x = powf(acc.x, job.inv_gamma);
            acc.y = powf(acc.y, job.inv_gamma);
            acc.z = powf(acc.z, job.inv_gamma);
        }
    }
    job.out[local] = acc;
}

// FP64 running sums of linear radiance for converged reference images.
__global__ void __launch_bounds__(kBlock) k_accumulate(const JobDesc* __restrict__ jobs, uint32_t n_jobs, Chunk c,
                                                       const float4* __restrict__ L, double4* __restrict__ acc) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n_pixels) return;
    const uint64_t gp = c.pixel0 + i;
    const uint32_t j = job_of_pixel(jobs, n_jobs, gp);
    const JobDesc& job = jobs[j];
    const uint64_t local = gp - job.pixel_offset;
    const float4* l = L + (job.path_offset + local * job.spp - c.path0);
    double4 a = acc[gp];
    for (uint32_t k = 0; k < job.spp; ++k) {
        const float4 v = l[k];
        a.x += v.x;
        a.y += v.y;
        a.z += v.z;
        a.w += v.w;
    }
    acc[gp] = a;
}

inline unsigned grid_for(uint64_t n) { return static_cast<unsigned>((n + kBlock - 1) / kBlock); }

// Resident blocks per SM x SMs for a persistent kernel (cached per kernel).
template <int BLOCK, class K> unsigned persistent_grid(K kernel, unsigned blocks_per_sm_cap, size_t dyn_smem = 0) {
    // resident blocks per SM, per kernel (kernels that share a signature
    // differ in registers) and per device
    static std::mutex mu;
    static std::map<std::pair<const void*, int>, std::pair<int, int>> cache;   // -> (SMs, blocks per SM)
    int dev = 0;
    cudaGetDevice(&dev);
    std::pair<int, int> v;
    {
        std::lock_guard<std::mutex> lock(mu);
        const auto key = std::make_pair(reinterpret_cast<const void*>(kernel), dev);
        auto it = cache.find(key);
        if (it == cache.end()) {
            int sms = 0, per_sm = 0;
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, BLOCK, dyn_smem);
            it = cache.emplace(key, std::make_pair(std::max(1, sms), std::max(1, per_sm))).first;
        }
        v = it->second;
    }
    const unsigned per = blocks_per_sm_cap ? std::min<unsigned>(v.second, blocks_per_sm_cap) : v.second;
    return static_cast<unsigned>(v.first) * per;
}

template <class Src, bool ANY, bool FAST, bool MULTI, int BLOCK, int STACK, bool MAILBOX, int MINB, int RING = 0>
void run_traverse_shape(const SceneView& single, const JobDesc* jobs, const Src& src, uint32_t capacity,
                        const TraverseCfg& cfg, cudaStream_t stream) {
    void (*kernel)(SceneView, const JobDesc*, Src, uint32_t*, uint32_t);
    if constexpr (MINB > 1) kernel = k_traverse_capped<Src, ANY, FAST, MULTI, BLOCK, STACK, MAILBOX, MINB, RING>;
    else kernel = k_traverse<Src, ANY, FAST, MULTI, BLOCK, STACK, MAILBOX, RING>;
    const size_t smem = RING > 0 ? size_t(RING) * 2 * sizeof(uint32_t) * BLOCK : 0;
    const unsigned need = static_cast<unsigned>((uint64_t(capacity) + BLOCK - 1) / BLOCK);
    const unsigned grid = std::min(persistent_grid<BLOCK>(kernel, cfg.blocks_per_sm, smem), std::max(1u, need));
    kernel<<<grid, BLOCK, smem, stream>>>(single, jobs, src, cfg.work, std::max(1u, std::min(32u, cfg.refill)));
}

// Dispatch on the tuned block size and stack depth. The stack must hold the
// scene's traversal depth (checked on upload against the largest, 128); the
// batch planner only selects 64 when every scene fits.
template <class Src, bool ANY, bool FAST, bool MULTI>
void run_traverse(const SceneView& single, const JobDesc* jobs, const Src& src, uint32_t capacity,
                  const TraverseCfg& cfg, cudaStream_t stream) {
    const bool small_stack = cfg.stack == 64;
    if (cfg.block == 256) {
        if (small_stack) {
            run_traverse_shape<Src, ANY, FAST, MULTI, 256, 64, false, 1>(single, jobs, src, capacity, cfg, stream);
        } else {
            run_traverse_shape<Src, ANY, FAST, MULTI, 256, kStackCap, false, 1>(single, jobs, src, capacity, cfg,
                                                                                stream);
        }
        return;
    }
    // 128-thread blocks: mailbox on/off x register cap for 10, 12 or 16 resident blocks (or none)
#define TURNER_SHAPE(ST, MB, MINB) \
    run_traverse_shape<Src, ANY, FAST, MULTI, 128, ST, MB, MINB>(single, jobs, src, capacity, cfg, stream)
#define TURNER_CAPS(ST, MB)                               \
    switch (cfg.min_blocks) {                             \
    case 10: TURNER_SHAPE(ST, MB, 10); break;             \
    case 12: TURNER_SHAPE(ST, MB, 12); break;             \
    case 16: TURNER_SHAPE(ST, MB, 16); break;             \
    default: TURNER_SHAPE(ST, MB, 1); break;              \
    }
    if (cfg.packet && !FAST && !cfg.mailbox && cfg.min_blocks == 10 && !cfg.speculative && !cfg.ring) {
        // warps of coherent fresh rays traverse as packets
        run_traverse_shape<Src, ANY, FAST, MULTI, 128, kStackCap, false, 10, -2>(single, jobs, src, capacity, cfg,
                                                                                 stream);
        return;
    }
    if (cfg.speculative && !FAST && !cfg.mailbox && cfg.min_blocks == 10) {
        // speculative rounds (not with FAST's early stop)
        run_traverse_shape<Src, ANY, FAST, MULTI, 128, kStackCap, false, 10, -1>(single, jobs, src, capacity, cfg,
                                                                                 stream);
        return;
    }
    if (cfg.ring && !cfg.mailbox && cfg.min_blocks == 10) {
        // the stack's newest 4 or 8 entries in shared memory
        if (cfg.ring == 4) run_traverse_shape<Src, ANY, FAST, MULTI, 128, kStackCap, false, 10, 4>(single, jobs, src,
                                                                                                 capacity, cfg, stream);
        else run_traverse_shape<Src, ANY, FAST, MULTI, 128, kStackCap, false, 10, 8>(single, jobs, src, capacity, cfg,
                                                                                     stream);
        return;
    }
    if (small_stack) {
        if (cfg.mailbox) { TURNER_CAPS(64, true) } else { TURNER_CAPS(64, false) }
    } else {
        if (cfg.mailbox) { TURNER_CAPS(kStackCap, true) } else { TURNER_CAPS(kStackCap, false) }
    }
#undef TURNER_CAPS
#undef TURNER_SHAPE
}

// One thread per queue slot (the non-persistent launch shape).
template <bool FAST>
__global__ void __launch_bounds__(kBlock) k_trace_flat(SceneView single, const JobDesc* __restrict__ jobs, bool multi,
                                                       RayQueue q, Hit* __restrict__ hits) {
    const uint32_t n = *q.count;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 o = q.o[i];
        const float4 d = q.d[i];
        const SceneView& sc = multi ? jobs[__float_as_uint(d.w)].sc : single;
        hits[i] = traverse<false, FAST>(sc, make_float3(o.x, o.y, o.z), make_float3(d.x, d.y, d.z), 0.f);
    }
}

__global__ void __launch_bounds__(kBlock) k_shadow_flat(SceneView single, const JobDesc* __restrict__ jobs, bool multi,
                                                        ShadowSrc src) {
    const uint32_t n = src.count();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 o = src.o[i];
        const float4 d = src.d[i];
        const SceneView& sc = multi ? jobs[src.jobs[i]].sc : single;
        src.store(i, traverse<true, false>(sc, make_float3(o.x, o.y, o.z), make_float3(d.x, d.y, d.z), d.w));
    }
}

// Gather-bandwidth probe: every thread makes `loads` independent loads of
// BYTES (8: one kd-tree node word; 32: one half of a triangle record, the
// traversal's 256-bit load) at pseudo-random positions in a buffer of
// n_units such units (a power of two), so nearly every load misses L1 and is
// served by L2 when the buffer fits there. Eight loads are in flight per
// thread, as in a warp of independent rays; the XOR of what was read is
// stored so that no load is removed.
template <int BYTES>
__global__ void __launch_bounds__(256) k_gather_probe(const float4* __restrict__ buf, uint32_t mask, uint32_t loads,
                                                      uint32_t seed, uint32_t* __restrict__ out) {
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t x[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) x[j] = static_cast<uint32_t>(splitmix64(uint64_t(tid) * 8 + j + (uint64_t(seed) << 40)));
    uint32_t acc = 0;
    for (uint32_t k = 0; k < loads; k += 8) {
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const uint32_t u = x[j] & mask;
            if (BYTES == 8) {
                const uint2 w = __ldg(reinterpret_cast<const uint2*>(buf) + u);
                acc ^= w.x ^ w.y;
            } else {
                float4 a, b;
                ldg_pair(buf + 2 * size_t(u), a, b);
                acc ^= __float_as_uint(a.x) ^ __float_as_uint(a.w) ^ __float_as_uint(b.y) ^ __float_as_uint(b.z);
            }
            x[j] = x[j] * 1664525u + 1013904223u;
        }
    }
    out[tid] = acc;
}

} // namespace

void launch_gather_probe(const void* buf, uint64_t buf_bytes, int load_bytes, uint32_t loads_per_thread,
                         uint32_t seed, uint32_t* out, unsigned blocks, cudaStream_t stream) {
    const uint32_t mask = static_cast<uint32_t>(buf_bytes / static_cast<uint64_t>(load_bytes) - 1);
    const float4* b = static_cast<const float4*>(buf);
    if (load_bytes == 8) k_gather_probe<8><<<blocks, 256, 0, stream>>>(b, mask, loads_per_thread, seed, out);
    else k_gather_probe<32><<<blocks, 256, 0, stream>>>(b, mask, loads_per_thread, seed, out);
}

void launch_intersect(const SceneView& sc, const float* ox, const float* oy, const float* oz, const float* dx,
                      const float* dy, const float* dz, uint64_t n, uint32_t* id, float* r, float* s, float* t,
                      int fast, const TraverseCfg& cfg, cudaStream_t stream) {
    if (n == 0) return;
    if (cfg.persistent && n < (1ull << 31)) {
        const SoaSrc src{ox, oy, oz, dx, dy, dz, static_cast<uint32_t>(n), id, r, s, t};
        if (fast) run_traverse<SoaSrc, false, true, false>(sc, nullptr, src, static_cast<uint32_t>(n), cfg, stream);
        else run_traverse<SoaSrc, false, false, false>(sc, nullptr, src, static_cast<uint32_t>(n), cfg, stream);
        return;
    }
    k_intersect<<<grid_for(n), kBlock, 0, stream>>>(sc, ox, oy, oz, dx, dy, dz, n, id, r, s, t, fast);
}

void launch_occluded(const SceneView& sc, const float* ox, const float* oy, const float* oz, const float* dx,
                     const float* dy, const float* dz, const float* tmax, uint32_t n, uint8_t* blocked,
                     const TraverseCfg& cfg, cudaStream_t stream) {
    if (n == 0) return;
    // the shadow kernels' default shape: persistent 128-thread blocks, registers capped for 10 per SM
    const OccSrc src{ox, oy, oz, dx, dy, dz, tmax, n, blocked};
    run_traverse_shape<OccSrc, true, false, false, 128, kStackCap, false, 10>(sc, nullptr, src, n, cfg, stream);
}

void launch_camera(const JobDesc* jobs, uint32_t n_jobs, const Chunk& c, const RayQueue& q, float4* L,
                   cudaStream_t stream) {
    k_camera<<<grid_for(c.n_paths), kBlock, 0, stream>>>(jobs, n_jobs, c, q, L);
}

void launch_trace(const SceneView* single, const JobDesc* jobs, const RayQueue& q, Hit* hits, uint32_t capacity,
                  int fast, const TraverseCfg& cfg, cudaStream_t stream) {
    const SceneView sv = single ? *single : SceneView{};
    if (cfg.persistent) {
        const QueueSrc src{q.o, q.d, q.count, hits};
        if (single) {
            if (fast) run_traverse<QueueSrc, false, true, false>(sv, jobs, src, capacity, cfg, stream);
            else run_traverse<QueueSrc, false, false, false>(sv, jobs, src, capacity, cfg, stream);
        } else {
            if (fast) run_traverse<QueueSrc, false, true, true>(sv, jobs, src, capacity, cfg, stream);
            else run_traverse<QueueSrc, false, false, true>(sv, jobs, src, capacity, cfg, stream);
        }
        return;
    }
    if (fast) k_trace_flat<true><<<grid_for(capacity), kBlock, 0, stream>>>(sv, jobs, single == nullptr, q, hits);
    else k_trace_flat<false><<<grid_for(capacity), kBlock, 0, stream>>>(sv, jobs, single == nullptr, q, hits);
}

void launch_shade(const JobDesc* jobs, int depth, const RayQueue& in, const Hit* hits, const RayQueue& out,
                  const ShadowQueue& sh, float4* L, unsigned long long* job_counts, const GuideQueue& gq,
                  const Records& recs, uint32_t capacity, bool mixed, cudaStream_t stream) {
    k_shade<<<grid_for(capacity), kBlock, 0, stream>>>(jobs, depth, in, hits, out, sh, L, job_counts, gq, recs,
                                                       mixed);
}

void launch_shade_classic(const JobDesc* jobs, int depth, const RayQueue& in, const Hit* hits, const RayQueue& out,
                          const ShadowQueue& sh, float4* L, unsigned long long* job_counts, uint32_t capacity,
                          cudaStream_t stream) {
    k_shade_classic<<<grid_for(capacity), kBlock, 0, stream>>>(jobs, depth, in, hits, out, sh, L, job_counts);
}

void launch_guide_features(const JobDesc* jobs, int depth, const RayQueue& q, const Hit* hits, float* feat,
                           uint32_t capacity, cudaStream_t stream) {
    k_guide_features<<<grid_for(capacity), kBlock, 0, stream>>>(jobs, depth, q, hits, feat);
}

void launch_shadow(const SceneView* single, const JobDesc* jobs, const ShadowQueue& sh, float4* L, uint32_t capacity,
                   bool atomic_l, float4* next_T, const TraverseCfg& cfg, cudaStream_t stream) {
    const SceneView sv = single ? *single : SceneView{};
    const ShadowSrc src{sh.o, sh.d, sh.c, sh.job, sh.count, L, atomic_l, sh.aux, jobs, next_T};
    if (cfg.persistent) {
        if (single) run_traverse<ShadowSrc, true, false, false>(sv, jobs, src, capacity, cfg, stream);
        else run_traverse<ShadowSrc, true, false, true>(sv, jobs, src, capacity, cfg, stream);
        return;
    }
    k_shadow_flat<<<grid_for(capacity), kBlock, 0, stream>>>(sv, jobs, single == nullptr, src);
}

void launch_resolve(const JobDesc* jobs, uint32_t n_jobs, const Chunk& c, const float4* L, cudaStream_t stream) {
    k_resolve<<<grid_for(c.n_pixels), kBlock, 0, stream>>>(jobs, n_jobs, c, L);
}

void launch_accumulate(const JobDesc* jobs, uint32_t n_jobs, const Chunk& c, const float4* L, double4* acc,
                       cudaStream_t stream) {
    k_accumulate<<<grid_for(c.n_pixels), kBlock, 0, stream>>>(jobs, n_jobs, c, L, acc);
}

} // namespace turner
