// Learned bounce proposal: the MLP's forward, backward and Adam kernels.
//
// Forward (k_mlp_forward): one persistent CTA per SM, six warpgroups, each
// an independent pipeline over tiles of 128 samples (one thread per sample)
// that shares the CTA's packed weights. The encoded inputs and every hidden
// activation stay in the group's shared-memory buffer as BF16 in the
// core-matrix K-major layout (tc.cuh), updated in place, with a column of
// ones that multiplies the bias column of the weights; the group's thread 0
// issues tcgen05.mma (M = 128, N = 64 or 48, K = 80 in steps of 16) into the
// group's 64 TMEM columns and waits for the commit, and each thread reads its
// row back with tcgen05.ld, applies ReLU with the BF16 conversion and writes
// the next layer's operand with 16-byte stores.
//
// Backward (k_mlp_backward): per tile, the vMF-mixture head gradient of the
// loss -c log q(w) (one thread per sample; the variance objective reweights
// it), then per layer from the top, on
// the tensor cores: dX = dY W (a second BF16 copy of the weights,
// transposed), masked by ReLU', and [dW, db] += dY^T [X, 1] accumulated in
// TMEM over all of a CTA's tiles. Each CTA adds its gradient to the global one
// once; in a training step the last CTA applies Adam and repacks the BF16
// weights.
//
// Every mbarrier wait is bounded; a timeout sets *err and the kernel drains
// its outstanding MMA (bounded), frees its TMEM and returns.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include <cuda_bf16.h>

#include "guide.cuh"
#include "kernels.h"
#include "tc.cuh"
#include "turner_gpu.h"

namespace turner {
namespace guide {


struct Weights {
    const uint8_t* fwd;      // packed BF16 forward operands (kFwdBytes)
    const uint8_t* bwd;      // packed BF16 transposed operands (kBwdBytes)
    const float* params;     // FP32 master (biases are read from here)
};

__device__ __forceinline__ void store_bf16(uint8_t* base, uint32_t off, float v) {
    *reinterpret_cast<__nv_bfloat16*>(base + off) = __float2bfloat16_rn(v);
}

// Issues the K / 16 MMAs of one layer and commits them to `mbar` (thread 0).
__device__ __forceinline__ void issue_layer(uint32_t tmem, const uint8_t* a, const uint8_t* b, int K, int N,
                                            uint64_t* mbar) {
    const uint32_t sa = tc::smem_u32(a), sb = tc::smem_u32(b);
    const uint32_t sbo = static_cast<uint32_t>(K / 8) * 128u;
    const uint32_t idesc = tc::idesc_bf16(128, static_cast<uint32_t>(N));
    for (int i = 0; i < K / 16; ++i) {
        const uint64_t ad = tc::smem_desc(sa + 256u * i, 128u, sbo);
        const uint64_t bd = tc::smem_desc(sb + 256u * i, 128u, sbo);
        tc::mma_bf16(tmem, ad, bd, idesc, i > 0);
    }
    tc::mma_commit(mbar);
}

// ---------------------------------------------------------------- forward
// One persistent CTA per SM runs kFwdGroups independent tile pipelines, one
// per warpgroup: the warpgroup's thread t owns row t of its 128-sample tile,
// its own activation buffer, 64 TMEM columns and mbarrier, and syncs on its
// own named barrier, so that one group's MMAs run while the others' epilogues
// (TMEM read-back, bias, ReLU, BF16 packing) do. The packed weights are
// loaded once per SM and shared by the groups.
constexpr int kFwdGroups = 6;
constexpr int kFwdThreads = 128 * kFwdGroups;
constexpr uint32_t kFwdTmemCols = 512;   // kFwdGroups x 64 columns, allocated as a power of two
static_assert(kFwdGroups * 64 <= static_cast<int>(kFwdTmemCols), "TMEM columns");

struct FwdSmem {
    uint8_t act[kFwdGroups][kFwdK * 128 * 2];   // per group: 128 x 80 inputs, then each layer's [128 x 64 output, 1, 0...] in place
    uint8_t w[kFwdBytes];
    uint64_t mbar[kFwdGroups];
    uint32_t tmem;
};

// Barrier `id` over the 128 threads of one warpgroup; returns whether any of
// them passed a non-zero `pred`.
__device__ __forceinline__ int group_sync_or(int id, int pred) {
    int r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\t"
        "setp.ne.s32 p, %1, 0;\n\t"
        "barrier.cta.red.or.pred q, %2, 128, p;\n\t"
        "selp.s32 %0, 1, 0, q;\n\t}\n"
        : "=r"(r)
        : "r"(pred), "r"(id)
        : "memory");
    return r;
}

__device__ __forceinline__ uint32_t pack_bf16x2(float a, float b) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const uint32_t*>(&h);
}

// Two FP32 values as BF16 (round to nearest even), max(x, 0) applied:
// lo in the low half, hi in the high half.
__device__ __forceinline__ uint32_t pack_bf16x2_relu(float lo, float hi) {
    uint32_t r;
    asm("cvt.rn.relu.bf16x2.f32 %0, %1, %2;\n" : "=r"(r) : "f"(hi), "f"(lo));
    return r;
}

// The 24 encoded inputs of one coordinate (see encode()): (sin, cos) of
// pi 2^i x for i = 0..11, as three groups of eight BF16. One sincospif, then
// the double-angle identities sin 2a = 2 sin a cos a, cos 2a = (cos a - sin a)
// (cos a + sin a): eleven doublings grow the FP32 error to about 2^11 times
// sincospif's (2e-4 at the highest frequency, emulated in FP32), a tenth of
// the BF16 rounding of the stored value (2^-9 relative).
__device__ __forceinline__ void encode_axis(float x, uint4 out[3]) {
    float sn, cs;
    sincospif(x, &sn, &cs);
#pragma unroll
    for (int g = 0; g < 3; ++g) {
        uint32_t w[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            w[j] = pack_bf16x2(sn, cs);
            const float s2 = 2.f * sn * cs;
            cs = (cs - sn) * (cs + sn);
            sn = s2;
        }
        out[g] = make_uint4(w[0], w[1], w[2], w[3]);
    }
}

// features: n x 9 floats (position in [0,1]^3, shading normal, albedo).
// out: n x 40 FP32 head values (may be null). acts (training): n x 336 BF16,
// the layer inputs X_0 (80) .. X_4 (64 each) per sample.
// n_dev (optional): the sample count is read from device memory (a queue
// length), capped at n.
//
// Group g of CTA b takes tiles b * kFwdGroups + g, then every gridDim.x *
// kFwdGroups-th. Every shared-memory write is one 16-byte store of 8 BF16
// values of the thread's row. A layer's output overwrites its input in
// place: the MMAs have read it once their commit has arrived.
__global__ void __launch_bounds__(kFwdThreads, 1) k_mlp_forward(
    uint32_t n, const uint32_t* __restrict__ n_dev, const float* __restrict__ features, Weights wts,
    float* __restrict__ out, __nv_bfloat16* __restrict__ acts, int* err) {
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    FwdSmem& sm = *reinterpret_cast<FwdSmem*>(smem_raw);
    const int tid = threadIdx.x, warp = tid >> 5;
    const int grp = tid >> 7;
    const uint32_t row = static_cast<uint32_t>(tid & 127);
    if (n_dev) n = min(n, *n_dev);
    for (int i = tid; i < kFwdBytes / 16; i += kFwdThreads) {
        reinterpret_cast<uint4*>(sm.w)[i] = reinterpret_cast<const uint4*>(wts.fwd)[i];
    }
    if (tid < kFwdGroups) {
        tc::mbar_init(&sm.mbar[tid], 1);
        tc::fence_mbar_init();
    }
    if (warp == 0) tc::tmem_alloc(&sm.tmem, kFwdTmemCols);
    tc::fence_async_smem();
    tc::tc_fence_before_sync();
    __syncthreads();
    tc::tc_fence_after_sync();
    // this group's accumulator: TMEM lanes 0-127 (warp w of the group reads
    // lanes 32w..32w+31), columns 64 grp .. 64 grp + 63
    const uint32_t tmem = sm.tmem + static_cast<uint32_t>(grp * 64) + (static_cast<uint32_t>(warp & 3) * 32u << 16);
    const uint32_t tmem_mma = sm.tmem + static_cast<uint32_t>(grp * 64);
    uint8_t* const act = sm.act[grp];
    uint64_t* const mbar = &sm.mbar[grp];
    const int bar_id = 1 + grp;   // named barrier 0 is __syncthreads'
    uint32_t phase = 0;
    const uint32_t tiles = (n + 127) / 128;
    const uint32_t stride = gridDim.x * kFwdGroups;

    // this row's 9 input floats; the next tile's are loaded while the
    // current tile runs through the layers
    float fin[9];
    auto load_features = [&](uint32_t t) {
        const uint32_t s = t * 128 + row;
        if (t < tiles && s < n) {
            const float* q = features + 9 * size_t(s);
#pragma unroll
            for (int k = 0; k < 9; ++k) fin[k] = q[k];
        }
    };
    const uint32_t first = blockIdx.x * kFwdGroups + static_cast<uint32_t>(grp);
    load_features(first);
    bool aborted = false;   // the same in every thread of the group: set after a group barrier
    for (uint32_t tile = first; tile < tiles && !aborted; tile += stride) {
        const uint32_t s = tile * 128 + row;
        const bool valid = s < n;
        uint4* const act_row = acts && valid ? reinterpret_cast<uint4*>(acts + size_t(s) * 336) : nullptr;
        {
            // groups 0-8: twelve frequencies of x, y, z (three independent
            // chains, unrolled for ILP); group 9: normal, albedo, zero padding
#pragma unroll
            for (int ax = 0; ax < 3; ++ax) {
                uint4 v[3] = {make_uint4(0u, 0u, 0u, 0u), make_uint4(0u, 0u, 0u, 0u), make_uint4(0u, 0u, 0u, 0u)};
                if (valid) encode_axis(ax == 0 ? fin[0] : ax == 1 ? fin[1] : fin[2], v);
#pragma unroll
                for (int j = 0; j < 3; ++j) {
                    *reinterpret_cast<uint4*>(act + tc::kmajor_offset(row, 8 * (3 * ax + j), kFwdK)) = v[j];
                    if (act_row) act_row[3 * ax + j] = v[j];
                }
            }
            // column 78 is the 1 that multiplies layer 1's bias (the stored X_0 keeps 0 there)
            const uint4 v = valid ? make_uint4(pack_bf16x2(fin[3], fin[4]), pack_bf16x2(fin[5], fin[6]),
                                               pack_bf16x2(fin[7], fin[8]), 0u)
                                  : make_uint4(0u, 0u, 0u, 0u);
            *reinterpret_cast<uint4*>(act + tc::kmajor_offset(row, 72, kFwdK)) =
                make_uint4(v.x, v.y, v.z, pack_bf16x2(1.f, 0.f));
            if (act_row) act_row[9] = v;
        }
        load_features(tile + stride);
        tc::fence_async_smem();
        tc::tc_fence_before_sync();
        group_sync_or(bar_id, 0);
        tc::tc_fence_after_sync();

#pragma unroll 1
        for (int l = 0; l < kLayers; ++l) {
            const int N = layer_out_pad(l);
            // one thread issues the layer's MMAs and waits for their commit;
            // the rest of the group waits at the barrier, without polling
            bool done = true;
            if (row == 0) {
                issue_layer(tmem_mma, act, sm.w + fwd_off(l), kFwdK, N, mbar);
                done = tc::mbar_wait(mbar, phase, err);
            }
            phase ^= 1;
            if (group_sync_or(bar_id, done ? 0 : 1)) {
                aborted = true;   // the wait gave up: nothing is read from TMEM
                break;
            }
            tc::tc_fence_after_sync();
            if (l < kLayers - 1) {
                // the MMA has added the bias: ReLU and BF16 packing only
#pragma unroll 1
                for (int c0 = 0; c0 < kHidden; c0 += 32) {
                    float v[32];
                    tc::tmem_ld32(tmem + static_cast<uint32_t>(c0), v);
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        const uint4 u = make_uint4(pack_bf16x2_relu(v[8 * q], v[8 * q + 1]),
                                                   pack_bf16x2_relu(v[8 * q + 2], v[8 * q + 3]),
                                                   pack_bf16x2_relu(v[8 * q + 4], v[8 * q + 5]),
                                                   pack_bf16x2_relu(v[8 * q + 6], v[8 * q + 7]));
                        *reinterpret_cast<uint4*>(act + tc::kmajor_offset(row, c0 + 8 * q, kFwdK)) = u;
                        if (act_row) act_row[10 + 8 * l + c0 / 8 + q] = u;
                    }
                }
                if (l == 0) {
                    // columns 64-79 of the hidden layers' operand: the 1 of the bias, then zeros
                    *reinterpret_cast<uint4*>(act + tc::kmajor_offset(row, 64, kFwdK)) =
                        make_uint4(pack_bf16x2(1.f, 0.f), 0u, 0u, 0u);
                    *reinterpret_cast<uint4*>(act + tc::kmajor_offset(row, 72, kFwdK)) = make_uint4(0u, 0u, 0u, 0u);
                }
            } else {
#pragma unroll 1
                for (int c0 = 0; c0 < kOut; c0 += 16) {
                    float v[16];
                    tc::tmem_ld16(tmem + static_cast<uint32_t>(c0), v);   // columns 40-47 are padding
                    if (out && valid) {
                        float4* o4 = reinterpret_cast<float4*>(out + size_t(s) * kOut + c0);
#pragma unroll
                        for (int q = 0; q < 4; ++q) {
                            if (c0 + 4 * q < kOut) o4[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
                        }
                    }
                }
            }
            tc::fence_async_smem();   // the next layer's MMAs read what this one wrote
            tc::tc_fence_before_sync();
            group_sync_or(bar_id, 0);
            tc::tc_fence_after_sync();
        }
    }
    if (aborted && row == 0) {
        // drain: an MMA may still be in flight; wait once more (bounded)
        tc::mbar_wait(mbar, phase ^ 1, nullptr, 1000000u);
    }
    tc::tc_fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(sm.tmem, kFwdTmemCols);
}

// ---------------------------------------------------------------- backward
// One CTA of 256 threads per SM, tiles of 128 samples. Per tile, the head
// gradient dY_5 of -c log q (threads 0-127, one sample each), then per layer
// from the top, with X_l and dY_l staged row-major in shared memory:
//   dX   = dY W          M = 128 samples, N = 64 inputs, K = outputs (48 / 64)
//   dW' += dY^T [X, 1]   M = 128 (output units in rows 0-63, rows 64-127 zero),
//                        N = inputs + a ones column (the bias gradient) padded
//                        to 80 / 96, K = 128 samples
// both on tcgen05 with BF16 operands in the core-matrix K-major layout. The
// transposed operands dY^T and [X, 1]^T are built in shared memory from the
// row-major staging buffers. dW' stays in TMEM for all of the CTA's tiles
// (480 of the 512 columns: dX 64, then 96 + 4 x 80); at the end each CTA adds
// it to the global gradient once, and with `adam` set the last CTA to finish
// applies the Adam step, repacks the BF16 operand tiles and clears the
// gradient for the next step (no separate Adam or pack launches).
constexpr int kBwdThreads = 256;
constexpr uint32_t kBwdTmemCols = 512;
constexpr int kXRow = 88, kDyRow = 72;   // row strides (elements) of the staging buffers
__host__ __device__ constexpr int dw_n(int l) { return l == 0 ? 96 : 80; }
__host__ __device__ constexpr int dw_col(int l) { return l == 0 ? 64 : 160 + 80 * (l - 1); }
static_assert(dw_col(4) + dw_n(4) <= static_cast<int>(kBwdTmemCols), "TMEM columns");

struct BwdSmem {
    uint8_t wt[kBwdBytes];                 // W_l^T operands, layers 1..4 (B of dX)
    uint8_t dy_km[128 * kHidden * 2];      // dY, K-major 128 x 48 / 64 (A of dX)
    uint8_t dyT[128 * 128 * 2];            // dY^T, K-major 128 x 128 samples, rows 64.. zero (A of dW)
    uint8_t xT[96 * 128 * 2];              // [X, 1]^T, K-major 80 / 96 x 128 samples (B of dW)
    __nv_bfloat16 xrow[2][128 * kXRow];    // X_l, row per sample; the other buffer receives the next X
    __nv_bfloat16 dyrow[128 * kDyRow];     // dY_l, row per sample
    float head_out[128 * kOut];            // the tile's network outputs (arrive with the tile's X_4)
    uint64_t mbar;
    uint32_t tmem;
    int abort;
    int last;
    float loss;
    float wsum;   // sum of the tile weights c' (variance objective)
};

// Per-step training state, resident on the device so that a training step
// needs no host synchronisation: the sample count may come from a device
// counter (the records of a render pass).
struct TrainState {
    uint32_t n;        // samples of this step
    int32_t skip;      // fewer than the step's minimum: no update
    uint32_t step;     // Adam steps taken
    float bc1, bc2;    // bias corrections of this step
    float scale;       // 1 / n (the loss is a mean over samples)
    float loss_mean;   // loss of the last step / n
    uint32_t done;     // backward CTAs finished in this step (the last one updates)
    float wsum;        // variance objective: sum of the step's weights c' (the gradient is divided by it)
};

struct AdamArgs {
    float* params;     // FP32 master
    float* m;
    float* v;
    uint8_t* fwd;      // packed BF16 operands, rewritten after the update
    uint8_t* bwd;
    TrainState* state;
    float lr, b1, b2, eps;
};

// Head gradient of L = -c' log q(w): writes dL/d raw (40), returns L and
// the weight c' used. Objective 0 (KL divergence): c' = c. Objective 1
// (variance of the sampling mixture p = q/2 + max(0, n.w)/(2 pi)): c' =
// c^2 q / (2 p), held constant; with c = F / p the sample's integrand over
// its pdf, -c' d log q is the gradient of F^2 / p, whose expectation is the
// estimator's second moment (Mueller et al., "Neural Importance Sampling",
// 2019, the chi-square divergence, with the cosine half of the mixture).
__device__ __forceinline__ float head_grad(const float raw[kOut], const float dir[3], float c, const float nrm[3],
                                           int objective, float g[kOut], float& c_used) {
    Mixture m;
    decode(raw, m);
    float p[kLobes], q = 0.f;
#pragma unroll
    for (int l = 0; l < kLobes; ++l) {
        p[l] = vmf_pdf(m.mu[l], m.kappa[l], dir);
        q += m.w[l] * p[l];
    }
    q = fmaxf(q, 1e-20f);
    if (objective == kObjectiveVariance) {
        const float cw = fmaxf(nrm[0] * dir[0] + nrm[1] * dir[1] + nrm[2] * dir[2], 0.f);
        const float pm = 0.5f * q + 0.5f * cw * kInvPi;
        c = c * c * (0.5f * q / pm);
    }
    c_used = c;
    const float loss = -c * logf(q);
    const float gq = -c / q;
    float gw[kLobes], wg = 0.f;
#pragma unroll
    for (int l = 0; l < kLobes; ++l) {
        gw[l] = gq * p[l];
        wg += m.w[l] * gw[l];
    }
#pragma unroll
    for (int l = 0; l < kLobes; ++l) {
        const float a = gq * m.w[l] * p[l];   // dL/d log p_l
        const float cosw = m.mu[l][0] * dir[0] + m.mu[l][1] * dir[1] + m.mu[l][2] * dir[2];
        // d log p / d mu = kappa * w ; project onto the tangent of the unit sphere, / |raw|
        float gm[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) gm[k] = a * m.kappa[l] * dir[k];
        const float dot = gm[0] * m.mu[l][0] + gm[1] * m.mu[l][1] + gm[2] * m.mu[l][2];
#pragma unroll
        for (int k = 0; k < 3; ++k) g[5 * l + k] = (gm[k] - dot * m.mu[l][k]) * m.inv_len[l];
        const float k2 = m.kappa[l];
        const float dlogp = 1.f / k2 - 2.f / expm1f(2.f * k2) + (cosw - 1.f);
        g[5 * l + 3] = a * dlogp * m.kexp[l];
        g[5 * l + 4] = m.w[l] * (gw[l] - wg);
    }
    return loss;
}

__device__ __forceinline__ uint32_t bf16_bits(__nv_bfloat16 h) { return static_cast<uint32_t>(__bfloat16_as_ushort(h)); }

// Eight BF16 values p[0], p[stride], ..., p[7 stride] as one 16-byte chunk.
__device__ __forceinline__ uint4 gather8(const __nv_bfloat16* p, int stride) {
    uint32_t w[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) w[i] = bf16_bits(p[(2 * i) * stride]) | (bf16_bits(p[(2 * i + 1) * stride]) << 16);
    return make_uint4(w[0], w[1], w[2], w[3]);
}

__device__ __forceinline__ void cp_async16(void* smem_dst, const void* src, bool valid) {
    // src-size 0 fills the 16 bytes with zeros and reads nothing
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(tc::smem_u32(smem_dst)), "l"(src),
                 "r"(valid ? 16 : 0)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Starts copying X_l of the tile at s0 (336 BF16 activations per sample: X_0
// 80, X_1..X_4 64 each) row-major into `dst`, zeros past n; with the head
// layer's X also the tile's 40 network outputs into head_out. Asynchronous
// (cp.async): the copies land while the current layer computes; every thread
// waits for its own copies (cp_async_wait_all) before the barrier that
// precedes their use.
__device__ __forceinline__ void stage_x_async(BwdSmem& sm, __nv_bfloat16* dst, const __nv_bfloat16* __restrict__ acts,
                                              const float* __restrict__ out, uint32_t n, uint32_t s0, int l) {
    const int chunks = layer_in(l) / 8;
    const int off = l == 0 ? 0 : 80 + 64 * (l - 1);
    for (int i = threadIdx.x; i < 128 * chunks; i += kBwdThreads) {
        const int r = i / chunks, c = i - r * chunks;
        const uint32_t s = s0 + static_cast<uint32_t>(r);
        cp_async16(dst + r * kXRow + 8 * c, s < n ? acts + size_t(s) * 336 + off + 8 * c : acts, s < n);
    }
    if (l == kLayers - 1) {
        for (int i = threadIdx.x; i < 128 * (kOut / 4); i += kBwdThreads) {
            const int r = i / (kOut / 4), c = i - r * (kOut / 4);
            const uint32_t s = s0 + static_cast<uint32_t>(r);
            cp_async16(sm.head_out + r * kOut + 4 * c, s < n ? out + size_t(s) * kOut + 4 * c : out, s < n);
        }
    }
    cp_async_commit();
}

// [X_l, 1]^T (rows: the layer's inputs, then a ones row, then zero rows up to
// dw_n(l)) and dY^T (rows: output units below n_pad, zeros up to 64), both
// K-major over the 128 samples, from the staging buffers.
__device__ __forceinline__ void build_transposes(BwdSmem& sm, const __nv_bfloat16* xrow, int l) {
    const int K = layer_in(l), N = dw_n(l), npad = layer_out_pad(l);
    const uint32_t one2 = 0x3F803F80u;   // two BF16 ones
    for (int c = threadIdx.x; c < N * 16; c += kBwdThreads) {
        const int k = c % N, j = c / N;
        uint4 u = make_uint4(0u, 0u, 0u, 0u);
        if (k < K) u = gather8(xrow + (8 * j) * kXRow + k, kXRow);
        else if (k == K) u = make_uint4(one2, one2, one2, one2);
        *reinterpret_cast<uint4*>(sm.xT + tc::kmajor_offset(static_cast<uint32_t>(k), 8u * j, 128)) = u;
    }
    for (int c = threadIdx.x; c < kHidden * 16; c += kBwdThreads) {
        const int o = c % kHidden, j = c / kHidden;
        uint4 u = make_uint4(0u, 0u, 0u, 0u);
        if (o < npad) u = gather8(sm.dyrow + (8 * j) * kDyRow + o, kDyRow);
        *reinterpret_cast<uint4*>(sm.dyT + tc::kmajor_offset(static_cast<uint32_t>(o), 8u * j, 128)) = u;
    }
}

// D (+)= A * B^T over K / 16 steps of K-major operands with R-row groups of
// K / 8 core matrices (no commit).
__device__ __forceinline__ void issue_steps(uint32_t tmem, const uint8_t* a, const uint8_t* b, int K, int N,
                                            bool accumulate) {
    const uint32_t sa = tc::smem_u32(a), sb = tc::smem_u32(b);
    const uint32_t sbo = static_cast<uint32_t>(K / 8) * 128u;
    const uint32_t idesc = tc::idesc_bf16(128, static_cast<uint32_t>(N));
    for (int i = 0; i < K / 16; ++i) {
        const uint64_t ad = tc::smem_desc(sa + 256u * i, 128u, sbo);
        const uint64_t bd = tc::smem_desc(sb + 256u * i, 128u, sbo);
        tc::mma_bf16(tmem, ad, bd, idesc, accumulate || i > 0);
    }
}

// features/acts/out as produced by k_mlp_forward for the same samples;
// dirs: n x 3 unit directions; weight: n target weights c; feat: the n x 9
// features (their normals enter the variance objective). grad +=
// dLoss/dparams; with do_adam, the last CTA then takes the Adam step (see
// above), on the gradient over n (KL objective) or over the sum of the
// weights c' (variance objective).
__global__ void __launch_bounds__(kBwdThreads, 1) k_mlp_backward(
    uint32_t n, const uint32_t* __restrict__ n_dev, const __nv_bfloat16* __restrict__ acts,
    const float* __restrict__ out, const float* __restrict__ dirs, const float* __restrict__ weight,
    const float* __restrict__ feat, int objective, Weights wts, float* __restrict__ grad,
    float* __restrict__ loss_sum, int* err, AdamArgs adam, int do_adam) {
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    BwdSmem& sm = *reinterpret_cast<BwdSmem*>(smem_raw);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (n_dev) n = min(n, *n_dev);
    for (int i = tid; i < kBwdBytes / 16; i += kBwdThreads) {
        reinterpret_cast<uint4*>(sm.wt)[i] = reinterpret_cast<const uint4*>(wts.bwd)[i];
    }
    // rows 64..127 of dY^T are never written again: zero the whole buffer once
    for (int i = tid; i < static_cast<int>(sizeof(sm.dyT) / 16); i += kBwdThreads) {
        reinterpret_cast<uint4*>(sm.dyT)[i] = make_uint4(0u, 0u, 0u, 0u);
    }
    if (tid == 0) {
        sm.abort = 0;
        sm.last = 0;
        sm.loss = 0.f;
        sm.wsum = 0.f;
        tc::mbar_init(&sm.mbar, 1);
        tc::fence_mbar_init();
    }
    if (warp == 0) tc::tmem_alloc(&sm.tmem, kBwdTmemCols);
    tc::fence_async_smem();
    tc::tc_fence_before_sync();
    __syncthreads();
    tc::tc_fence_after_sync();
    const uint32_t tmem = sm.tmem;
    const uint32_t quad = static_cast<uint32_t>(warp & 3), colh = static_cast<uint32_t>(warp >> 2);
    const uint32_t lane_base = (quad * 32u) << 16;
    uint32_t phase = 0;
    const uint32_t tiles = (n + 127) / 128;
    float my_loss = 0.f, my_w = 0.f;
    bool had_tile = false;

    int cur = 0;   // xrow buffer holding the current X
    if (blockIdx.x < tiles) stage_x_async(sm, sm.xrow[0], acts, out, n, blockIdx.x * 128, kLayers - 1);
    for (uint32_t tile = blockIdx.x; tile < tiles && !sm.abort; tile += gridDim.x) {
        const bool first = !had_tile;
        had_tile = true;
        const uint32_t s0 = tile * 128;
        cp_async_wait_all();   // this tile's X_4 and network outputs
        __syncthreads();
        if (tid < 128) {
            // head: dY of the output layer, 40 columns padded to 48
            const uint32_t s = s0 + static_cast<uint32_t>(tid);
            float g[kOut];
            if (s < n) {
                float raw[kOut];
                const float4* o4 = reinterpret_cast<const float4*>(sm.head_out + tid * kOut);
#pragma unroll
                for (int q = 0; q < kOut / 4; ++q) {
                    const float4 v = o4[q];
                    raw[4 * q] = v.x;
                    raw[4 * q + 1] = v.y;
                    raw[4 * q + 2] = v.z;
                    raw[4 * q + 3] = v.w;
                }
                const float d[3] = {dirs[3 * size_t(s)], dirs[3 * size_t(s) + 1], dirs[3 * size_t(s) + 2]};
                float nrm[3] = {0.f, 0.f, 0.f};
                if (objective == kObjectiveVariance) {
#pragma unroll
                    for (int k = 0; k < 3; ++k) nrm[k] = feat[9 * size_t(s) + 3 + k];
                }
                float cu;
                my_loss += head_grad(raw, d, weight[s], nrm, objective, g, cu);
                my_w += cu;
            } else {
#pragma unroll
                for (int k = 0; k < kOut; ++k) g[k] = 0.f;
            }
#pragma unroll
            for (int q = 0; q < kOutPad / 8; ++q) {
                float y[8];
#pragma unroll
                for (int j = 0; j < 8; ++j) y[j] = 8 * q + j < kOut ? g[8 * q + j] : 0.f;
                const uint4 u = make_uint4(pack_bf16x2(y[0], y[1]), pack_bf16x2(y[2], y[3]), pack_bf16x2(y[4], y[5]),
                                           pack_bf16x2(y[6], y[7]));
                *reinterpret_cast<uint4*>(sm.dyrow + tid * kDyRow + 8 * q) = u;
                *reinterpret_cast<uint4*>(sm.dy_km + tc::kmajor_offset(static_cast<uint32_t>(tid), 8u * q, kOutPad)) = u;
            }
        }
        for (int l = kLayers - 1; l >= 0; --l) {
            // xrow[cur] = X_l, dyrow / dy_km = dY_l
            __syncthreads();
            build_transposes(sm, sm.xrow[cur], l);
            tc::fence_async_smem();
            tc::tc_fence_before_sync();
            __syncthreads();
            tc::tc_fence_after_sync();
            if (tid == 0) {
                // dX = dY W (not needed below the first layer), then dW' += dY^T [X, 1]
                if (l > 0) issue_steps(tmem, sm.dy_km, sm.wt + bwd_off(l), layer_out_pad(l), layer_in(l), false);
                issue_steps(tmem + static_cast<uint32_t>(dw_col(l)), sm.dyT, sm.xT, 128, dw_n(l), !first);
                tc::mma_commit(&sm.mbar);
            }
            // the next X into the other buffer while the products run: this
            // tile's X_{l-1}, or after the first layer the next tile's X_4
            // and network outputs (the other buffer's last reader finished
            // before the barrier above)
            if (l > 0) stage_x_async(sm, sm.xrow[cur ^ 1], acts, out, n, s0, l - 1);
            else if (tile + gridDim.x < tiles) stage_x_async(sm, sm.xrow[cur ^ 1], acts, out, n,
                                                             (tile + gridDim.x) * 128, kLayers - 1);
            if (!tc::mbar_wait(&sm.mbar, phase, err)) sm.abort = 1;
            phase ^= 1;
            tc::tc_fence_after_sync();
            __syncthreads();
            if (sm.abort || l == 0) break;
            // dY of the layer below: dX masked by ReLU' (X_l > 0); warp w reads
            // lanes 32 (w % 4).. (its samples) and columns 32 (w / 4)..
            {
                const int r = static_cast<int>(quad) * 32 + lane;
                const uint32_t c0 = colh * 32u;
                const __nv_bfloat16* xr = sm.xrow[cur];
                float v[32];
                tc::tmem_ld16(tmem + lane_base + c0, v);
                tc::tmem_ld16(tmem + lane_base + c0 + 16u, v + 16);
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const uint4 xv = *reinterpret_cast<const uint4*>(xr + r * kXRow + c0 + 8 * q);
                    const uint32_t xw[4] = {xv.x, xv.y, xv.z, xv.w};
                    float y[8];
#pragma unroll
                    for (int j = 0; j < 8; ++j) {
                        const uint32_t h = (xw[j >> 1] >> (16 * (j & 1))) & 0xFFFFu;   // BF16 bits of X
                        y[j] = __uint_as_float(h << 16) > 0.f ? v[8 * q + j] : 0.f;
                    }
                    const uint4 u = make_uint4(pack_bf16x2(y[0], y[1]), pack_bf16x2(y[2], y[3]),
                                               pack_bf16x2(y[4], y[5]), pack_bf16x2(y[6], y[7]));
                    *reinterpret_cast<uint4*>(sm.dyrow + r * kDyRow + c0 + 8 * q) = u;
                    *reinterpret_cast<uint4*>(sm.dy_km + tc::kmajor_offset(static_cast<uint32_t>(r), c0 + 8u * q,
                                                                           kHidden)) = u;
                }
            }
            cp_async_wait_all();   // X_{l-1} has landed (the barrier at the top of the loop publishes it)
            cur ^= 1;
        }
        cur ^= 1;   // the next tile's X_4 went to the other buffer
    }
    cp_async_wait_all();   // no copy may outlive the kernel (an abort can leave one in flight)
    // loss, and this CTA's dW' out of TMEM into the global gradient
    for (int off = 16; off > 0; off >>= 1) {
        my_loss += __shfl_xor_sync(0xFFFFFFFFu, my_loss, off);
        my_w += __shfl_xor_sync(0xFFFFFFFFu, my_w, off);
    }
    if (lane == 0) {
        atomicAdd(&sm.loss, my_loss);
        atomicAdd(&sm.wsum, my_w);
    }
    if (sm.abort && tid == 0) tc::mbar_wait(&sm.mbar, phase ^ 1, nullptr, 1000000u);
    tc::tc_fence_before_sync();
    __syncthreads();
    tc::tc_fence_after_sync();
    if (had_tile && !sm.abort && quad < 2) {
        const int o = static_cast<int>(quad) * 32 + lane;   // output unit = TMEM lane
#pragma unroll 1
        for (int l = 0; l < kLayers; ++l) {
            const int K = layer_in(l), N = dw_n(l), nout = layer_out(l);
            for (int c = static_cast<int>(colh) * 16; c < N; c += 32) {
                float v[16];
                tc::tmem_ld16(tmem + lane_base + static_cast<uint32_t>(dw_col(l) + c), v);
                if (o < nout) {
#pragma unroll
                    for (int j = 0; j < 16; ++j) {
                        const int k = c + j;
                        if (k < K) atomicAdd(grad + layer_w(l) + o * K + k, v[j]);
                        else if (k == K) atomicAdd(grad + layer_b(l) + o, v[j]);
                    }
                }
            }
        }
    }
    tc::tc_fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, kBwdTmemCols);
    if (tid == 0 && loss_sum) atomicAdd(loss_sum, sm.loss);
    if (!do_adam) return;
    if (tid == 0) atomicAdd(&adam.state->wsum, sm.wsum);
    // the last CTA to finish takes the Adam step on the complete gradient
    __threadfence();
    __syncthreads();
    if (tid == 0) sm.last = atomicAdd(&adam.state->done, 1u) == gridDim.x - 1 ? 1 : 0;
    __syncthreads();
    if (!sm.last) return;
    __threadfence();
    TrainState* st = adam.state;
    if (!st->skip) {
        const float scale = objective == kObjectiveVariance ? 1.f / fmaxf(__ldcg(&st->wsum), 1e-30f) : st->scale;
        const float bc1 = st->bc1, bc2 = st->bc2;
        for (int i = tid; i < kParams; i += kBwdThreads) {
            const float gi = __ldcg(grad + i) * scale;
            const float mi = adam.b1 * adam.m[i] + (1.f - adam.b1) * gi;
            const float vi = adam.b2 * adam.v[i] + (1.f - adam.b2) * gi * gi;
            adam.m[i] = mi;
            adam.v[i] = vi;
            adam.params[i] -= adam.lr * (mi / bc1) / (sqrtf(vi / bc2) + adam.eps);
        }
        if (tid == 0 && loss_sum) st->loss_mean = __ldcg(loss_sum) * scale;
        __syncthreads();
        // BF16 operand tiles from the updated parameters
        for (int l = 0; l < kLayers; ++l) {
            const int K = layer_in(l), nout = layer_out(l), pad = layer_out_pad(l);
            const float* W = adam.params + layer_w(l);
            for (int e = tid; e < pad * kFwdK; e += kBwdThreads) {
                const int r = e / kFwdK, k = e - r * kFwdK;
                store_bf16(adam.fwd + fwd_off(l), tc::kmajor_offset(static_cast<uint32_t>(r), static_cast<uint32_t>(k),
                                                                    static_cast<uint32_t>(kFwdK)),
                           fwd_operand(adam.params, l, r, k));
            }
            if (l == 0) continue;
            for (int e = tid; e < pad * K; e += kBwdThreads) {
                const int r = e / K, k = e - r * K;
                const float w = r < nout ? W[r * K + k] : 0.f;
                store_bf16(adam.bwd + bwd_off(l), tc::kmajor_offset(static_cast<uint32_t>(k), static_cast<uint32_t>(r),
                                                                    static_cast<uint32_t>(pad)), w);
            }
        }
    }
    // a clean gradient for the next step
    for (int i = tid; i < kParams; i += kBwdThreads) grad[i] = 0.f;
    if (tid == 0) {
        if (loss_sum) *loss_sum = 0.f;
        st->done = 0;
    }
}

// ------------------------------------------------------------ Adam + pack
__global__ void k_train_prep(const uint32_t* __restrict__ n_dev, uint32_t n, uint32_t min_n, TrainState* s, float b1,
                             float b2) {
    if (n_dev) n = min(n, *n_dev);
    s->n = n;
    s->skip = n < min_n ? 1 : 0;
    s->done = 0;
    s->wsum = 0.f;
    if (s->skip) return;
    s->step += 1;
    s->bc1 = 1.f - powf(b1, static_cast<float>(s->step));
    s->bc2 = 1.f - powf(b2, static_cast<float>(s->step));
    s->scale = 1.f / static_cast<float>(n);
}

// BF16 operand tiles from the FP32 parameters.
__global__ void k_pack(const float* __restrict__ p, uint8_t* __restrict__ fwd, uint8_t* __restrict__ bwd) {
    const int l = blockIdx.y;
    const int K = layer_in(l), out = layer_out(l), pad = layer_out_pad(l);
    const float* W = p + layer_w(l);
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < pad * kFwdK; e += gridDim.x * blockDim.x) {
        const int r = e / kFwdK, k = e - r * kFwdK;   // forward: row = output, column = input (+ bias)
        store_bf16(fwd + fwd_off(l), tc::kmajor_offset(r, k, kFwdK), fwd_operand(p, l, r, k));
    }
    if (l == 0) return;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < pad * K; e += gridDim.x * blockDim.x) {
        const int r = e / K, k = e - r * K;   // backward: row = input k, column = output r
        const float w = r < out ? W[r * K + k] : 0.f;
        store_bf16(bwd + bwd_off(l), tc::kmajor_offset(k, r, pad), w);
    }
}

size_t fwd_smem() { return sizeof(FwdSmem) + 1024; }
size_t bwd_smem() { return sizeof(BwdSmem) + 1024; }

} // namespace guide
} // namespace turner

// ===================================================================== C ABI
using namespace turner;
using namespace turner::guide;

struct turner_guide {
    turner_ctx* ctx = nullptr;
    int device = 0;
    cudaStream_t stream = nullptr;
    float* params = nullptr;   // FP32 master
    float* m = nullptr;
    float* v = nullptr;
    float* grad = nullptr;
    uint8_t* fwd = nullptr;
    uint8_t* bwd = nullptr;
    float* loss = nullptr;
    int* err = nullptr;
    TrainState* state = nullptr;
    // training-batch scratch, grown on demand
    size_t cap = 0;
    float* feat = nullptr;
    float* dirs = nullptr;
    float* wts = nullptr;
    float* out = nullptr;
    __nv_bfloat16* acts = nullptr;
    bool grad_dirty = false;   // grad / loss hold a turner_guide_gradient result, not zeros
    int objective = kObjectiveKL;   // training objective (turner_guide_set_objective)
    int sms = 1;
    double train_ms = 0, infer_ms = 0;
    uint64_t train_steps = 0;
};

namespace {

int cuda_status(cudaError_t e) {
    return e == cudaSuccess ? TURNER_OK : (e == cudaErrorMemoryAllocation ? TURNER_ERR_OUT_OF_MEMORY : TURNER_ERR_CUDA);
}

#define GCK(call)                                      \
    do {                                               \
        const cudaError_t e_ = (call);                 \
        if (e_ != cudaSuccess) return cuda_status(e_); \
    } while (0)

int ensure_batch(turner_guide* g, size_t n) {
    if (n <= g->cap) return TURNER_OK;
    cudaFree(g->feat);
    cudaFree(g->dirs);
    cudaFree(g->wts);
    cudaFree(g->out);
    cudaFree(g->acts);
    g->feat = g->dirs = g->wts = g->out = nullptr;
    g->acts = nullptr;
    g->cap = 0;
    GCK(cudaMalloc(&g->feat, n * 9 * sizeof(float)));
    GCK(cudaMalloc(&g->dirs, n * 3 * sizeof(float)));
    GCK(cudaMalloc(&g->wts, n * sizeof(float)));
    GCK(cudaMalloc(&g->out, n * kOut * sizeof(float)));
    GCK(cudaMalloc(&g->acts, n * 336 * sizeof(__nv_bfloat16)));
    g->cap = n;
    return TURNER_OK;
}

int check_err(turner_guide* g) {
    int e = 0;
    GCK(cudaMemcpyAsync(&e, g->err, sizeof(int), cudaMemcpyDeviceToHost, g->stream));
    GCK(cudaStreamSynchronize(g->stream));
    if (e) {
        cudaMemsetAsync(g->err, 0, sizeof(int), g->stream);
        return TURNER_ERR_TIMEOUT;
    }
    return TURNER_OK;
}

// One CTA per SM for the backward pass (its shared memory fills an SM).
unsigned grid_tiles(turner_guide* g, uint32_t n) {
    return std::max(1u, std::min<unsigned>(static_cast<unsigned>(g->sms), (n + 127) / 128));
}

// One persistent forward CTA per SM (its groups share the weights).
unsigned grid_tiles_fwd(turner_guide* g, uint32_t n) {
    const unsigned tiles = (n + 127) / 128;
    return std::max(1u, std::min<unsigned>(static_cast<unsigned>(g->sms), (tiles + kFwdGroups - 1) / kFwdGroups));
}

} // namespace

namespace turner {
namespace guide {

// Device-buffer forward for the renderer (features n x 9 -> out n x 40).
int forward_device(turner_guide* g, const float* feat, uint32_t n, float* out, cudaStream_t stream) {
    if (n == 0) return TURNER_OK;
    Weights w{g->fwd, g->bwd, g->params};
    k_mlp_forward<<<grid_tiles_fwd(g, n), kFwdThreads, fwd_smem(), stream>>>(n, nullptr, feat, w, out, nullptr, g->err);
    return cuda_status(cudaGetLastError());
}

// Forward over a ray queue whose length is on the device (at most cap).
int forward_queue(turner_guide* g, const float* feat, const uint32_t* n_dev, uint32_t cap, float* out,
                  cudaStream_t stream) {
    if (cap == 0) return TURNER_OK;
    Weights w{g->fwd, g->bwd, g->params};
    k_mlp_forward<<<grid_tiles_fwd(g, cap), kFwdThreads, fwd_smem(), stream>>>(cap, n_dev, feat, w, out, nullptr, g->err);
    return cuda_status(cudaGetLastError());
}

// Target weights of the recorded bounces: the incident radiance along the
// sampled direction is what the rest of the path added after the bounce,
// divided by the throughput after it: L_in = (L_end - L_before) / T_after;
// weight = L_in * f cos / p (the integrand over the sampling pdf, luminance).
// mode 1 also weighs each record by the path throughput that reached the
// bounce (luminance, t_after / fcos_pdf), so that the shared network spends
// its capacity where the pixels' variance comes from: the weight becomes the
// luminance the path gained after the bounce. Mode 2 weighs by the square
// root of that throughput.
__global__ void k_finalize_records(const uint32_t* __restrict__ count, uint32_t cap, const float4* __restrict__ L,
                                   const uint32_t* __restrict__ path, const float* __restrict__ l_before,
                                   const float* __restrict__ t_after, const float* __restrict__ fcos_pdf,
                                   float* __restrict__ weight, int mode) {
    const uint32_t n = min(*count, cap);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 l = L[path[i]];
        const float lum = 0.2126f * l.x + 0.7152f * l.y + 0.0722f * l.z;
        const float t = t_after[i];
        const float fc = fcos_pdf[i];
        const float gained = fmaxf(lum - l_before[i], 0.f);
        const float lin = t > 0.f ? gained / t : 0.f;
        float w = lin * fc;
        if (mode == 1) w = gained;
        else if (mode == 2) w = fc > 0.f ? w * sqrtf(t / fc) : 0.f;
        weight[i] = fminf(w, 1e4f);
    }
}

int finalize_records(const uint32_t* count, uint32_t cap, const float4* L, const uint32_t* path,
                     const float* l_before, const float* t_after, const float* fcos_pdf, float* weight, int mode,
                     cudaStream_t stream) {
    k_finalize_records<<<(cap + 255) / 256, 256, 0, stream>>>(count, cap, L, path, l_before, t_after, fcos_pdf,
                                                              weight, mode);
    return cuda_status(cudaGetLastError());
}

// One Adam step on n device-resident samples (features n x 9, dirs n x 3,
// weights n); optional loss (mean of -c log q) copied out.
int train_device(turner_guide* g, const float* feat, const float* dirs, const float* wts, uint32_t n,
                 const uint32_t* n_dev, uint32_t min_n, float lr, cudaStream_t stream, float* loss_out) {
    if (n == 0) return TURNER_OK;
    int st = ensure_batch(g, n);
    if (st != TURNER_OK) return st;
    Weights w{g->fwd, g->bwd, g->params};
    const float b1 = 0.9f, b2 = 0.999f;
    if (g->grad_dirty) {
        // the backward's last CTA leaves them zero; only a gradient query does not
        GCK(cudaMemsetAsync(g->grad, 0, kParams * sizeof(float), stream));
        GCK(cudaMemsetAsync(g->loss, 0, sizeof(float), stream));
        g->grad_dirty = false;
    }
    k_train_prep<<<1, 1, 0, stream>>>(n_dev, n, min_n, g->state, b1, b2);
    const uint32_t* n_step = &g->state->n;
    k_mlp_forward<<<grid_tiles_fwd(g, n), kFwdThreads, fwd_smem(), stream>>>(n, n_step, feat, w, g->out, g->acts,
                                                                             g->err);
    const AdamArgs adam{g->params, g->m, g->v, g->fwd, g->bwd, g->state, lr, b1, b2, 1e-8f};
    k_mlp_backward<<<grid_tiles(g, n), kBwdThreads, bwd_smem(), stream>>>(n, n_step, g->acts, g->out, dirs, wts, feat,
                                                                         g->objective, w, g->grad, g->loss, g->err,
                                                                         adam, 1);
    GCK(cudaGetLastError());
    g->train_steps += 1;
    if (loss_out) {
        TrainState s{};
        GCK(cudaMemcpyAsync(&s, g->state, sizeof(s), cudaMemcpyDeviceToHost, stream));
        GCK(cudaStreamSynchronize(stream));
        *loss_out = s.loss_mean;
    }
    return TURNER_OK;
}

turner_ctx* owner(const turner_guide* g) { return g->ctx; }

void orphan(turner_guide* g) {
    g->ctx = nullptr;
    g->stream = nullptr;
}

int train_state(turner_guide* g, uint64_t* steps, float* last_loss) {
    TrainState s{};
    GCK(cudaMemcpyAsync(&s, g->state, sizeof(s), cudaMemcpyDeviceToHost, g->stream));
    GCK(cudaStreamSynchronize(g->stream));
    if (steps) *steps = s.step;
    if (last_loss) *last_loss = s.loss_mean;
    return TURNER_OK;
}

} // namespace guide
} // namespace turner

namespace turner {
cudaStream_t ctx_stream(turner_ctx* ctx);
int ctx_device(turner_ctx* ctx);
void ctx_add_guide(turner_ctx* ctx, turner_guide* g);
void ctx_remove_guide(turner_ctx* ctx, turner_guide* g);
} // namespace turner

extern "C" {

int turner_guide_create(turner_ctx* ctx, uint64_t seed, turner_guide** out) {
    if (!ctx || !out) return TURNER_ERR_INVALID_ARG;
    *out = nullptr;
    auto* g = new (std::nothrow) turner_guide;
    if (!g) return TURNER_ERR_OUT_OF_MEMORY;
    g->ctx = ctx;
    g->device = turner::ctx_device(ctx);
    g->stream = turner::ctx_stream(ctx);
    cudaSetDevice(g->device);
    cudaDeviceGetAttribute(&g->sms, cudaDevAttrMultiProcessorCount, g->device);
    cudaError_t e = cudaSuccess;
    if (e == cudaSuccess) e = cudaMalloc(&g->params, kParams * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&g->m, kParams * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&g->v, kParams * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&g->grad, kParams * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&g->fwd, kFwdBytes);
    if (e == cudaSuccess) e = cudaMalloc(&g->bwd, kBwdBytes);
    if (e == cudaSuccess) e = cudaMalloc(&g->loss, sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&g->err, sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&g->state, sizeof(TrainState));
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_mlp_forward, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                   static_cast<int>(fwd_smem()));
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_mlp_backward, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                   static_cast<int>(bwd_smem()));
    if (e != cudaSuccess) {
        turner_guide_destroy(g);
        return cuda_status(e);
    }
    // He-uniform initialisation (seeded splitmix64 stream), zero biases;
    // lobe directions start spread by the random last layer.
    std::vector<float> p(kParams, 0.f);
    uint64_t s = seed ? seed : 1;
    auto uni = [&s]() {
        s += 0x9E3779B97F4A7C15ULL;
        uint64_t z = s;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
        z ^= z >> 31;
        return static_cast<float>(static_cast<double>(z >> 11) * (1.0 / 9007199254740992.0));
    };
    for (int l = 0; l < kLayers; ++l) {
        const int fan_in = l == 0 ? kInUsed : kHidden;
        const float a = std::sqrt(6.f / static_cast<float>(fan_in));
        for (int r = 0; r < layer_out(l); ++r) {
            for (int k = 0; k < layer_in(l); ++k) {
                const float w = (l == 0 && k >= kInUsed) ? 0.f : (2.f * uni() - 1.f) * a;
                p[layer_w(l) + r * layer_in(l) + k] = w;
            }
        }
    }
    e = cudaMemcpy(g->params, p.data(), kParams * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(g->m, 0, kParams * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(g->v, 0, kParams * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(g->err, 0, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(g->state, 0, sizeof(TrainState));
    if (e == cudaSuccess) e = cudaMemset(g->grad, 0, kParams * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(g->loss, 0, sizeof(float));
    if (e == cudaSuccess) {
        k_pack<<<dim3(16, kLayers), 256, 0, g->stream>>>(g->params, g->fwd, g->bwd);
        e = cudaStreamSynchronize(g->stream);
    }
    if (e != cudaSuccess) {
        turner_guide_destroy(g);
        return cuda_status(e);
    }
    turner::ctx_add_guide(ctx, g);
    *out = g;
    return TURNER_OK;
}

void turner_guide_destroy(turner_guide* g) {
    if (!g) return;
    cudaSetDevice(g->device);
    if (g->ctx) turner::ctx_remove_guide(g->ctx, g);   // unbinds it where it is the context's proposal
    if (g->stream) cudaStreamSynchronize(g->stream);
    else cudaDeviceSynchronize();   // orphaned: the context's stream is gone
    for (void* p : {static_cast<void*>(g->params), static_cast<void*>(g->m), static_cast<void*>(g->v),
                    static_cast<void*>(g->grad), static_cast<void*>(g->fwd), static_cast<void*>(g->bwd),
                    static_cast<void*>(g->loss), static_cast<void*>(g->err), static_cast<void*>(g->feat),
                    static_cast<void*>(g->dirs), static_cast<void*>(g->wts), static_cast<void*>(g->out),
                    static_cast<void*>(g->acts), static_cast<void*>(g->state)}) {
        if (p) cudaFree(p);
    }
    delete g;
}

int turner_guide_params(turner_guide* g, float* host, int set) {
    if (!g || !g->ctx || !host) return TURNER_ERR_INVALID_ARG;
    cudaSetDevice(g->device);
    if (set) {
        GCK(cudaMemcpyAsync(g->params, host, kParams * sizeof(float), cudaMemcpyHostToDevice, g->stream));
        k_pack<<<dim3(16, kLayers), 256, 0, g->stream>>>(g->params, g->fwd, g->bwd);
        GCK(cudaGetLastError());
    } else {
        GCK(cudaMemcpyAsync(host, g->params, kParams * sizeof(float), cudaMemcpyDeviceToHost, g->stream));
    }
    GCK(cudaStreamSynchronize(g->stream));
    return TURNER_OK;
}

int turner_guide_set_objective(turner_guide* g, int objective) {
    if (!g || !g->ctx || (objective != kObjectiveKL && objective != kObjectiveVariance)) return TURNER_ERR_INVALID_ARG;
    g->objective = objective;
    return TURNER_OK;
}

int turner_guide_forward(turner_guide* g, const float* features, uint32_t n, float* out) {
    if (!g || !g->ctx || !features || !out) return TURNER_ERR_INVALID_ARG;
    if (n == 0) return TURNER_OK;
    cudaSetDevice(g->device);
    int st = ensure_batch(g, n);
    if (st != TURNER_OK) return st;
    GCK(cudaMemcpyAsync(g->feat, features, n * 9 * sizeof(float), cudaMemcpyHostToDevice, g->stream));
    st = guide::forward_device(g, g->feat, n, g->out, g->stream);
    if (st != TURNER_OK) return st;
    GCK(cudaMemcpyAsync(out, g->out, n * kOut * sizeof(float), cudaMemcpyDeviceToHost, g->stream));
    GCK(cudaStreamSynchronize(g->stream));
    return check_err(g);
}

int turner_guide_gradient(turner_guide* g, const float* features, const float* dirs, const float* weights, uint32_t n,
                          float* grad_out, float* loss_out) {
    if (!g || !g->ctx || !features || !dirs || !weights || !grad_out || n == 0) return TURNER_ERR_INVALID_ARG;
    cudaSetDevice(g->device);
    int st = ensure_batch(g, n);
    if (st != TURNER_OK) return st;
    GCK(cudaMemcpyAsync(g->feat, features, n * 9 * sizeof(float), cudaMemcpyHostToDevice, g->stream));
    GCK(cudaMemcpyAsync(g->dirs, dirs, n * 3 * sizeof(float), cudaMemcpyHostToDevice, g->stream));
    GCK(cudaMemcpyAsync(g->wts, weights, n * sizeof(float), cudaMemcpyHostToDevice, g->stream));
    GCK(cudaMemsetAsync(g->grad, 0, kParams * sizeof(float), g->stream));
    GCK(cudaMemsetAsync(g->loss, 0, sizeof(float), g->stream));
    g->grad_dirty = true;
    Weights w{g->fwd, g->bwd, g->params};
    k_mlp_forward<<<grid_tiles_fwd(g, n), kFwdThreads, fwd_smem(), g->stream>>>(n, nullptr, g->feat, w, g->out, g->acts, g->err);
    k_mlp_backward<<<grid_tiles(g, n), kBwdThreads, bwd_smem(), g->stream>>>(n, nullptr, g->acts, g->out, g->dirs,
                                                                            g->wts, g->feat, g->objective, w, g->grad,
                                                                            g->loss, g->err, AdamArgs{}, 0);
    GCK(cudaGetLastError());
    GCK(cudaMemcpyAsync(grad_out, g->grad, kParams * sizeof(float), cudaMemcpyDeviceToHost, g->stream));
    float l = 0;
    GCK(cudaMemcpyAsync(&l, g->loss, sizeof(float), cudaMemcpyDeviceToHost, g->stream));
    GCK(cudaStreamSynchronize(g->stream));
    if (loss_out) *loss_out = l;
    return check_err(g);
}

int turner_guide_train(turner_guide* g, const float* features, const float* dirs, const float* weights, uint32_t n,
                       float lr, uint32_t steps, float* loss_out) {
    if (!g || !g->ctx || !features || !dirs || !weights || n == 0) return TURNER_ERR_INVALID_ARG;
    cudaSetDevice(g->device);
    int st = ensure_batch(g, n);
    if (st != TURNER_OK) return st;
    GCK(cudaMemcpyAsync(g->feat, features, n * 9 * sizeof(float), cudaMemcpyHostToDevice, g->stream));
    GCK(cudaMemcpyAsync(g->dirs, dirs, n * 3 * sizeof(float), cudaMemcpyHostToDevice, g->stream));
    GCK(cudaMemcpyAsync(g->wts, weights, n * sizeof(float), cudaMemcpyHostToDevice, g->stream));
    float loss = 0;
    for (uint32_t i = 0; i < steps; ++i) {
        st = guide::train_device(g, g->feat, g->dirs, g->wts, n, nullptr, 1, lr, g->stream,
                                 i + 1 == steps ? &loss : nullptr);
        if (st != TURNER_OK) return st;
    }
    if (loss_out) *loss_out = loss;
    return check_err(g);
}

} // extern "C"
