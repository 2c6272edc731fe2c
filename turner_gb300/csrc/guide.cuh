// Learned bounce proposal: network shape, input encoding and the
// von Mises-Fisher mixture head, shared by the MLP kernels (guide.cu) and the
// shading kernel that samples from it (trace_kernels.cu).
//
// Network (no counterpart in the reference, whose bounces are uniform on the
// hemisphere, lib/sampling.h:20-32):
//   input  78 = 12-frequency sin/cos of the position normalised to the scene
//          box (3 x 12 x 2 = 72) + shading normal (3) + albedo (3), padded to 80
//   hidden 4 x 64, ReLU, BF16 weights, FP32 accumulation
//   output 40 = 8 lobes x (direction 3, log concentration 1, weight logit 1)
// Proposal pdf mixed with cosine sampling at weight 1/2, so it stays positive
// on the hemisphere: p(w) = 0.5 q(w) + 0.5 max(0, n.w) / pi.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace turner {
namespace guide {

constexpr int kIn = 80, kInUsed = 78, kHidden = 64, kOut = 40, kOutPad = 48, kLobes = 8, kFreqs = 12;
constexpr int kLayers = 5;

// Parameter layout (FP32 master copy): W_l [out x in] row-major, then b_l.
constexpr int kW1 = 0, kB1 = kW1 + kHidden * kIn;
constexpr int kW2 = kB1 + kHidden, kB2 = kW2 + kHidden * kHidden;
constexpr int kW3 = kB2 + kHidden, kB3 = kW3 + kHidden * kHidden;
constexpr int kW4 = kB3 + kHidden, kB4 = kW4 + kHidden * kHidden;
constexpr int kW5 = kB4 + kHidden, kB5 = kW5 + kOut * kHidden;
constexpr int kParams = kB5 + kOut;   // 20,264

__host__ __device__ constexpr int layer_in(int l) { return l == 0 ? kIn : kHidden; }
__host__ __device__ constexpr int layer_out(int l) { return l == 4 ? kOut : kHidden; }
__host__ __device__ constexpr int layer_out_pad(int l) { return l == 4 ? kOutPad : kHidden; }
__host__ __device__ constexpr int layer_w(int l) { return l == 0 ? kW1 : l == 1 ? kW2 : l == 2 ? kW3 : l == 3 ? kW4 : kW5; }
__host__ __device__ constexpr int layer_b(int l) { return l == 0 ? kB1 : l == 1 ? kB2 : l == 2 ? kB3 : l == 3 ? kB4 : kB5; }

// Packed BF16 operand tiles (core-matrix K-major, see tc.cuh), in bytes:
//   forward  [W_l | b_l] as [out_pad x 80]  (B operand of [X, 1] * [W, b]^T):
//            the bias sits in column fwd_bias_col(l) (layer 1: column 78,
//            the first padding column of the encoded input; the others:
//            column 64, after the 64 hidden inputs), where the forward's
//            operand A holds 1; the other columns past the inputs are zero
//   backward W_l^T as [in x out_pad]        (B operand of dY * W), layers 2-5 only
constexpr int kFwdK = 80;
__host__ __device__ constexpr int fwd_bias_col(int l) { return l == 0 ? kInUsed : kHidden; }
__host__ __device__ constexpr int fwd_bytes(int l) { return layer_out_pad(l) * kFwdK * 2; }
__host__ __device__ constexpr int fwd_off(int l) {
    return l == 0 ? 0 : fwd_off(l - 1) + fwd_bytes(l - 1);
}
constexpr int kFwdBytes = fwd_off(kLayers);                      // 48,640
// Element (r, k) of layer l's forward operand from the FP32 parameters.
__host__ __device__ inline float fwd_operand(const float* params, int l, int r, int k) {
    if (r >= layer_out(l)) return 0.f;
    if (k == fwd_bias_col(l)) return params[layer_b(l) + r];
    return k < layer_in(l) ? params[layer_w(l) + r * layer_in(l) + k] : 0.f;
}
__host__ __device__ constexpr int bwd_bytes(int l) { return l == 0 ? 0 : layer_in(l) * layer_out_pad(l) * 2; }
__host__ __device__ constexpr int bwd_off(int l) {
    return l == 0 ? 0 : bwd_off(l - 1) + bwd_bytes(l - 1);
}
constexpr int kBwdBytes = bwd_off(kLayers);                      // 30,720

// 72 Fourier features of a position in [0, 1]^3, then normal and albedo.
__device__ __forceinline__ void encode(const float p[3], const float n[3], const float a[3], float f[kIn]) {
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
#pragma unroll
        for (int i = 0; i < kFreqs; ++i) {
            float s, c;
            sincospif(p[ax] * static_cast<float>(1 << i), &s, &c);
            f[ax * 2 * kFreqs + 2 * i] = s;
            f[ax * 2 * kFreqs + 2 * i + 1] = c;
        }
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        f[72 + k] = n[k];
        f[75 + k] = a[k];
    }
    f[78] = 0.f;
    f[79] = 0.f;
}

struct Mixture {
    float mu[kLobes][3];
    float kappa[kLobes];
    float w[kLobes];
    float inv_len[kLobes];   // 1 / |raw direction|, for the gradient
    float kexp[kLobes];      // d kappa / d raw (0 where the raw value is clamped)
};

constexpr float kKappaRawMin = -3.f, kKappaRawMax = 5.f, kKappaFloor = 1e-3f;
constexpr float kInvTwoPi = 0.159154943091895335769f;
constexpr float kInvPi = 0.318309886183790671538f;
// training objectives of the proposal (turner_guide_set_objective)
constexpr int kObjectiveKL = 0, kObjectiveVariance = 1;

__device__ __forceinline__ void decode(const float raw[kOut], Mixture& m) {
    float mx = -1e30f;
#pragma unroll
    for (int l = 0; l < kLobes; ++l) mx = fmaxf(mx, raw[5 * l + 4]);
    float sum = 0.f;
#pragma unroll
    for (int l = 0; l < kLobes; ++l) {
        const float x = raw[5 * l], y = raw[5 * l + 1], z = raw[5 * l + 2];
        const float len = fmaxf(sqrtf(x * x + y * y + z * z), 1e-6f);
        m.inv_len[l] = 1.f / len;
        m.mu[l][0] = x * m.inv_len[l];
        m.mu[l][1] = y * m.inv_len[l];
        m.mu[l][2] = z * m.inv_len[l];
        const float kr = raw[5 * l + 3];
        const float krc = fminf(fmaxf(kr, kKappaRawMin), kKappaRawMax);
        const float e = __expf(krc);
        m.kappa[l] = e + kKappaFloor;
        m.kexp[l] = (kr > kKappaRawMin && kr < kKappaRawMax) ? e : 0.f;
        m.w[l] = __expf(raw[5 * l + 4] - mx);
        sum += m.w[l];
    }
    const float inv = 1.f / sum;
#pragma unroll
    for (int l = 0; l < kLobes; ++l) m.w[l] *= inv;
}

// vMF density on the sphere: kappa / (2 pi (1 - e^{-2 kappa})) e^{kappa (mu.w - 1)}
__device__ __forceinline__ float vmf_pdf(const float mu[3], float kappa, const float w[3]) {
    const float c = mu[0] * w[0] + mu[1] * w[1] + mu[2] * w[2];
    return kappa * kInvTwoPi / (-expm1f(-2.f * kappa)) * __expf(kappa * (c - 1.f));
}

__device__ __forceinline__ float mixture_pdf(const Mixture& m, const float w[3]) {
    float q = 0.f;
#pragma unroll
    for (int l = 0; l < kLobes; ++l) q += m.w[l] * vmf_pdf(m.mu[l], m.kappa[l], w);
    return q;
}

// Sample lobe l's vMF (Jakob, "Numerically stable sampling of the von
// Mises-Fisher distribution on S^2", 2012) in the frame of its mean.
__device__ __forceinline__ void vmf_sample(const float mu[3], float kappa, float u1, float u2, const float rot[9],
                                           float out[3]) {
    const float W = 1.f + logf(u1 + (1.f - u1) * __expf(-2.f * kappa)) / kappa;
    const float W2 = fminf(1.f, W * W);
    const float r = sqrtf(1.f - W2);
    float s, c;
    sincospif(2.f * u2, &s, &c);
    const float x = r * c, y = r * s, z = W;
    out[0] = rot[0] * x + rot[1] * y + rot[2] * z;
    out[1] = rot[3] * x + rot[4] * y + rot[5] * z;
    out[2] = rot[6] * x + rot[7] * y + rot[8] * z;
    (void)mu;
}

} // namespace guide
} // namespace turner
