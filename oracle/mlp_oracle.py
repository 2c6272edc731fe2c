"""ORACLE — test infrastructure only: FP64 reference of the learned bounce
proposal (network in turner_gb300/csrc/guide.cuh, kernels in guide.cu).

The reference renderer has no learned proposal (its bounces are uniform on
the hemisphere, lib/sampling.h:20-32), so this oracle is pinned by central
finite differences of its own loss (tests/test_guide_oracle.py) and checked
against the GPU kernels (tests/test_gpu_guide.py).

  input   12-frequency sin/cos of the position in [0,1]^3 (72), normal (3),
          albedo (3), zero padding (2)
  hidden  4 x 64 ReLU;  output 40 = 8 lobes x (direction, log kappa, logit)
  head    q(w) = sum_l softmax(logit)_l vMF(w; mu_l, kappa_l),
          mu_l = d_l / |d_l|, kappa_l = exp(clip(r_l, -3, 5)) + 1e-3
  loss    mean over samples of -c_i log q(w_i) (objective "kl"); objective
          "variance": -c'_i log q(w_i) with c' = c^2 q / (2 p) held constant,
          p = q/2 + max(0, n.w)/(2 pi) the sampling mixture and n the normal
          of the features: the gradient of sum c^2 p0 / p(params) at p0 = p,
          the second moment of the mixture estimator (variance_objective)
With bf16=True the GPU's roundings are applied: weights, biases, the encoded
input and hidden activations to BF16; every layer's output gradient dY to BF16,
as it enters the tensor-core products dY W, dY^T X and the bias sums.
"""
from __future__ import annotations

import numpy as np

IN, IN_USED, H, OUT, LOBES, FREQS = 80, 78, 64, 40, 8, 12
SHAPES = [(H, IN), (H, H), (H, H), (H, H), (OUT, H)]


def n_params() -> int:
    return sum(o * i + o for o, i in SHAPES)


def unpack(p: np.ndarray):
    """[(W, b)] per layer from the flat layout W1 b1 W2 b2 ... W5 b5."""
    out, k = [], 0
    for o, i in SHAPES:
        W = p[k:k + o * i].reshape(o, i)
        k += o * i
        b = p[k:k + o]
        k += o
        out.append((W, b))
    return out


def bf16(x: np.ndarray) -> np.ndarray:
    """Round to the nearest BF16 (ties to even) and back, as __float2bfloat16_rn."""
    f = np.asarray(x, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def encode(feat: np.ndarray) -> np.ndarray:
    """feat: (n, 9) = position in [0,1]^3, normal, albedo -> (n, 80)."""
    n = feat.shape[0]
    f = np.zeros((n, IN))
    for ax in range(3):
        for i in range(FREQS):
            a = np.pi * feat[:, ax] * (1 << i)
            f[:, ax * 2 * FREQS + 2 * i] = np.sin(a)
            f[:, ax * 2 * FREQS + 2 * i + 1] = np.cos(a)
    f[:, 72:75] = feat[:, 3:6]
    f[:, 75:78] = feat[:, 6:9]
    return f


def forward(p: np.ndarray, feat: np.ndarray, use_bf16: bool = False):
    """Returns (raw outputs (n, 40), list of layer inputs X_0..X_4)."""
    layers = unpack(np.asarray(p, np.float64))
    x = encode(np.asarray(feat, np.float64))
    if use_bf16:
        x = bf16(x)
    xs = []
    for l, (W, b) in enumerate(layers):
        xs.append(x)
        Wq = bf16(W) if use_bf16 else W
        y = x @ Wq.T + (bf16(b) if use_bf16 else b)   # the GPU's MMA adds the bias as a BF16 weight
        if l < 4:
            x = np.maximum(y, 0.0)
            if use_bf16:
                x = bf16(x)
        else:
            x = y
    return x, xs


def decode(raw: np.ndarray):
    d = raw.reshape(-1, LOBES, 5)
    vec = d[:, :, 0:3]
    length = np.maximum(np.linalg.norm(vec, axis=-1), 1e-6)
    mu = vec / length[..., None]
    kr = d[:, :, 3]
    krc = np.clip(kr, -3.0, 5.0)
    kappa = np.exp(krc) + 1e-3
    kexp = np.where((kr > -3.0) & (kr < 5.0), np.exp(krc), 0.0)
    logits = d[:, :, 4]
    e = np.exp(logits - logits.max(axis=1, keepdims=True))
    w = e / e.sum(axis=1, keepdims=True)
    return mu, kappa, w, length, kexp


def vmf_pdf(mu, kappa, dirs):
    c = np.einsum("nlk,nk->nl", mu, dirs)
    return kappa / (2 * np.pi * (-np.expm1(-2 * kappa))) * np.exp(kappa * (c - 1))


def mixture_pdf(raw: np.ndarray, dirs: np.ndarray) -> np.ndarray:
    mu, kappa, w, _, _ = decode(raw)
    return (w * vmf_pdf(mu, kappa, dirs)).sum(axis=1)


def variance_weights(raw, feat, dirs, c) -> np.ndarray:
    """c' = c^2 q / (2 p), p = q/2 + max(0, n.w)/(2 pi) (guide.cu head_grad)."""
    q = np.maximum(mixture_pdf(raw, dirs), 1e-20)
    cw = np.maximum((np.asarray(feat, np.float64)[:, 3:6] * dirs).sum(axis=1), 0.0)
    pm = 0.5 * q + 0.5 * cw / np.pi
    return c * c * (0.5 * q / pm)


def sampling_pdf(p, feat, dirs, use_bf16=False) -> np.ndarray:
    """The mixture p = q/2 + max(0, n.w)/(2 pi) the renderer samples."""
    raw, _ = forward(p, feat, use_bf16)
    q = np.maximum(mixture_pdf(raw, dirs), 1e-20)
    cw = np.maximum((np.asarray(feat, np.float64)[:, 3:6] * dirs).sum(axis=1), 0.0)
    return 0.5 * q + 0.5 * cw / np.pi


def variance_objective(p, feat, dirs, c, p0) -> float:
    """sum c^2 p0 / p(params): with c = F / p0 the estimator's second moment
    over samples drawn from p0; its gradient at p = p0 is the variance
    objective's gradient."""
    return float(np.sum(c * c * p0 / sampling_pdf(p, feat, dirs)))


def loss_sum(p, feat, dirs, c, use_bf16=False, objective="kl") -> float:
    raw, _ = forward(p, feat, use_bf16)
    q = np.maximum(mixture_pdf(raw, dirs), 1e-20)
    if objective == "variance":
        c = variance_weights(raw, feat, dirs, c)
    return float(np.sum(-c * np.log(q)))


def head_grad(raw: np.ndarray, dirs: np.ndarray, c: np.ndarray) -> np.ndarray:
    """d(sum -c log q)/d raw, (n, 40)."""
    mu, kappa, w, length, kexp = decode(raw)
    p = vmf_pdf(mu, kappa, dirs)
    q = np.maximum((w * p).sum(axis=1), 1e-20)
    gq = -c / q
    gw = gq[:, None] * p
    wg = (w * gw).sum(axis=1, keepdims=True)
    a = gq[:, None] * w * p
    cosw = np.einsum("nlk,nk->nl", mu, dirs)
    gm = (a * kappa)[..., None] * dirs[:, None, :]
    dot = (gm * mu).sum(-1, keepdims=True)
    gdir = (gm - dot * mu) / length[..., None]
    dlogp = 1 / kappa - 2 / np.expm1(2 * kappa) + (cosw - 1)
    gk = a * dlogp * kexp
    glog = w * (gw - wg)
    g = np.concatenate([gdir, gk[..., None], glog[..., None]], axis=-1)
    return g.reshape(-1, OUT)


def gradient(p, feat, dirs, c, use_bf16=False, objective="kl") -> np.ndarray:
    """Analytic d(sum_i -c_i log q_i)/d params, same layout as the params
    (objective "variance": with the weights c' of variance_weights)."""
    p = np.asarray(p, np.float64)
    raw, xs = forward(p, feat, use_bf16)
    layers = unpack(p)
    dirs = np.asarray(dirs, np.float64)
    c = np.asarray(c, np.float64)
    if objective == "variance":
        c = variance_weights(raw, feat, dirs, c)
    dy = head_grad(raw, dirs, c)
    grads = [None] * 5
    for l in range(4, -1, -1):
        W, _ = layers[l]
        x = xs[l]
        dyq = bf16(dy) if use_bf16 else dy
        grads[l] = (dyq.T @ x, dyq.sum(axis=0))
        if l == 0:
            break
        Wq = bf16(W) if use_bf16 else W
        dx = dyq @ Wq
        dy = dx * (x > 0)
    return np.concatenate([np.concatenate([gW.ravel(), gb]) for gW, gb in grads])


def init_params(seed: int) -> np.ndarray:
    """He-uniform weights, zero biases (the GPU uses its own seeded stream)."""
    rng = np.random.default_rng(seed)
    out = []
    for l, (o, i) in enumerate(SHAPES):
        a = np.sqrt(6.0 / (IN_USED if l == 0 else H))
        W = rng.uniform(-a, a, (o, i))
        if l == 0:
            W[:, IN_USED:] = 0
        out += [W.ravel(), np.zeros(o)]
    return np.concatenate(out)
