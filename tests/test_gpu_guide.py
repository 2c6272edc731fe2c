"""The learned proposal's tcgen05 kernels against the FP64 oracle.

Tolerances (BF16 weights and activations, FP32 accumulation on the tensor
cores; the oracle applies the same BF16 roundings in FP64):
  forward   relative Frobenius error of the 40 outputs < 1e-2
  gradient  relative Frobenius error < 3e-2, cosine similarity > 0.999
"""
import numpy as np
import pytest

import turner_gb300 as tg
from oracle import mlp_oracle as mo

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = tg.Context(0)
    yield c
    c.close()


def batch(n, seed):
    rng = np.random.default_rng(seed)
    feat = np.concatenate([rng.uniform(0, 1, (n, 3)), rng.normal(size=(n, 3)), rng.uniform(0, 1, (n, 3))], 1)
    feat[:, 3:6] /= np.linalg.norm(feat[:, 3:6], axis=1, keepdims=True)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    c = rng.uniform(0.1, 2.0, n)
    return feat.astype(np.float32), d.astype(np.float32), c.astype(np.float32)


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


@pytest.mark.parametrize("n", [1, 128, 293, 5000, 100_003])   # the last: several tiles per persistent CTA
def test_forward_matches_oracle(ctx, n):
    g = tg.Guide(ctx, seed=3)
    p = mo.init_params(11).astype(np.float32)
    p[mo.n_params() - 40:] = np.random.default_rng(4).normal(size=40) * 0.1   # non-zero output biases
    g.set_params(p)
    assert np.array_equal(g.get_params(), p)
    feat, _, _ = batch(n, 5)
    out = g.forward(feat)
    ref, _ = mo.forward(p.astype(np.float64), feat.astype(np.float64), use_bf16=True)
    assert np.isfinite(out).all()
    assert rel(out, ref) < 1e-2, rel(out, ref)


@pytest.mark.parametrize("objective", ["kl", "variance"])
def test_gradient_matches_oracle(ctx, objective):
    g = tg.Guide(ctx, seed=3)
    g.set_objective(tg.GUIDE_OBJECTIVE_VARIANCE if objective == "variance" else tg.GUIDE_OBJECTIVE_KL)
    p = mo.init_params(12).astype(np.float32)
    g.set_params(p)
    feat, d, c = batch(700, 6)
    grad, loss = g.gradient(feat, d, c)
    ref = mo.gradient(p.astype(np.float64), feat.astype(np.float64), d.astype(np.float64), c.astype(np.float64),
                      use_bf16=True, objective=objective)
    ref_loss = mo.loss_sum(p.astype(np.float64), feat.astype(np.float64), d.astype(np.float64),
                           c.astype(np.float64), use_bf16=True, objective=objective)
    # the variance weights c' carry q itself (BF16 network against FP64)
    assert abs(loss - ref_loss) < (1e-3 if objective == "kl" else 5e-3) * abs(ref_loss)
    cos = float(grad @ ref / (np.linalg.norm(grad) * np.linalg.norm(ref)))
    assert cos > 0.999 and rel(grad, ref) < 3e-2, (cos, rel(grad, ref))
    # every layer gets a gradient, not only the head
    for (o, i), start in zip(mo.SHAPES, np.cumsum([0] + [o * i + o for o, i in mo.SHAPES[:-1]])):
        assert np.abs(grad[start:start + o * i]).max() > 0


def test_training_fits_a_direction_field(ctx):
    """Targets concentrated around a direction that depends on the position:
    Adam steps on the tensor-core gradient lower the loss a lot."""
    rng = np.random.default_rng(8)
    n = 4096
    feat, _, _ = batch(n, 9)
    axis = np.stack([np.cos(2 * np.pi * feat[:, 0]), np.sin(2 * np.pi * feat[:, 0]), 0.5 + feat[:, 1]], 1)
    axis /= np.linalg.norm(axis, axis=1, keepdims=True)
    d = axis + 0.15 * rng.normal(size=(n, 3))
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    c = np.ones(n, np.float32)
    g = tg.Guide(ctx, seed=21)
    first = g.train(feat, d, c, lr=3e-3, steps=1)
    last = g.train(feat, d, c, lr=3e-3, steps=300)
    assert np.isfinite(last) and last < first - 2.0, (first, last)
    raw = g.forward(feat)
    q = mo.mixture_pdf(raw.astype(np.float64), d.astype(np.float64))
    assert np.median(q) > 5 / (4 * np.pi)   # far above the uniform density


def test_adam_step_fused_into_backward(ctx):
    """One training step: the backward's last CTA applies Adam (first step:
    p -= lr * g / (|g| + eps), i.e. lr times the sign of the mean gradient),
    repacks the BF16 operands (the next forward uses the new weights) and
    leaves a zero gradient for the next step, also after a gradient query."""
    p = mo.init_params(13).astype(np.float32)
    feat, d, c = batch(3000, 14)
    ref = mo.gradient(p.astype(np.float64), feat.astype(np.float64), d.astype(np.float64), c.astype(np.float64),
                      use_bf16=True) / feat.shape[0]
    lr = 1e-3
    a = tg.Guide(ctx, seed=3)
    a.set_params(p)
    a.gradient(feat, d, c)            # leaves its gradient in the device buffer
    a.train(feat, d, c, lr=lr, steps=1)
    pa = a.get_params()
    step = (p - pa) / lr
    big = np.abs(ref) > 1e-5
    assert np.abs(step).max() <= 1.0 + 1e-3
    assert (np.sign(step[big]) == np.sign(ref[big])).mean() > 0.99
    assert (np.abs(step[big]) > 0.9).mean() > 0.99
    # the same step on a guide that never answered a gradient query
    b = tg.Guide(ctx, seed=3)
    b.set_params(p)
    b.train(feat, d, c, lr=lr, steps=1)
    assert np.allclose(b.get_params(), pa, atol=1e-5)
    # the repacked BF16 operands: the forward now computes with the new weights
    out = a.forward(feat[:500])
    want, _ = mo.forward(pa.astype(np.float64), feat[:500].astype(np.float64), use_bf16=True)
    assert rel(out, want) < 1e-2
