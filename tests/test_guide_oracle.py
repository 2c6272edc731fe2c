"""The learned-proposal oracle pinned by central finite differences (FP64)."""
import numpy as np

from oracle import mlp_oracle as mo


def _batch(n, seed):
    rng = np.random.default_rng(seed)
    feat = np.concatenate([rng.uniform(0, 1, (n, 3)), rng.normal(size=(n, 3)), rng.uniform(0, 1, (n, 3))], 1)
    feat[:, 3:6] /= np.linalg.norm(feat[:, 3:6], axis=1, keepdims=True)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    c = rng.uniform(0.1, 2.0, n)
    return feat, d, c


def test_parameter_count():
    assert mo.n_params() == 20264


def test_mixture_is_a_density():
    """q integrates to 1 over the sphere (Monte Carlo with 200k directions)."""
    rng = np.random.default_rng(1)
    p = mo.init_params(3)
    feat, _, _ = _batch(4, 2)
    raw, _ = mo.forward(p, feat)
    d = rng.normal(size=(200_000, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    for i in range(4):
        q = mo.mixture_pdf(np.repeat(raw[i:i + 1], len(d), 0), d)
        assert abs(q.mean() * 4 * np.pi - 1) < 0.03


def test_head_gradient_matches_finite_differences():
    rng = np.random.default_rng(5)
    raw = rng.normal(size=(6, 40)) * 0.7
    feat, d, c = _batch(6, 6)
    g = mo.head_grad(raw, d, c)
    eps = 1e-6
    for i in range(6):
        for k in rng.choice(40, 12, replace=False):
            rp, rm = raw.copy(), raw.copy()
            rp[i, k] += eps
            rm[i, k] -= eps
            lp = -c[i] * np.log(mo.mixture_pdf(rp[i:i + 1], d[i:i + 1]))[0]
            lm = -c[i] * np.log(mo.mixture_pdf(rm[i:i + 1], d[i:i + 1]))[0]
            fd = (lp - lm) / (2 * eps)
            assert abs(fd - g[i, k]) <= 1e-5 * max(1.0, abs(fd)), (i, k, fd, g[i, k])


def test_network_gradient_matches_finite_differences():
    p = mo.init_params(7) + np.random.default_rng(8).normal(size=mo.n_params()) * 0.01
    feat, d, c = _batch(16, 9)
    g = mo.gradient(p, feat, d, c)
    rng = np.random.default_rng(10)
    eps = 1e-6
    for k in rng.choice(mo.n_params(), 60, replace=False):
        pp, pm = p.copy(), p.copy()
        pp[k] += eps
        pm[k] -= eps
        fd = (mo.loss_sum(pp, feat, d, c) - mo.loss_sum(pm, feat, d, c)) / (2 * eps)
        assert abs(fd - g[k]) <= 1e-4 * max(1.0, abs(fd)), (k, fd, g[k])


def test_variance_gradient_matches_finite_differences():
    """The variance objective's per-sample weights c' = c^2 q / (2 p) make
    -c' d log q the gradient of sum c^2 p0 / p, the mixture estimator's second
    moment over samples drawn from p0, at p = p0."""
    p = mo.init_params(17) + np.random.default_rng(18).normal(size=mo.n_params()) * 0.01
    feat, d, c = _batch(16, 19)
    p0 = mo.sampling_pdf(p, feat, d)
    g = mo.gradient(p, feat, d, c, objective="variance")
    rng = np.random.default_rng(20)
    eps = 1e-6
    for k in rng.choice(mo.n_params(), 60, replace=False):
        pp, pm = p.copy(), p.copy()
        pp[k] += eps
        pm[k] -= eps
        fd = (mo.variance_objective(pp, feat, d, c, p0) - mo.variance_objective(pm, feat, d, c, p0)) / (2 * eps)
        assert abs(fd - g[k]) <= 1e-4 * max(1.0, abs(fd)), (k, fd, g[k])


def test_bf16_rounding():
    x = np.array([1.0, 1.00390625, 1.005859375, -3.3e-5, 65504.0])
    r = mo.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0  # 1 + 2^-8 ties to even
    assert r[2] == 1.0078125
    assert abs(r[3] + 3.3e-5) < 3.3e-5 * 2 ** -7
