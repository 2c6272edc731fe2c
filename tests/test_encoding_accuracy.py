"""The forward kernel encodes each coordinate with one sincospi and eleven
double-angle steps (guide.cu encode_axis). Emulated in FP32 here: the error
against the exact features grows about twofold per step to 2e-4 at the
highest frequency, a tenth of the BF16 rounding (2^-9 relative) the encoded
values then get."""
import numpy as np


def doubling_chain(x: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """(sin, cos) of pi 2^i x for i = 0..11, FP32 like the kernel."""
    sn = np.sin(np.pi * x.astype(np.float64)).astype(np.float32)   # sincospif: correctly rounded here
    cs = np.cos(np.pi * x.astype(np.float64)).astype(np.float32)
    out_s, out_c = [], []
    two = np.float32(2.0)
    for _ in range(12):
        out_s.append(sn)
        out_c.append(cs)
        s2 = two * sn * cs
        cs = (cs - sn) * (cs + sn)
        sn = s2
    return np.stack(out_s, 1), np.stack(out_c, 1)


def test_eleven_doublings_stay_far_below_bf16_rounding():
    rng = np.random.default_rng(3)
    x = np.concatenate([rng.uniform(0, 1, 200_000), np.linspace(0, 1, 4097)]).astype(np.float32)
    s, c = doubling_chain(x)
    k = (2.0 ** np.arange(12))[None, :]
    a = np.pi * x.astype(np.float64)[:, None] * k
    err = np.maximum(np.abs(s - np.sin(a)), np.abs(c - np.cos(a)))
    assert err.max() < 2.5e-4, err.max()
    assert err.max() < 2.0 ** -9 / 8   # an eighth of the BF16 rounding step near 1
    # the error grows about twofold per doubling, as the bound says
    per_level = err.max(axis=0)
    assert per_level[-1] < 2.0 ** 11 * max(per_level[0], 2.0 ** -24) * 2
