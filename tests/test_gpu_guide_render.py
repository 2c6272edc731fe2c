"""Rendering with the learned proposal: unbiased, trained online by the
renderer, and better than the method without it.

Small indirect-lit room (walls tessellated 64x64, baffle under the light),
128x128, depth 5, linear output, against an FP64-accumulated cosine render of
4096 samples per pixel."""
import numpy as np
import pytest

import turner_gb300 as tg

pytestmark = pytest.mark.gpu
SIDE, DEPTH = 128, 5


@pytest.fixture(scope="module")
def setup():
    ctx = tg.Context(0)
    mesh = tg.make_scene(tg.SCENE_BAFFLE_ROOM, detail=64)
    sid = ctx.upload_tree(tg.KDTree.from_mesh(mesh))

    def job(sampling, spp, seed):
        j = tg.make_job(sid, mesh, SIDE, SIDE, pixel_samples=spp, max_depth=DEPTH, seed=seed, sampling=sampling)
        j.linear_output = 1
        return j

    ref, n = ctx.accumulate(job(tg.SAMPLING_COSINE, 256, 4242), 16)
    assert n == 4096
    yield ctx, job, ref
    ctx.set_guide(None)
    ctx.close()


def mse(img, ref):
    return float(((img[..., :3] - ref[..., :3]) ** 2).mean())


def test_guided_sampling_requires_a_guide(setup):
    ctx, job, _ = setup
    ctx.set_guide(None)
    with pytest.raises(tg.TurnerError):
        ctx.render([job(tg.SAMPLING_GUIDED, 1, 1)])


def test_guide_and_context_destroy_in_either_order(setup):
    """Destroying a bound proposal unbinds it; a proposal whose context was
    destroyed first refuses every call but its own destroy; a proposal is
    bound only to the context that created it."""
    ctx, job, _ = setup
    g = tg.Guide(ctx, seed=5)
    ctx.set_guide(g, train=False)
    ctx.render([job(tg.SAMPLING_GUIDED, 1, 1)])
    g.close()
    with pytest.raises(tg.TurnerError) as e:   # no proposal bound any more
        ctx.render([job(tg.SAMPLING_GUIDED, 1, 1)])
    assert e.value.status == tg.ERR_INVALID_ARG
    other = tg.Context(0)
    g2 = tg.Guide(other, seed=6)
    with pytest.raises(tg.TurnerError) as e:
        ctx.set_guide(g2)
    assert e.value.status == tg.ERR_INVALID_ARG
    other.set_guide(g2, train=False)
    params = g2.get_params()
    other.close()
    with pytest.raises(tg.TurnerError) as e:
        g2.get_params()
    assert e.value.status == tg.ERR_INVALID_ARG
    with pytest.raises(tg.TurnerError):
        g2.set_params(params)
    g2.close()


def test_untrained_proposal_is_unbiased(setup):
    """Any network output keeps the estimator unbiased (cosine floor weight 1/2)."""
    ctx, job, ref = setup
    g = tg.Guide(ctx, seed=3)
    ctx.set_guide(g, train=False)
    img, n = ctx.accumulate(job(tg.SAMPLING_GUIDED, 256, 77), 4)
    assert n == 1024
    rel = abs(img[..., :3].mean() - ref[..., :3].mean()) / ref[..., :3].mean()
    assert rel < 5e-3, rel
    ctx.set_guide(None)


def test_online_training_beats_cosine_sampling(setup):
    """The renderer trains the network on its own bounces (Adam, lr 1e-3,
    2^18 records per pass); afterwards the learned proposal has lower error
    than cosine sampling at the same number of samples, and stays unbiased."""
    ctx, job, ref = setup
    g = tg.Guide(ctx, seed=7)
    ctx.set_guide(g, train=True, lr=1e-3, records=1 << 18)
    ctx.set_chunk_paths(1 << 17)
    try:
        for it in range(60):
            ctx.render([job(tg.SAMPLING_GUIDED, 16, 1000 + it)])
        steps, loss, train_ms = ctx.guide_stats()
        assert steps >= 100 and np.isfinite(loss) and train_ms > 0
    finally:
        ctx.set_chunk_paths(1 << 24)
    ctx.set_guide(g, train=False)
    errs_g, errs_c = [], []
    for seed in (5, 6, 7):
        (gi,), _ = ctx.render([job(tg.SAMPLING_GUIDED, 16, seed)])
        (ci,), _ = ctx.render([job(tg.SAMPLING_COSINE, 16, seed)])
        errs_g.append(mse(gi, ref))
        errs_c.append(mse(ci, ref))
    assert np.mean(errs_g) < 0.95 * np.mean(errs_c), (errs_g, errs_c)
    img, _ = ctx.accumulate(job(tg.SAMPLING_GUIDED, 256, 91), 4)
    rel = abs(img[..., :3].mean() - ref[..., :3].mean()) / ref[..., :3].mean()
    assert rel < 5e-3, rel
    ctx.set_guide(None)
