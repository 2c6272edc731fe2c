"""Batches of uneven jobs in one launch sequence, FP64 accumulation, linear output.

A job's pixels depend only on its own (pixel, sample) streams, so a job
rendered inside a batch of other scenes, sizes, sample counts and depths must
come out bit-identical to the same job rendered alone."""
import numpy as np
import pytest

import turner_gb300 as tg
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = tg.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def scenes(ctx):
    out = {}
    for name, kw in {"room": dict(kind=tg.SCENE_ROOM), "sphere3": dict(kind=tg.SCENE_SPHERE_ROOM, detail=3),
                     "soup": dict(kind=tg.SCENE_SOUP, count=3000, seed=9),
                     "baffle": dict(kind=tg.SCENE_BAFFLE_ROOM, detail=8)}.items():
        m = tg.make_scene(**kw)
        nodes, tris, box = tg.KDTree.from_mesh(m).export()
        out[name] = (m, ctx.upload(nodes, tris, box), orc.Scene(nodes, tris, box))
    return out


def make_jobs(scenes):
    spec = [("room", 32, 32, 2, 3), ("sphere3", 48, 24, 3, 2), ("soup", 40, 40, 1, 4), ("baffle", 17, 13, 5, 5),
            ("room", 8, 8, 64, 1)]
    jobs = []
    for k, (name, w, h, spp, depth) in enumerate(spec):
        m, sid, _ = scenes[name]
        jobs.append(tg.make_job(sid, m, w, h, pixel_samples=spp, max_depth=depth, seed=100 + k))
    return jobs


def test_batch_equals_single_renders(ctx, scenes):
    jobs = make_jobs(scenes)
    g0 = ctx.graph_launch_count()
    imgs, stats = ctx.render(jobs)
    assert ctx.graph_launch_count() == g0 + 1          # one captured graph for the batch
    for job, img, st in zip(jobs, imgs, stats):
        (alone,), (sa,) = ctx.render([job])
        assert np.array_equal(img, alone)
        assert st.rays == sa.rays and st.shadow_rays == sa.shadow_rays
        assert st.primary_rays == job.width * job.height * job.pixel_samples


def test_batch_with_short_passes(ctx, scenes):
    """Passes of 1024 paths: passes split jobs and hold pieces of several."""
    jobs = make_jobs(scenes)
    a, sa = ctx.render(jobs)
    ctx.set_chunk_paths(1024)
    try:
        b, sb = ctx.render(jobs)
    finally:
        ctx.set_chunk_paths(1 << 24)
    for x, y, p, q in zip(a, b, sa, sb):
        assert np.array_equal(x, y) and p.rays == q.rays


def test_batch_matches_oracle(ctx, scenes):
    jobs = make_jobs(scenes)[:3]
    imgs, stats = ctx.render(jobs)
    names = ["room", "sphere3", "soup"]
    for name, job, img, st in zip(names, jobs, imgs, stats):
        m, _, ref = scenes[name]
        rimg, rst = ref.render(m.camera, m.light, job.width, job.height, job.pixel_samples, job.max_depth,
                               seed=job.seed)
        diff = np.abs(img - rimg).max(axis=-1)
        assert (diff <= 2e-3).mean() >= 0.99 and np.abs(img - rimg).mean() < 1e-3
        assert abs(int(st.rays) - int(rst[0])) <= 0.005 * int(rst[0]) + 2


def test_graph_mode_single_job(ctx, scenes):
    m, sid, _ = scenes["sphere3"]
    job = tg.make_job(sid, m, 24, 24, pixel_samples=2, max_depth=3, seed=3)
    (a,), _ = ctx.render([job])
    ctx.set_graph_mode(True)
    try:
        g0 = ctx.graph_launch_count()
        (b,), _ = ctx.render([job])
        assert ctx.graph_launch_count() == g0 + 1
    finally:
        ctx.set_graph_mode(False)
    assert np.array_equal(a, b)


def test_graph_reuse_across_batches(ctx, scenes):
    """Batches of the same shape update the instantiated graph in place; the
    images equal uncaptured renders, also after a batch of another shape."""
    import copy
    jobs = make_jobs(scenes)
    reseeded = [copy.copy(j) for j in jobs]
    for j in reseeded:
        j.seed += 1000
    a, _ = ctx.render(jobs)
    b, _ = ctx.render(reseeded)
    ctx.render(jobs[:3])                      # another topology in between
    c, _ = ctx.render(jobs)
    ctx.set_graph_mode(tg.GRAPH_NEVER)
    try:
        d, _ = ctx.render(reseeded)
    finally:
        ctx.set_graph_mode(tg.GRAPH_AUTO)
    assert all(np.array_equal(x, y) for x, y in zip(a, c))
    assert all(np.array_equal(x, y) for x, y in zip(b, d))
    assert not all(np.array_equal(x, y) for x, y in zip(a, b))
    with pytest.raises(tg.TurnerError):
        ctx.set_graph_mode(7)


def test_linear_output_matches_oracle(ctx, scenes):
    m, sid, ref = scenes["room"]
    job = tg.make_job(sid, m, 32, 32, pixel_samples=4, max_depth=3, seed=21)
    job.linear_output = 1
    (img,), _ = ctx.render([job])
    rimg, _ = ref.render(m.camera, m.light, 32, 32, 4, 3, seed=21, tone_map=False)
    close = np.abs(img - rimg) <= 1e-4 * np.maximum(1.0, np.abs(rimg))
    assert close.all(axis=-1).mean() >= 0.99


def test_fp64_accumulation(ctx, scenes):
    """Two passes of 4 samples: the FP64 mean equals the mean of the oracle's
    two linear renders with the pass seeds; more passes extend the same sum;
    another seed starts a new one."""
    m, sid, ref = scenes["sphere3"]
    job = tg.make_job(sid, m, 24, 16, pixel_samples=4, max_depth=3, seed=77)
    mean, total = ctx.accumulate(job, 2)
    assert total == 8
    golden = np.zeros((16, 24, 4))
    for p in range(2):
        seed = 77 ^ ((0x9E3779B97F4A7C15 * (p + 1)) & 0xFFFFFFFFFFFFFFFF)
        img, _ = ref.render(m.camera, m.light, 24, 16, 4, 3, seed=seed, tone_map=False)
        golden += img.astype(np.float64) / 2
    close = np.abs(mean - golden) <= 1e-4 * np.maximum(1.0, np.abs(golden))
    assert close.all(axis=-1).mean() >= 0.99
    mean3, total3 = ctx.accumulate(job, 1)
    assert total3 == 12
    job2 = tg.make_job(sid, m, 24, 16, pixel_samples=4, max_depth=3, seed=78)
    _, total_new = ctx.accumulate(job2, 1)
    assert total_new == 4


def test_autotune_caches_and_keeps_images(ctx, scenes, tmp_path, monkeypatch):
    """The tuner times launch shapes on the batch, applies the fastest and
    caches it per GPU and batch shape; any tuned shape renders the same image."""
    monkeypatch.setenv("TURNER_TUNE_CACHE", str(tmp_path / "tuning.txt"))
    default = ctx.get_tuning()
    jobs = make_jobs(scenes)[:3]
    before, _ = ctx.render(jobs)
    t = ctx.autotune(jobs, force=True)
    assert t.candidates >= 5 and t.ms > 0
    assert t.block in (128, 256) and t.stack in (64, 128) and t.chunk_paths >= 1024
    cached = ctx.autotune(jobs)
    assert cached.candidates == 0 and cached.as_dict()["block"] == t.block
    after, _ = ctx.render(jobs)
    for a, b in zip(before, after):
        assert np.array_equal(a, b)
    assert 1 <= t.refill_camera <= 32 and 1 <= t.refill_bounce <= 32 and t.packets in (0, 1)
    for shape in ({"block": 256, "stack": 64, "mailbox": 0, "min_blocks": 0, "refill_camera": 16, "packets": 0},
                  {"block": 128, "stack": 128, "mailbox": 1, "min_blocks": 12, "refill_bounce": 4},
                  {"block": 128, "stack": 64, "mailbox": 1, "min_blocks": 0, "refill_camera": 8,
                   "refill_bounce": 1}):
        tt = ctx.get_tuning()
        for k, v in shape.items():
            setattr(tt, k, v)
        ctx.set_tuning(tt)
        again, _ = ctx.render(jobs)
        for a, b in zip(before, again):
            assert np.array_equal(a, b)
    for field, bad in (("refill_camera", 0), ("refill_bounce", 33), ("packets", 2)):
        tt = ctx.get_tuning()
        setattr(tt, field, bad)
        with pytest.raises(tg.TurnerError) as e:
            ctx.set_tuning(tt)
        assert e.value.status == tg.ERR_INVALID_ARG
    ctx.set_tuning(default)


def test_too_many_jobs_rejected(ctx, scenes):
    m, sid, _ = scenes["room"]
    with pytest.raises(tg.TurnerError) as e:
        ctx.render([tg.make_job(sid, m, 2, 2)] * 4097)
    assert e.value.status == tg.ERR_TOO_LARGE
