"""Image parity at the configured workloads' sizes, row bands, and per-ray
shadow decisions, all through the C ABI against the oracle.

Image tolerance (the same as tests/test_gpu_render.py): the GPU and the oracle
trace the same rays with bit-identical traversal and differ only in the last
ulp of cosf/sinf/expf/powf and in the order a path's radiance is summed, so
  - at least 99% of pixels agree within 2e-3 on every channel after tone
    mapping, and
  - the mean absolute difference is below 1e-3, and
  - the reference ray count (pathtracer.cpp:21) agrees within 0.5%.
Shadow decisions and row bands are exact (bit for bit)."""
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


def check_close(img, ref, frac=0.99, tol=2e-3, mean_tol=1e-3):
    assert img.shape == ref.shape
    assert np.isfinite(img).all()
    diff = np.abs(img - ref).max(axis=-1)
    assert (diff <= tol).mean() >= frac, f"only {(diff <= tol).mean():.4f} of pixels within {tol}"
    assert np.abs(img - ref).mean() < mean_tol, f"mean |diff| {np.abs(img - ref).mean():.2e}"


def check_rays(gpu_rays, ref_rays):
    assert abs(int(gpu_rays) - int(ref_rays)) <= 0.005 * int(ref_rays) + 2, (gpu_rays, ref_rays)


def oracle_render(sc, m, job, rows=None):
    return sc.render(m.camera, m.light, job.width, job.height, job.pixel_samples, job.max_depth,
                     mc=job.monte_carlo_samples, seed=job.seed, exposure=job.exposure,
                     inverse_gamma=job.inverse_gamma, gamma=bool(job.gamma_correction),
                     background=tuple(job.background), sampling=job.sampling, rows=rows)


def test_room_320_full_frame(ctx):
    """The README's workload in full: 36-triangle room, 320x320, 8 pixel
    samples, depth 3, -m 1 (819,200 paths)."""
    m = tg.make_scene(tg.SCENE_ROOM)
    nodes, tris, box = tg.KDTree.from_mesh(m).export()
    sid = ctx.upload(nodes, tris, box)
    sc = orc.Scene(nodes, tris, box)
    job = tg.make_job(sid, m, 320, pixel_samples=8, max_depth=3, seed=42)
    assert job.height == 320
    (img,), (st,) = ctx.render([job])
    ref, rst = oracle_render(sc, m, job)
    check_close(img, ref)
    assert st.primary_rays == 320 * 320 * 8 == int(rst[1])
    check_rays(st.rays, rst[0])


# eight bands of four rows spread over the 1080 rows of the large-mesh frame
SPHERE_BANDS = [(y, y + 4) for y in np.linspace(0, 1076, 8).astype(int)]


def test_sphere_room_1920_rows_spread(ctx, sphere_room_327k):
    """32 rows spread over the large-mesh frame (327,692 triangles, 1920
    wide, 16 pixel samples, depth 3), each band rendered on its own through
    the job's row range and compared with the oracle's render of those rows."""
    m, nodes, tris, box, sc = sphere_room_327k
    sid = ctx.upload(nodes, tris, box)
    gpu_rays = ref_rays = 0
    imgs, refs = [], []
    for y0, y1 in SPHERE_BANDS:
        job = tg.make_job(sid, m, 1920, pixel_samples=16, max_depth=3, seed=5, rows=(y0, y1))
        assert job.height == 1080
        (img,), (st,) = ctx.render([job])
        ref, rst = oracle_render(sc, m, job, rows=(y0, y1))
        assert st.primary_rays == 1920 * 4 * 16 == int(rst[1])
        imgs.append(img)
        refs.append(ref[y0:y1])
        gpu_rays += st.rays
        ref_rays += int(rst[0])
    check_close(np.concatenate(imgs), np.concatenate(refs))
    check_rays(gpu_rays, ref_rays)


@pytest.mark.parametrize("sampling", [tg.SAMPLING_UNIFORM, tg.SAMPLING_COSINE])
def test_baffle_room_40k_band_depth5(ctx, sampling):
    """The indirect-lit room at its configured tessellation (64 x 64 quads per
    wall, 40,962 triangles) and depth 5: a 16-row band through the middle of
    the 1024x1024 frame, 8 pixel samples, uniform (the reference's) and cosine
    (the plain tracer the learned proposal is compared with) sampling."""
    m = tg.make_scene(tg.SCENE_BAFFLE_ROOM, detail=64)
    assert m.n_triangles > 40000
    nodes, tris, box = tg.KDTree.from_mesh(m).export()
    sid = ctx.upload(nodes, tris, box)
    sc = orc.Scene(nodes, tris, box)
    job = tg.make_job(sid, m, 1024, 1024, pixel_samples=8, max_depth=5, seed=11, sampling=sampling,
                      rows=(504, 520))
    (img,), (st,) = ctx.render([job])
    ref, rst = oracle_render(sc, m, job, rows=(504, 520))
    check_close(img, ref[504:520])
    check_rays(st.rays, rst[0])


def test_row_bands_equal_full_frame(ctx):
    """Rows [y0, y1) rendered alone are bit-identical to those rows of the
    full render, so a frame partitioned by rows over GPUs equals the
    single-GPU frame (the reference's unit of work is one row,
    main.cpp:193-226)."""
    m = tg.make_scene(tg.SCENE_SPHERE_ROOM, detail=4, aspect=16 / 9)
    sid = ctx.upload_tree(tg.KDTree.from_mesh(m))
    full_job = tg.make_job(sid, m, 160, pixel_samples=4, max_depth=3, seed=21)
    h = full_job.height
    (full,), (fst,) = ctx.render([full_job])
    parts, rays = [], 0
    from turner_gb300.shard import row_range

    for r in range(3):
        y0, y1 = row_range(h, r, 3)
        job = tg.make_job(sid, m, 160, pixel_samples=4, max_depth=3, seed=21, rows=(y0, y1))
        (img,), (st,) = ctx.render([job])
        assert img.shape == (y1 - y0, 160, 4)
        assert st.primary_rays == (y1 - y0) * 160 * 4
        parts.append(img)
        rays += st.rays
    assert np.array_equal(np.concatenate(parts).view(np.uint32), full.view(np.uint32))
    assert rays == fst.rays
    # a band inside a multi-job batch is the same band
    j1 = tg.make_job(sid, m, 160, pixel_samples=4, max_depth=3, seed=21, rows=(10, 30))
    j2 = tg.make_job(sid, m, 64, pixel_samples=2, max_depth=2, seed=3)
    (a, _), _ = ctx.render([j1, j2])
    assert np.array_equal(a.view(np.uint32), full[10:30].view(np.uint32))
    # FP64 accumulation of a band
    acc, n = ctx.accumulate(tg.make_job(sid, m, 160, pixel_samples=2, max_depth=3, seed=4, rows=(40, 42)), 2)
    assert acc.shape == (2, 160, 4) and n == 4 and np.isfinite(acc).all()


def test_row_range_rejected(ctx):
    m = tg.make_scene(tg.SCENE_ROOM)
    sid = ctx.upload_tree(tg.KDTree.from_mesh(m))
    for rows in ((5, 5), (10, 4), (0, 33), (32, 0)):
        job = tg.make_job(sid, m, 32, 32, rows=rows)
        with pytest.raises(tg.TurnerError) as e:
            ctx.render([job])
        assert e.value.status == tg.ERR_INVALID_ARG


def _frame_hits(ctx, sid, m, tris, box, w, h):
    """Hit points of the frame's primary rays (pixel centres) and of random
    rays in the room, with the shading normal and offset point of
    pathtracer.cpp:30-36."""
    cam = m.camera
    dx = np.float32(cam.delta_x)
    dy = np.float32(cam.delta_x) / np.float32(cam.aspect)
    ys, xs = np.mgrid[0:h, 0:w].astype(np.float32)
    px, py = xs + np.float32(0.5), ys + np.float32(0.5)
    v = np.stack([-dx * (1 - 2 * px / np.float32(w)), dy * (1 - 2 * py / np.float32(h)),
                  -np.ones_like(px)]).reshape(3, -1)
    rot = np.array(cam.trafo, np.float32).reshape(3, 3)
    d = (rot @ v).astype(np.float32)
    o = np.repeat(np.array(cam.position, np.float32)[:, None], d.shape[1], axis=1)
    o2, d2 = tg.make_rays(1 << 20, box, seed=77)
    o = np.concatenate([o, o2], 1)
    d = np.concatenate([d, d2], 1)
    hid, r, s, t = ctx.intersect(sid, o, d)
    keep = hid < tg.MISS
    o, d, hid, r, s, t = o[:, keep], d[:, keep], hid[keep], r[keep], s[keep], t[keep]
    p = o + r * d
    nrm = tris.reshape(-1, 48)[hid][:, 9:18].reshape(-1, 3, 3)   # n0, n1, n2
    wts = np.stack([np.float32(1) - s - t, s, t], 1)[:, :, None]
    n = (wts * nrm).sum(1).T
    n = n / np.sqrt((n * n).sum(0))
    p2 = (p + np.float32(1e-4) * n).astype(np.float32)
    return p, p2


def test_shadow_decisions_per_ray(ctx, sphere_room_327k):
    """Every shadow ray of the large-mesh frame's hit points decides "blocked"
    exactly as the reference does: it traces the closest hit from p2 toward
    the light and calls the point lit iff there is no hit or r > |L - p2|
    (pathtracer.cpp:44-58). turner_occluded (the any-hit test the renders
    use) must agree ray by ray, also with the distance set exactly to the
    closest hit (blocked) and one ulp below it (not blocked)."""
    m, nodes, tris, box, sc = sphere_room_327k
    sid = ctx.upload(nodes, tris, box)
    p, p2 = _frame_hits(ctx, sid, m, tris, box, 480, 270)
    light = np.array(m.light.position, np.float32)[:, None]
    lv = light - p
    ld = (lv / np.sqrt((lv * lv).sum(0))).astype(np.float32)
    qv = light - p2
    dist = np.sqrt((qv * qv).sum(0)).astype(np.float32)
    rid, rr, _, _ = sc.intersect(p2, ld)
    ref_blocked = (rid < tg.MISS) & ~(rr > dist)
    got = ctx.occluded(sid, p2, ld, dist)
    assert 0.05 < ref_blocked.mean() < 0.95, ref_blocked.mean()
    mism = np.nonzero(got != ref_blocked)[0]
    assert mism.size == 0, f"{mism.size} of {got.size} shadow decisions differ, first {mism[:5]}"
    # the boundary: tmax = the closest hit's r is blocked, one ulp less is not
    hit = rid < tg.MISS
    at = ctx.occluded(sid, p2[:, hit], ld[:, hit], rr[hit])
    below = ctx.occluded(sid, p2[:, hit], ld[:, hit], np.nextafter(rr[hit], np.float32(-np.inf)))
    assert at.all()
    assert not below.any()
    # the same rays through the closest-hit entry point: the decision is that of its answer
    gid, gr, _, _ = ctx.intersect(sid, p2, ld)
    assert np.array_equal(gid, rid) and np.array_equal(gr.view(np.uint32), rr.view(np.uint32))


@pytest.mark.parametrize("sampling", [tg.SAMPLING_UNIFORM, tg.SAMPLING_COSINE])
def test_baffle_sphere_view_band_depth5(ctx, sampling):
    """The 16-view workload's scene (the 327,680-triangle displaced sphere in
    the baffled room, 368,654 triangles) seen from the circle view that looks
    through the room's open front, 1920x1080 at depth 5: rows 536-544, 4
    pixel samples."""
    m = tg.make_scene(tg.SCENE_BAFFLE_SPHERE, detail=7, count=64, aspect=16 / 9)
    nodes, tris, box = tg.KDTree.from_mesh(m).export()
    sid = ctx.upload(nodes, tris, box)
    sc = orc.Scene(nodes, tris, box)
    cam = tg.look_at_camera((2.78, 1.5, -3.5 + 4.0), (2.78, 1.65, -3.5), 16 / 9)
    job = tg.make_job(sid, m, 1920, 1080, pixel_samples=4, max_depth=5, seed=17, sampling=sampling, rows=(536, 544))
    job.camera = cam
    (img,), (st,) = ctx.render([job])
    ref, rst = sc.render(cam, m.light, 1920, 1080, 4, 5, seed=17, sampling=sampling, rows=(536, 544))
    check_close(img, ref[536:544])
    check_rays(st.rays, rst[0])


def test_large_soup_band(ctx):
    """A scene of the batched workload's kind at its larger end: a clustered
    soup of 100,000 triangles in the room, 1024 wide, 16 pixel samples,
    depth 4, a 12-row band."""
    m = tg.make_scene(tg.SCENE_SOUP, count=100_000, seed=1234)
    nodes, tris, box = tg.KDTree.from_mesh(m).export()
    sid = ctx.upload(nodes, tris, box)
    sc = orc.Scene(nodes, tris, box)
    job = tg.make_job(sid, m, 1024, 1024, pixel_samples=16, max_depth=4, seed=9, rows=(500, 512))
    (img,), (st,) = ctx.render([job])
    ref, rst = oracle_render(sc, m, job, rows=(500, 512))
    check_close(img, ref[500:512])
    check_rays(st.rays, rst[0])
