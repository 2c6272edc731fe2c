"""GPU closest-hit traversal == KDTreeIntersection::intersect, bit for bit.

Every case goes through the C ABI (turner_intersect) and is compared with the
CPU oracle on the same tree and rays: triangle ids equal, r, s, t equal as
bit patterns (the kernels round like the reference's C++)."""
from pathlib import Path

import numpy as np
import pytest

import turner_gb300 as tg
from oracle import oracle as orc

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"


@pytest.fixture(scope="module")
def ctx():
    c = tg.Context(0)
    yield c
    c.close()


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def assert_same(gpu, ref, exact_rst=True):
    hid, r, s, t = gpu
    rid, rr, rs, rt = ref
    mism = np.nonzero(hid != rid)[0]
    assert mism.size == 0, f"{mism.size} id mismatches, first {mism[:5]}"
    if exact_rst:
        for a, b in ((r, rr), (s, rs), (t, rt)):
            assert np.array_equal(bits(a), bits(b))


SCENES = {
    "room": dict(kind=tg.SCENE_ROOM),
    "sphere5": dict(kind=tg.SCENE_SPHERE_ROOM, detail=5),
    "soup20k": dict(kind=tg.SCENE_SOUP, count=20000, seed=4),
    "baffle32": dict(kind=tg.SCENE_BAFFLE_ROOM, detail=32),
}


@pytest.fixture(scope="module")
def uploaded(ctx):
    out = {}
    for name, kw in SCENES.items():
        t = tg.KDTree.from_mesh(tg.make_scene(**kw))
        nodes, tris, box = t.export()
        out[name] = (ctx.upload(nodes, tris, box), orc.Scene(nodes, tris, box), box)
    return out


@pytest.mark.parametrize("name", list(SCENES))
def test_parity_random_rays(ctx, uploaded, name):
    sid, ref, box = uploaded[name]
    o, d = tg.make_rays(200_000, box, seed=17)
    d[0, ::13] = 0       # fix_direction paths
    d[2, ::19] = 0
    assert_same(ctx.intersect(sid, o, d), ref.intersect(o, d))


@pytest.mark.parametrize("name", ["sphere5", "soup20k"])
def test_fast_mode_matches_parity(ctx, uploaded, name):
    """FAST (early exit with margin) gives the same closest hit as PARITY."""
    sid, ref, box = uploaded[name]
    o, d = tg.make_rays(300_000, box, seed=23)
    assert_same(ctx.intersect(sid, o, d, mode=tg.TRAVERSAL_FAST), ref.intersect(o, d))


@pytest.mark.parametrize("persistent,blocks", [(False, 0), (True, 0), (True, 1), (True, 3)])
def test_launch_shapes_agree(ctx, uploaded, persistent, blocks):
    """One thread per ray, or persistent lanes with ray replacement at any
    number of resident blocks: the same bit-exact answers."""
    sid, ref, box = uploaded["soup20k"]
    o, d = tg.make_rays(100_000, box, seed=31)
    ctx.set_traversal_launch(persistent, blocks)
    try:
        gpu = ctx.intersect(sid, o, d)
    finally:
        ctx.set_traversal_launch(True, 0)
    assert_same(gpu, ref.intersect(o, d))


@pytest.mark.parametrize("block,stack,mailbox,min_blocks", [(128, 128, 1, 0), (128, 64, 1, 12), (256, 64, 0, 0),
                                                           (128, 128, 0, 12), (128, 64, 0, 10), (128, 128, 0, 16),
                                                           (128, 128, 1, 16), (128, 128, 0, 0)])
def test_tuned_shapes_agree(ctx, uploaded, block, stack, mailbox, min_blocks):
    """Every tuning variant (block size, stack depth, triangle mailbox,
    register cap) returns the same bit-exact closest hits."""
    default = ctx.get_tuning()
    for name in ("sphere5", "soup20k"):
        sid, ref, box = uploaded[name]
        o, d = tg.make_rays(150_000, box, seed=41)
        ctx.set_tuning(tg.Tuning(1, 0, block, stack, 1 << 24, mailbox, min_blocks, 0.0, 0, 32, 2, 1))
        try:
            gpu = ctx.intersect(sid, o, d)
            fast = ctx.intersect(sid, o, d, mode=tg.TRAVERSAL_FAST)
        finally:
            ctx.set_tuning(default)
        cpu = ref.intersect(o, d)
        assert_same(gpu, cpu)
        assert np.array_equal(fast[0], cpu[0])


def test_reference_fixture_scenes(ctx):
    """The reference's kd-tree tests (tests/test_kdtree.cpp) on the GPU."""
    kd = dict(np.load(GOLD / "ref_kdtree_tests.npz"))
    for name in ["four"] + [f"coplanar{a}" for a in range(3)] + [f"stacked{a}" for a in range(3)]:
        sid = ctx.upload(kd[f"{name}_nodes"], kd[f"{name}_tris"], kd[f"{name}_box"])
        hid, r, s, t = ctx.intersect(sid, kd[f"{name}_rays_o"], kd[f"{name}_rays_d"])
        assert np.array_equal(hid, kd[f"{name}_hit_i"]), name
        for k, v in zip("rst", (r, s, t)):
            gold = kd[f"{name}_hit_{k}"]
            hit = hid != tg.MISS
            assert np.array_equal(bits(v)[hit], bits(gold)[hit]), (name, k)
    # four separated triangles: exact known answers (test_kdtree.cpp:34-62)
    sid = ctx.upload(kd["four_nodes"], kd["four_tris"], kd["four_box"])
    hid, r, s, t = ctx.intersect(sid, kd["four_rays_o"], kd["four_rays_d"])
    assert hid.tolist() == [0, 1, 2, 3] and (r == 1).all() and s.tolist() == [0.5, 0, 0, 0] and (t == 0.5).all()


def test_golden_scene_rays(ctx):
    """GPU hits == the reference's recorded hits (tests/golden/ref_scenes.npz)."""
    g = dict(np.load(GOLD / "ref_scenes.npz"))
    for name, kw in {"room": dict(kind=tg.SCENE_ROOM), "sphere3": dict(kind=tg.SCENE_SPHERE_ROOM, detail=3),
                     "soup2000": dict(kind=tg.SCENE_SOUP, count=2000, seed=7),
                     "baffle8": dict(kind=tg.SCENE_BAFFLE_ROOM, detail=8)}.items():
        sid = ctx.upload_tree(tg.KDTree.from_mesh(tg.make_scene(**kw)))
        hid, r, s, t = ctx.intersect(sid, g[f"{name}_rays_o"], g[f"{name}_rays_d"])
        assert np.array_equal(hid, g[f"{name}_hit_i"]), name
        for k, v in zip("rst", (r, s, t)):
            assert np.array_equal(bits(v), bits(g[f"{name}_hit_{k}"])), (name, k)


def test_edge_rays(ctx, uploaded):
    """Axis-aligned, zero, NaN and huge components, origins outside the box:
    no fault, same answers as the oracle."""
    sid, ref, box = uploaded["sphere5"]
    o = np.array([[2.78, 2.78, -1.0], [-10, 2, -2], [2.78, 2.78, 0.0], [np.nan, 1, 1], [1, 1, 1], [2, 2, -2],
                  [1e30, 0, 0], [2.78, 1.65, -3.5]], np.float32).T
    d = np.array([[0, 0, -1], [1, 0, 0], [0, 0, 0], [1, 0, 0], [np.nan, 1, 0], [0, -1e-30, 0], [-1, 0, 0],
                  [0, 1, 0]], np.float32).T
    gpu = ctx.intersect(sid, o, d)
    cpu = ref.intersect(o, d)
    assert np.array_equal(gpu[0], cpu[0])


@pytest.mark.parametrize("kind,kw", [(tg.SCENE_SPHERE_ROOM, dict(detail=5)), (tg.SCENE_SOUP, dict(count=5000, seed=9))])
def test_vertex_and_edge_aimed_rays(ctx, kind, kw):
    """Rays aimed at triangle vertices, edge midpoints and points just inside
    and outside edges: the barycentric numerators are zero or a few ulps from
    it, where the sign tests that skip divides must agree with dividing."""
    mesh = tg.make_scene(kind, **kw)
    t = tg.KDTree.from_mesh(mesh)
    nodes, tris, box = t.export()
    sid, ref = ctx.upload(nodes, tris, box), orc.Scene(nodes, tris, box)
    rng = np.random.default_rng(31)
    v = mesh.vertices.reshape(-1, 3, 3).astype(np.float64)
    pick = rng.integers(0, v.shape[0], 40_000)
    a, b, c = v[pick, 0], v[pick, 1], v[pick, 2]
    w = rng.integers(0, 4, pick.size)[:, None]
    eps = rng.choice([0.0, 1e-7, -1e-7, 1e-6, -1e-6], pick.size)[:, None]
    mid = 0.5 * (a + b)
    target = np.where(w == 0, a, np.where(w == 1, mid, np.where(w == 2, mid + eps * (c - mid), (a + b + c) / 3)))
    lo, hi = np.array(box[:3]), np.array(box[3:])
    org = lo + (hi - lo) * rng.random((pick.size, 3))
    d = target - org
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    o32, d32 = org.T.astype(np.float32).copy(), d.T.astype(np.float32).copy()
    assert_same(ctx.intersect(sid, o32, d32), ref.intersect(o32, d32))


def test_device_buffers(ctx, uploaded):
    torch = pytest.importorskip("torch")
    sid, ref, box = uploaded["sphere5"]
    o, d = tg.make_rays(65_536, box, seed=5)
    dev = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (*o, *d)]
    out_i = torch.empty(o.shape[1], dtype=torch.int32, device="cuda")
    outs = [torch.empty(o.shape[1], dtype=torch.float32, device="cuda") for _ in range(3)]
    ctx.intersect_device(sid, [t.data_ptr() for t in dev], o.shape[1], [out_i.data_ptr()] + [t.data_ptr() for t in outs])
    hid = out_i.cpu().numpy().view(np.uint32)
    rid, rr, rs, rt = ref.intersect(o, d)
    assert np.array_equal(hid, rid)
    assert np.array_equal(bits(outs[0].cpu().numpy()), bits(rr))


def test_empty_batch(ctx, uploaded):
    sid = uploaded["room"][0]
    z = np.zeros((3, 0), np.float32)
    hid, r, s, t = ctx.intersect(sid, z, z)
    assert hid.size == 0


def test_bad_scene_rejected(ctx):
    t = tg.KDTree.from_mesh(tg.make_scene(tg.SCENE_SPHERE_ROOM, detail=2))
    nodes, tris, box = t.export()
    bad = nodes.copy()
    inner = np.nonzero((nodes & np.uint64(3)) != np.uint64(3))[0][0]
    bad[inner] = (bad[inner] & np.uint64(0xFFFFFFFF00000003)) | np.uint64((nodes.size + 3) << 2)
    with pytest.raises(tg.TurnerError) as e:
        ctx.upload(bad, tris, box)
    assert e.value.status == tg.ERR_BAD_SCENE
    with pytest.raises(tg.TurnerError):
        ctx.intersect(999, np.zeros((3, 1), np.float32), np.ones((3, 1), np.float32))


@pytest.mark.slow
def test_full_hit_test_set(ctx, sphere_room_327k):
    """16,777,216 rays (origins uniform in the room, directions uniform on the
    sphere) against the 327,692-triangle tree: every hit index equal."""
    _, nodes, tris, box, ref = sphere_room_327k
    sid = ctx.upload(nodes, tris, box)
    n = 1 << 24
    o, d = tg.make_rays(n, box, seed=2024)
    gpu = ctx.intersect(sid, o, d)
    cpu = ref.intersect(o, d)
    assert_same(gpu, cpu)
    fast = ctx.intersect(sid, o, d, mode=tg.TRAVERSAL_FAST)
    assert np.array_equal(fast[0], cpu[0])


@pytest.mark.parametrize("ring", [4, 8, "speculative", "packet"])
def test_shared_memory_stack_is_exact(ctx, uploaded, ring):
    """The traversal stack with its newest 4 or 8 entries in shared memory
    and older ones in local memory, and speculative traversal rounds:
    identical hits, for closest-hit and shadow (any-hit) traversal, on trees
    much deeper than the ring."""
    def setting(on):
        if ring == "speculative":
            ctx.set_traversal_speculative(on)
        elif ring == "packet":
            ctx.set_traversal_packet(tg.PACKET_CAMERA | (tg.PACKET_BATCHED if on else 0))
        else:
            ctx.set_traversal_ring(ring if on else 0)

    for name in ("sphere5", "baffle32", "soup20k"):
        sid, ref, box = uploaded[name]
        o, d = tg.make_rays(100_000, box, seed=23)
        tm = np.random.default_rng(3).uniform(0, 6, o.shape[1]).astype(np.float32)
        base = ctx.intersect(sid, o, d)
        occ = ctx.occluded(sid, o, d, tm)
        assert_same(base, ref.intersect(o, d))
        setting(True)
        try:
            got = ctx.intersect(sid, o, d)
            occ2 = ctx.occluded(sid, o, d, tm)
        finally:
            setting(False)
        assert_same(got, base)
        assert np.array_equal(occ, occ2)
    with pytest.raises(tg.TurnerError):
        ctx.set_traversal_ring(5)


def test_packet_traversal_of_coherent_rays_is_exact(ctx, uploaded):
    """Camera-like ray bundles (32 rays with nearly one direction from one
    point, so whole warps share their direction signs) traverse as packets
    and give the oracle's answers bit for bit, for closest-hit and shadow
    traversal, also with some bundles mixing direction signs."""
    rng = np.random.default_rng(41)
    for name in ("sphere5", "baffle32", "room"):
        sid, ref, box = uploaded[name]
        lo, hi = box[:3], box[3:]
        n_b = 4096
        orig = (lo + (hi - lo) * rng.uniform(0.2, 0.8, (n_b, 3))).astype(np.float32)
        axis = rng.normal(size=(n_b, 3))
        axis /= np.linalg.norm(axis, axis=1, keepdims=True)
        spread = np.where(np.arange(n_b)[:, None] % 7 == 0, 0.5, 0.02)   # every 7th bundle mixes signs
        d = axis[:, None, :] + spread[:, None, :] * rng.normal(size=(n_b, 32, 3))
        o = np.repeat(orig[:, None, :], 32, axis=1)
        o, d = o.reshape(-1, 3).T.astype(np.float32), d.reshape(-1, 3).T.astype(np.float32)
        tm = rng.uniform(0, 6, o.shape[1]).astype(np.float32)
        want = ref.intersect(o, d)
        occ0 = ctx.occluded(sid, o, d, tm)
        ctx.set_traversal_packet(tg.PACKET_CAMERA | tg.PACKET_BATCHED)
        try:
            got = ctx.intersect(sid, o, d)
            occ1 = ctx.occluded(sid, o, d, tm)
        finally:
            ctx.set_traversal_packet(tg.PACKET_CAMERA)
        assert_same(got, want)
        assert np.array_equal(occ0, occ1)
        rid, rr = want[0], want[1]
        assert np.array_equal(occ1, (rid < tg.MISS) & ~(rr > tm))
