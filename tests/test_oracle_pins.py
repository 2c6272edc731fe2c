"""The CPU oracle pinned to the reference: its known-answer unit tests and
golden outputs of the reference itself (tests/golden/, from oracle/_ref)."""
import hashlib
import math
import platform
from pathlib import Path

import numpy as np
import pytest

import turner_gb300 as tg
from oracle import oracle as orc

GOLD = Path(__file__).resolve().parent / "golden"
X86 = platform.machine() in ("x86_64", "AMD64")


@pytest.fixture(scope="module")
def kd():
    return dict(np.load(GOLD / "ref_kdtree_tests.npz"))


@pytest.fixture(scope="module")
def scenes():
    return dict(np.load(GOLD / "ref_scenes.npz"))


@pytest.fixture(scope="module")
def renders():
    return dict(np.load(GOLD / "ref_renders.npz"))


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def scene_from(kd, name):
    return orc.Scene(kd[f"{name}_nodes"], kd[f"{name}_tris"], kd[f"{name}_box"])


# ---------------------------------------------------- tests/test_kdtree.cpp
def test_four_separated_triangles(kd):
    """test_kdtree.cpp:23-63: height 1, 5 nodes, exact r, s, t per ray."""
    assert int(kd["four_height"]) == 1 and kd["four_nodes"].size == 5
    sc = scene_from(kd, "four")
    hid, r, s, t = sc.intersect(kd["four_rays_o"], kd["four_rays_d"])
    assert hid.tolist() == [0, 1, 2, 3]
    assert (r == 1).all()
    assert s.tolist() == [0.5, 0.0, 0.0, 0.0] and (t == 0.5).all()
    for k, v in zip("irst", (hid, r, s, t)):
        assert np.array_equal(bits(v) if k != "i" else v, bits(kd[f"four_hit_{k}"]) if k != "i" else kd["four_hit_i"])


def test_cube_and_overlap_heights(kd):
    """test_kdtree.cpp:16-21 (overlap: height 0) and :162-186 (cube: height 0, 7 nodes)."""
    assert int(kd["overlap_height"]) == 0
    assert int(kd["cube_height"]) == 0 and kd["cube_nodes"].size == 7


@pytest.mark.parametrize("axis", [0, 1, 2])
def test_all_triangles_coplanar(kd, axis):
    """test_kdtree.cpp:188-209: parallel ray misses, ray through zero hits."""
    sc = scene_from(kd, f"coplanar{axis}")
    hid, r, s, t = sc.intersect(kd[f"coplanar{axis}_rays_o"], kd[f"coplanar{axis}_rays_d"])
    assert hid[0] == orc.MISS and hid[1] != orc.MISS
    assert np.array_equal(hid, kd[f"coplanar{axis}_hit_i"])
    assert np.array_equal(bits(r), bits(kd[f"coplanar{axis}_hit_r"]))


@pytest.mark.parametrize("axis", [0, 1, 2])
def test_intersect_coplanar_stack(kd, axis):
    """test_kdtree.cpp:211-245: from -100 hit id 0 at int(r) == 100; from +100 id 9 at 91."""
    sc = scene_from(kd, f"stacked{axis}")
    hid, r, s, t = sc.intersect(kd[f"stacked{axis}_rays_o"], kd[f"stacked{axis}_rays_d"])
    assert hid.tolist() == [0, 9]
    assert int(r[0]) == 100 and int(r[1]) == 91
    assert (np.abs(s - 1 / 3) < 1e-5).all() and (np.abs(t - 1 / 3) < 1e-5).all()
    for k, v in zip("rst", (r, s, t)):
        assert np.array_equal(bits(v), bits(kd[f"stacked{axis}_hit_{k}"]))


# ------------------------------------------------ tests/test_intersection.cpp
@pytest.mark.parametrize("ray,box,expect", [
    ((0, 0, 0, 1, 1, 1), (-1, -1, -1, 1, 1, 1), True),
    ((10, 0, 0, -1, 0, 0), (-1, -1, -1, 1, 1, 1), True),
    ((0, 10, 0, 0, -1, 0), (-1, -1, -1, 1, 1, 1), True),
    ((0, 0, 10, 0, 0, -1), (-1, -1, -1, 1, 1, 1), True),
    ((0, 0, 0, 1, 0, 0), (-1, -1, 1, 1, 1, 1), False),
    ((-2, -2, -2, -1, 0, 0), (-1, -1, 1, 1, 1, 1), False),
    ((-1, 0, 0, -1, 0, 0), (0, 0, 0, 1, 1, 1), False),
])
def test_ray_box(ray, box, expect):
    """test_intersection.cpp:15-38 (seven ray/AABB cases)."""
    hit, _ = orc.ray_box(ray, box)
    assert hit == expect


# ------------------------------------------------------- golden scene hits
@pytest.mark.parametrize("name", ["room", "sphere3", "soup2000", "baffle8", "mirror"])
def test_oracle_hits_match_reference(scenes, name):
    """Oracle traversal == the reference's traversal, bit for bit, on trees
    identical to the reference's (node/triangle hashes, the mirror room's
    with its reflective materials), 8192 rays incl. zero direction
    components and origins on vertices."""
    kw = {"room": dict(kind=tg.SCENE_ROOM), "sphere3": dict(kind=tg.SCENE_SPHERE_ROOM, detail=3),
          "soup2000": dict(kind=tg.SCENE_SOUP, count=2000, seed=7),
          "baffle8": dict(kind=tg.SCENE_BAFFLE_ROOM, detail=8),
          "mirror": dict(kind=tg.SCENE_MIRROR_ROOM)}[name]
    tree = tg.KDTree.from_mesh(tg.make_scene(**kw))
    nodes, tris, box = tree.export()
    assert hashlib.sha256(nodes.tobytes()).hexdigest() == str(scenes[f"{name}_nodes_sha"])
    assert hashlib.sha256(tris.tobytes()).hexdigest() == str(scenes[f"{name}_tris_sha"])
    sc = orc.Scene(nodes, tris, box)
    hid, r, s, t = sc.intersect(scenes[f"{name}_rays_o"], scenes[f"{name}_rays_d"])
    assert np.array_equal(hid, scenes[f"{name}_hit_i"])
    for k, v in zip("rst", (r, s, t)):
        assert np.array_equal(bits(v), bits(scenes[f"{name}_hit_{k}"])), k


# --------------------------------------------------------- golden renders
RENDERS = {
    "room_48": dict(scene=dict(kind=tg.SCENE_ROOM), w=48, h=48, spp=4, depth=3, seed=7),
    "room_bg_nogamma": dict(scene=dict(kind=tg.SCENE_ROOM), w=40, h=40, spp=2, depth=2, seed=9,
                            background=(0.2, 0.3, 0.4), gamma=False, exposure=0.5),
    "sphere3_32": dict(scene=dict(kind=tg.SCENE_SPHERE_ROOM, detail=3), w=32, h=24, spp=2, depth=3, seed=11),
    "room_depth0": dict(scene=dict(kind=tg.SCENE_ROOM), w=24, h=24, spp=1, depth=0, seed=3),
    "baffle8_32": dict(scene=dict(kind=tg.SCENE_BAFFLE_ROOM, detail=8), w=32, h=32, spp=2, depth=4, seed=5),
    # raytracer.cpp (renderer 1) and raycaster.cpp (renderer 2)
    "mirror_raytrace": dict(scene=dict(kind=tg.SCENE_MIRROR_ROOM), w=48, h=48, spp=1, depth=3, seed=13,
                            renderer=1),
    "mirror_raytrace_d1_shadow08": dict(scene=dict(kind=tg.SCENE_MIRROR_ROOM), w=40, h=32, spp=2, depth=1,
                                        seed=17, renderer=1, shadow=0.8, background=(0.1, 0.2, 0.3)),
    "room_raytrace": dict(scene=dict(kind=tg.SCENE_ROOM), w=32, h=32, spp=1, depth=3, seed=19, renderer=1),
    "room_raycast": dict(scene=dict(kind=tg.SCENE_ROOM), w=40, h=40, spp=2, depth=3, seed=23, renderer=2,
                         max_visibility=6.0),
    "sphere3_raycast_default": dict(scene=dict(kind=tg.SCENE_SPHERE_ROOM, detail=3), w=32, h=24, spp=1, depth=3,
                                    seed=29, renderer=2),
}


@pytest.mark.parametrize("name", list(RENDERS))
def test_oracle_render_matches_reference(renders, name):
    """trace() restated == the reference's trace() under the same per-path
    seeds (path tracer, raytracer and raycaster): identical ray counts; images
    bit-identical on the same libm (x86-64 glibc here), within 1e-6
    elsewhere."""
    cfg = RENDERS[name]
    m = tg.make_scene(**cfg["scene"])
    nodes, tris, box = tg.KDTree.from_mesh(m).export()
    sc = orc.Scene(nodes, tris, box)
    img, st = sc.render(m.camera, m.light, cfg["w"], cfg["h"], cfg["spp"], cfg["depth"], seed=cfg["seed"],
                        exposure=cfg.get("exposure", 1.0), gamma=cfg.get("gamma", True),
                        background=cfg.get("background", (0.0, 0.0, 0.0)), renderer=cfg.get("renderer", 0),
                        shadow_intensity=cfg.get("shadow", 0.5), max_visibility=cfg.get("max_visibility", 2.0))
    gold = renders[f"{name}_image"]
    assert int(st[0]) == int(renders[f"{name}_rays"])
    assert int(st[1]) == int(renders[f"{name}_primary"])
    if X86:
        assert np.array_equal(bits(img), bits(gold))
        p3 = orc.write_p3(img)
        assert hashlib.sha256(p3.encode()).hexdigest() == str(renders[f"{name}_p3_sha"])
    else:
        assert np.abs(img - gold).max() <= 1e-6


# --------------------------------------------------- tests/test_raster.cpp
P3_2X2 = "P3\n2 2\n255\n  0   0   0   0   0   0\n255 255 255   0   0   0"


def test_p3_golden():
    """test_raster.cpp:44-57: exact P3 text of a 2x2 image."""
    img = np.zeros((2, 2, 4), np.float32)
    img[1, 0] = (1, 1, 1, 1)
    assert orc.write_p3(img) == P3_2X2
    assert tg.write_p3(img) == P3_2X2


def test_p3_clamps_and_alpha():
    img = np.array([[[2.0, -1.0, 0.5, 1.0], [1.0, 1.0, 1.0, 0.5]]], np.float32)
    assert orc.write_p3(img) == tg.write_p3(img) == "P3\n2 1\n255\n255   0 127 127 127 127"


# --------------------------------------------------- tests/test_effects.cpp
def test_exposure_and_gamma():
    """test_effects.cpp:4-72: zero exposure is dark, alpha kept; exposure and
    gamma move light in the documented direction."""
    c = np.array([[0.5, 0.5, 0.5, 1.0]], np.float32)
    assert orc.tone(c, 0.0, 1.0, gamma=False).tolist() == [[0, 0, 0, 1]]
    assert orc.tone(c, 1.0, 1.0, gamma=False)[0, 0] < 0.5
    assert orc.tone(c, 10.0, 1.0, gamma=False)[0, 0] > 0.5
    g = orc.tone(np.array([[1 - math.exp(-1) * 0 + 0.0, 0, 0, 0.7]], np.float32), 1.0, 1 / 2.2)
    assert g[0, 3] == np.float32(0.7)


# ------------------------------------------------------------ RNG, sampling
def test_xorshift64star_floats():
    """lib/xorshift.h:27-70: x ^= x>>12; x ^= x<<25; x ^= x>>27; x * 2685821657736338717,
    float = (x & (2^24-1)) * 2^-24."""
    s = 42
    want = []
    for _ in range(8):
        s ^= s >> 12
        s ^= (s << 25) & 0xFFFFFFFFFFFFFFFF
        s ^= s >> 27
        x = (s * 2685821657736338717) & 0xFFFFFFFFFFFFFFFF
        want.append(np.float32((x & 0xFFFFFF) / 2 ** 24))
    assert orc.xorshift_floats(42, 8).tolist() == want


def test_from_to_rotation():
    """test_sampling.cpp:12-39: the rotation takes +z onto the normal and keeps
    sampled directions unit length with cos = dot(sample, normal)."""
    rng = np.random.default_rng(0)
    for v in list(rng.normal(size=(50, 3))) + [np.array([0, 0, 1.0]), np.array([0, 0, -1.0]),
                                                np.array([1e-7, 0, 1.0])]:
        n = (v / np.linalg.norm(v)).astype(np.float32)
        m = orc.from_to(n).astype(np.float64)
        assert np.allclose(m @ [0, 0, 1], n, atol=1e-5)
        assert np.allclose(m @ m.T, np.eye(3), atol=1e-5)
        u1, u2 = rng.uniform(size=2)
        rr = math.sqrt(max(0.0, 1 - u1 * u1))
        smp = np.array([rr * math.cos(2 * math.pi * u2), rr * math.sin(2 * math.pi * u2), u1])
        w = m @ smp
        assert abs(np.linalg.norm(w) - 1) < 0.01
        assert abs(np.dot(w, n) - u1) <= 0.01 * max(u1, 1e-3) + 1e-5
