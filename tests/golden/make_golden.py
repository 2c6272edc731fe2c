"""Writes the golden fixtures in tests/golden/ from the reference itself.

Run where the reference sources exist (they are compiled into
oracle/_ref/libturner_ref.so by oracle/build_ref.sh):

    python tests/golden/make_golden.py

Everything recorded here comes out of the reference's own code: its kd-tree
builder and traversal (lib/kdtree.cpp), trace() (pathtracer.cpp), camera
(lib/types.h), tone map (lib/effects.h), P3 writer (lib/raster.h) and test
fixtures (tests/helper.h). Scene geometry comes from the product's seeded
generators (turner_gb300), which only supply inputs.
"""
from __future__ import annotations

import hashlib
import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

import turner_gb300 as tg  # noqa: E402
from oracle import oracle as orc  # noqa: E402


def sha(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def ref_hfov(mesh) -> np.float32:
    """An hfov for which the reference's Camera derives exactly our delta_x."""
    hf = np.float32(mesh.hfov)
    for c in (hf, np.nextafter(hf, np.float32(1)), np.nextafter(hf, np.float32(0)),
              np.nextafter(np.nextafter(hf, np.float32(1)), np.float32(1)),
              np.nextafter(np.nextafter(hf, np.float32(0)), np.float32(0))):
        if np.float32(orc.ref_delta_x(c, mesh.camera.aspect)) == np.float32(mesh.camera.delta_x):
            return c
    raise RuntimeError("no hfov reproduces delta_x")


SCENES = {
    "room": dict(kind=tg.SCENE_ROOM),
    "sphere3": dict(kind=tg.SCENE_SPHERE_ROOM, detail=3),
    "soup2000": dict(kind=tg.SCENE_SOUP, count=2000, seed=7),
    "baffle8": dict(kind=tg.SCENE_BAFFLE_ROOM, detail=8),
    "mirror": dict(kind=tg.SCENE_MIRROR_ROOM),
}


def kdtree_tests() -> None:
    """The reference's kd-tree unit tests (tests/test_kdtree.cpp), recorded."""
    out = {}
    tri = lambda *p: np.array(p, np.float32).reshape(9)  # noqa: E731
    four = np.stack([tri(0, 0, 1, 0, 1, 1, 1, 0, 1), tri(2, 0, 1, 3, 0, 1, 3, 1, 1),
                     tri(0, 2, 1, 0, 3, 1, 1, 3, 1), tri(3, 2, 1, 3, 3, 1, 2, 3, 1)])
    cube = np.stack([
        tri(-1, -1, -1, 1, -1, -1, 1, 1, -1), tri(-1, -1, -1, -1, 1, -1, 1, 1, -1),
        tri(-1, -1, 1, 1, -1, 1, 1, 1, 1), tri(-1, -1, 1, -1, 1, 1, 1, 1, 1),
        tri(-1, -1, -1, -1, -1, 1, -1, 1, 1), tri(-1, -1, -1, -1, 1, -1, -1, 1, 1),
        tri(1, -1, -1, 1, -1, 1, 1, 1, 1), tri(1, -1, -1, 1, 1, -1, 1, 1, 1),
        tri(-1, 1, -1, -1, 1, 1, 1, 1, 1), tri(-1, 1, -1, 1, 1, -1, 1, 1, 1),
        tri(-1, -1, -1, -1, -1, 1, 1, -1, 1), tri(-1, -1, -1, 1, -1, -1, 1, -1, 1)])
    overlap = np.stack([tri(-1, -1, 0, 1, -1, 0, 1, 1, 0), tri(0, 0, 0, 1, 0, 0, 1, 2, 0)])
    lib = orc.ref_lib()
    import ctypes as C
    lib.ref_fixture_coplanar.argtypes = [C.c_void_p, C.c_void_p]
    lib.ref_fixture_stacked.argtypes = [C.c_void_p]
    coplanar = np.zeros((3, 1000, 9), np.float32)
    dirs = np.zeros((3, 3), np.float32)
    lib.ref_fixture_coplanar(coplanar.ctypes.data, dirs.ctypes.data)
    stacked = np.zeros((3, 10, 9), np.float32)
    lib.ref_fixture_stacked(stacked.ctypes.data)

    for name, verts in (("four", four), ("cube", cube), ("overlap", overlap)):
        t = orc.RefTree(verts)
        nodes, tris, box = t.export()
        out[f"{name}_vertices"] = verts
        out[f"{name}_nodes"] = nodes
        out[f"{name}_tris"] = tris
        out[f"{name}_box"] = box
        out[f"{name}_height"] = np.int64(t.height())
    # rays of "Four separated triangles" (test_kdtree.cpp:34-62)
    o = np.zeros((3, 4), np.float32)
    d = np.array([[0.5, 2.5, 0.5, 2.5], [0.5, 0.5, 2.5, 2.5], [1, 1, 1, 1]], np.float32)
    res = orc.RefTree(four).intersect(o, d, threads=1)
    out["four_rays_o"], out["four_rays_d"] = o, d
    for k, v in zip("irst", res):
        out[f"four_hit_{k}"] = v

    for a in range(3):
        verts = coplanar[a]
        t = orc.RefTree(verts)
        nodes, tris, box = t.export()
        ro = np.array([[1, -1], [1, -1], [1, -1]], np.float32)   # parallel ray, ray through zero
        rd = np.stack([dirs[a], np.array([1, 1, 1], np.float32)], 1)
        res = t.intersect(ro, rd, threads=1)
        out[f"coplanar{a}_vertices"] = verts
        out[f"coplanar{a}_nodes"] = nodes
        out[f"coplanar{a}_tris"] = tris
        out[f"coplanar{a}_box"] = box
        out[f"coplanar{a}_rays_o"], out[f"coplanar{a}_rays_d"] = ro, rd
        for k, v in zip("irst", res):
            out[f"coplanar{a}_hit_{k}"] = v

        verts = stacked[a]
        t = orc.RefTree(verts)
        nodes, tris, box = t.export()
        ro = np.zeros((3, 2), np.float32)
        rd = np.zeros((3, 2), np.float32)
        ro[a] = [-100, 100]
        rd[a] = [1, -1]
        res = t.intersect(ro, rd, threads=1)
        out[f"stacked{a}_vertices"] = verts
        out[f"stacked{a}_nodes"] = nodes
        out[f"stacked{a}_tris"] = tris
        out[f"stacked{a}_box"] = box
        out[f"stacked{a}_rays_o"], out[f"stacked{a}_rays_d"] = ro, rd
        for k, v in zip("irst", res):
            out[f"stacked{a}_hit_{k}"] = v
    np.savez_compressed(HERE / "ref_kdtree_tests.npz", **out)


def scenes() -> None:
    out = {}
    for name, kw in SCENES.items():
        m = tg.make_scene(**kw)
        t = orc.RefTree(m.vertices, m.normals, m.diffuse, m.reflective)
        nodes, tris, box = t.export()
        out[f"{name}_nodes_sha"] = np.array(sha(nodes))
        out[f"{name}_tris_sha"] = np.array(sha(tris))
        out[f"{name}_box"] = box
        out[f"{name}_height"] = np.int64(t.height())
        out[f"{name}_num_nodes"] = np.int64(nodes.size)
        o, d = tg.make_rays(8192, box, seed=101)
        # a few rays with zero direction components exercise fix_direction
        d[0, ::17] = 0
        d[1, ::23] = 0
        # ... and some start exactly on a triangle vertex
        idx = np.arange(0, o.shape[1], 29)
        o[:, idx] = m.vertices[idx % m.n_triangles, :3].T
        hid, r, s, tt = t.intersect(o, d)
        out[f"{name}_rays_o"], out[f"{name}_rays_d"] = o, d
        out[f"{name}_hit_i"], out[f"{name}_hit_r"], out[f"{name}_hit_s"], out[f"{name}_hit_t"] = hid, r, s, tt
    # the full-size mesh: tree identity only
    m = tg.make_scene(tg.SCENE_SPHERE_ROOM, detail=7, aspect=16 / 9)
    t = orc.RefTree(m.vertices, m.normals, m.diffuse)
    nodes, tris, box = t.export()
    out["sphere7_nodes_sha"] = np.array(sha(nodes))
    out["sphere7_tris_sha"] = np.array(sha(tris))
    out["sphere7_box"] = box
    out["sphere7_height"] = np.int64(t.height())
    out["sphere7_num_nodes"] = np.int64(nodes.size)
    np.savez_compressed(HERE / "ref_scenes.npz", **out)


RENDERS = {
    "room_48": dict(scene="room", w=48, h=48, spp=4, depth=3, seed=7),
    "room_bg_nogamma": dict(scene="room", w=40, h=40, spp=2, depth=2, seed=9, background=(0.2, 0.3, 0.4),
                            gamma=False, exposure=0.5),
    "sphere3_32": dict(scene="sphere3", w=32, h=24, spp=2, depth=3, seed=11),
    "room_depth0": dict(scene="room", w=24, h=24, spp=1, depth=0, seed=3),
    "baffle8_32": dict(scene="baffle8", w=32, h=32, spp=2, depth=4, seed=5),
    # raytracer.cpp (renderer 1) and raycaster.cpp (renderer 2)
    "mirror_raytrace": dict(scene="mirror", w=48, h=48, spp=1, depth=3, seed=13, renderer=1),
    "mirror_raytrace_d1_shadow08": dict(scene="mirror", w=40, h=32, spp=2, depth=1, seed=17, renderer=1,
                                        shadow=0.8, background=(0.1, 0.2, 0.3)),
    "room_raytrace": dict(scene="room", w=32, h=32, spp=1, depth=3, seed=19, renderer=1),
    "room_raycast": dict(scene="room", w=40, h=40, spp=2, depth=3, seed=23, renderer=2, max_visibility=6.0),
    "sphere3_raycast_default": dict(scene="sphere3", w=32, h=24, spp=1, depth=3, seed=29, renderer=2),
}


def renders() -> None:
    out = {}
    for name, cfg in RENDERS.items():
        m = tg.make_scene(**SCENES[cfg["scene"]])
        t = orc.RefTree(m.vertices, m.normals, m.diffuse, m.reflective)
        img, st = t.render(m.camera.position, m.camera.trafo, ref_hfov(m), m.camera.aspect, m.light, cfg["w"],
                           cfg["h"], cfg["spp"], cfg["depth"], seed=cfg["seed"],
                           exposure=cfg.get("exposure", 1.0), gamma=cfg.get("gamma", True),
                           background=cfg.get("background", (0.0, 0.0, 0.0)), renderer=cfg.get("renderer", 0),
                           shadow_intensity=cfg.get("shadow", 0.5), max_visibility=cfg.get("max_visibility", 2.0))
        out[f"{name}_image"] = img
        out[f"{name}_rays"] = st[0]
        out[f"{name}_primary"] = st[1]
        out[f"{name}_p3_sha"] = np.array(hashlib.sha256(orc.ref_write_p3(img).encode()).hexdigest())
    np.savez_compressed(HERE / "ref_renders.npz", **out)


if __name__ == "__main__":
    if not orc.ref_available():
        subprocess.run(["bash", str(ROOT / "oracle" / "build_ref.sh")], check=True)
    kdtree_tests()
    scenes()
    renders()
    for f in sorted(HERE.glob("*.npz")):
        print(f.name, f.stat().st_size)
