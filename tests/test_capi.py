"""The C ABI library: loads, exports every declared symbol, host-side calls."""
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

import turner_gb300 as tg

ROOT = Path(__file__).resolve().parent.parent


def declared_symbols():
    text = (ROOT / "include" / "turner_gpu.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(turner_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    out = subprocess.run(["nm", "-D", "--defined-only", str(tg.LIB_PATH)], capture_output=True, text=True,
                         check=True).stdout
    exported = set(re.findall(r"\bT (turner_\w+)", out))
    missing = [s for s in declared_symbols() if s not in exported]
    assert not missing, missing
    assert len(declared_symbols()) >= 30


def test_library_loads_and_binds():
    lib = tg._lib()
    for s in declared_symbols():
        assert hasattr(lib, s)


def test_strerror_covers_all_codes():
    lib = tg._lib()
    for code in range(0, -10, -1):
        assert lib.turner_strerror(code).decode() not in ("", "unknown status")
    assert lib.turner_strerror(-99).decode() == "unknown status"


def test_scene_generators_are_deterministic():
    a = tg.make_scene(tg.SCENE_SPHERE_ROOM, detail=3, seed=5)
    b = tg.make_scene(tg.SCENE_SPHERE_ROOM, detail=3, seed=5)
    c = tg.make_scene(tg.SCENE_SPHERE_ROOM, detail=3, seed=6)
    assert np.array_equal(a.vertices, b.vertices) and not np.array_equal(a.vertices, c.vertices)
    assert a.n_triangles == 12 + 20 * 4 ** 3
    room = tg.make_scene(tg.SCENE_ROOM)
    assert room.n_triangles == 36
    assert tg.make_scene(tg.SCENE_BAFFLE_ROOM, detail=64).n_triangles == 5 * 2 * 64 * 64 + 24 + 2 + 12
    assert tg.make_scene(tg.SCENE_SOUP, count=1000, seed=3).n_triangles == 1012
    n = room.normals.reshape(-1, 3)
    assert np.allclose(np.linalg.norm(n, axis=1), 1, atol=1e-6)


def test_camera_conventions():
    m = tg.make_scene(tg.SCENE_ROOM, aspect=16 / 9)
    assert np.float32(m.camera.delta_x) == np.float32(0.36397023426620236 * (16 / 9))
    assert np.isclose(np.tan(m.hfov), m.camera.delta_x, rtol=1e-6)
    assert list(m.camera.trafo) == [1, 0, 0, 0, 1, 0, 0, 0, 1]
    assert m.light is not None and list(m.light.color) == [50, 50, 50, 1]


def test_make_rays_unit_and_deterministic():
    box = np.array([0, 0, -5.56, 5.56, 5.56, 0], np.float32)
    o, d = tg.make_rays(10000, box, seed=3)
    o2, d2 = tg.make_rays(10000, box, seed=3)
    assert np.array_equal(o, o2) and np.array_equal(d, d2)
    assert np.allclose(np.linalg.norm(d, axis=0), 1, atol=1e-6)
    assert (o >= box[:3, None]).all() and (o <= box[3:, None]).all()
    assert abs(d.mean()) < 0.05


def test_invalid_arguments_are_rejected_without_device():
    lib = tg._lib()
    import ctypes as C
    h = C.c_void_p()
    assert lib.turner_scene_make(99, 0, 0, 1, 1.0, C.byref(h)) == tg.ERR_INVALID_ARG
    assert lib.turner_scene_make(tg.SCENE_ROOM, 0, 0, 1, -1.0, C.byref(h)) == tg.ERR_INVALID_ARG
    assert lib.turner_scene_make(tg.SCENE_SPHERE_ROOM, 12, 0, 1, 1.0, C.byref(h)) == tg.ERR_TOO_LARGE
    assert lib.turner_create(None, 0) == tg.ERR_INVALID_ARG
    assert lib.turner_kdtree_build(None, None, None, 3, 0, C.byref(h)) == tg.ERR_INVALID_ARG


def test_create_without_gpu_reports_no_device():
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    with pytest.raises(tg.TurnerError) as e:
        tg.Context(0)
    assert e.value.status == tg.ERR_NO_DEVICE


def test_cli_help_and_flag_errors():
    cli = tg.LIB_DIR / "turner_pathtracer"
    r = subprocess.run([str(cli), "--help"], capture_output=True, text=True)
    assert r.returncode == 0 and "--monte-carlo-samples" in r.stderr and "--pixel-samples" in r.stderr
    r = subprocess.run([str(cli), "room", "--bogus"], capture_output=True, text=True)
    assert r.returncode == 1
    r = subprocess.run([str(cli), "room", "-d", "0"], capture_output=True, text=True)   # TracerConfig::check
    assert r.returncode == 1
    # a tree file is keyed by the triangles alone: GPU-built trees stay out of the cache
    r = subprocess.run([str(cli), "room", "--gpu-kdtree", "--kdtree-cache", "/nonexistent"], capture_output=True,
                       text=True)
    assert r.returncode == 1 and "--gpu-kdtree" in r.stderr
