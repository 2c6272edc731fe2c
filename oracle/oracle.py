"""ORACLE binding — test infrastructure only.

ctypes access to oracle/liboracle.so (the CPU restatement in oracle/oracle.cpp)
and, where it was built, oracle/_ref/libturner_ref.so (the reference's own
sources compiled by oracle/build_ref.sh). Only tests/, __graft_entry__.smoke()
and bench.py's CPU-baseline leg use this module, as the checker.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ORACLE_SO = HERE / "liboracle.so"
INPUTS_SO = HERE / "libinputs.so"
REF_SO = HERE / "_ref" / "libturner_ref.so"
MISS = 0x40000000
_P = C.c_void_p


class OrcCamera(C.Structure):
    _fields_ = [("position", C.c_float * 3), ("trafo", C.c_float * 9), ("delta_x", C.c_float),
                ("aspect", C.c_float)]


class OrcParams(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("pixel_samples", C.c_uint32),
                ("max_depth", C.c_int32), ("monte_carlo_samples", C.c_int32), ("exposure", C.c_float),
                ("inverse_gamma", C.c_float), ("gamma_correction", C.c_int32), ("background", C.c_float * 3),
                ("seed", C.c_uint64), ("n_lights", C.c_int32), ("light_position", C.c_float * 3),
                ("light_color", C.c_float * 4), ("sampling", C.c_int32), ("tone_map", C.c_int32),
                ("renderer", C.c_int32), ("shadow_intensity", C.c_float), ("max_visibility", C.c_float)]


class RefCamera(C.Structure):
    _fields_ = [("position", C.c_float * 3), ("trafo", C.c_float * 9), ("hfov", C.c_float),
                ("aspect", C.c_float)]


class RefParams(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("pixel_samples", C.c_uint32),
                ("max_depth", C.c_int32), ("monte_carlo_samples", C.c_int32), ("exposure", C.c_float),
                ("inverse_gamma", C.c_float), ("gamma_correction", C.c_int32), ("background", C.c_float * 3),
                ("seed", C.c_uint64), ("n_lights", C.c_int32), ("light_position", C.c_float * 3),
                ("light_color", C.c_float * 4), ("threads", C.c_int32), ("renderer", C.c_int32),
                ("shadow_intensity", C.c_float), ("max_visibility", C.c_float)]


_ORC = None
_REF = None


def build_oracle() -> None:
    """Compiles liboracle.so if it is missing (g++, no GPU needed)."""
    if ORACLE_SO.exists():
        return
    import subprocess
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-o", str(ORACLE_SO),
                    str(HERE / "oracle.cpp"), "-lpthread"], check=True)


def lib() -> C.CDLL:
    global _ORC
    if _ORC is None:
        build_oracle()
        L = C.CDLL(str(ORACLE_SO))
        L.orc_scene_create.restype = _P
        L.orc_scene_create.argtypes = [_P, C.c_uint64, _P, C.c_uint64, _P]
        L.orc_scene_free.argtypes = [_P]
        L.orc_intersect.argtypes = [_P, _P, C.c_uint64] + [_P] * 5 + [C.c_int]
        L.orc_render.argtypes = [_P, C.POINTER(OrcCamera), C.POINTER(OrcParams), _P, _P, C.c_int, C.c_uint32,
                                 C.c_uint32, C.c_uint32]
        L.orc_write_p3.restype = C.c_uint64
        L.orc_write_p3.argtypes = [_P, C.c_uint32, C.c_uint32, _P, C.c_uint64]
        L.orc_xorshift_floats.argtypes = [C.c_uint64, C.c_uint64, _P]
        L.orc_from_to.argtypes = [_P, _P]
        L.orc_ray_box.restype = C.c_int
        L.orc_ray_box.argtypes = [_P, _P, _P]
        L.orc_tone.argtypes = [_P, C.c_uint64, C.c_float, C.c_float, C.c_int, _P]
        _ORC = L
    return _ORC


class InputCamera(C.Structure):
    _fields_ = [("position", C.c_float * 3), ("trafo", C.c_float * 9), ("delta_x", C.c_float),
                ("aspect", C.c_float)]


class InputLight(C.Structure):
    _fields_ = [("position", C.c_float * 3), ("color", C.c_float * 4)]


class SceneInputs:
    """Input of the CPU reference arm: a seeded synthetic scene and the
    reference's kd-tree on it (node words identical to KDTree's, pinned by
    tests/test_builder.py), from oracle/libinputs.so, which holds only the
    host scene generator and builder (no CUDA). Fields: camera, light (or
    None), nodes, tris (n, 48), box, n_triangles."""

    def __init__(self, kind: int, detail: int = 0, count: int = 0, seed: int = 1, aspect: float = 1.0):
        L = C.CDLL(str(INPUTS_SO))
        L.turner_scene_make.argtypes = [C.c_int, C.c_uint32, C.c_uint32, C.c_uint64, C.c_float, C.POINTER(_P)]
        L.turner_mesh_num_triangles.restype = C.c_uint32
        L.turner_mesh_num_triangles.argtypes = [_P]
        for f in ("turner_mesh_vertices", "turner_mesh_normals", "turner_mesh_diffuse"):
            getattr(L, f).restype = _P
            getattr(L, f).argtypes = [_P]
        L.turner_mesh_camera.argtypes = [_P, C.POINTER(InputCamera), C.POINTER(C.c_float)]
        L.turner_mesh_light.argtypes = [_P, C.POINTER(InputLight)]
        L.turner_mesh_free.argtypes = [_P]
        L.turner_kdtree_build.argtypes = [_P, _P, _P, C.c_uint32, C.c_int, C.POINTER(_P)]
        L.turner_kdtree_num_nodes.restype = C.c_uint32
        L.turner_kdtree_num_nodes.argtypes = [_P]
        L.turner_kdtree_export.argtypes = [_P] * 4
        L.turner_kdtree_free.argtypes = [_P]
        mesh = _P()
        if L.turner_scene_make(kind, detail, count, seed, aspect, C.byref(mesh)) != 0:
            raise RuntimeError("turner_scene_make failed")
        try:
            n = L.turner_mesh_num_triangles(mesh)
            self.camera = InputCamera()
            hfov = C.c_float()
            L.turner_mesh_camera(mesh, C.byref(self.camera), C.byref(hfov))
            light = InputLight()
            self.light = light if L.turner_mesh_light(mesh, C.byref(light)) > 0 else None
            tree = _P()
            if L.turner_kdtree_build(L.turner_mesh_vertices(mesh), L.turner_mesh_normals(mesh),
                                     L.turner_mesh_diffuse(mesh), n, 0, C.byref(tree)) != 0:
                raise RuntimeError("turner_kdtree_build failed")
        finally:
            L.turner_mesh_free(mesh)
        try:
            self.nodes = np.empty(L.turner_kdtree_num_nodes(tree), np.uint64)
            self.tris = np.empty((n, 48), np.float32)
            self.box = np.empty(6, np.float32)
            L.turner_kdtree_export(tree, _ptr(self.nodes), _ptr(self.tris), _ptr(self.box))
        finally:
            L.turner_kdtree_free(tree)
        self.n_triangles = int(n)


def ref_available() -> bool:
    return REF_SO.exists()


def ref_lib() -> C.CDLL:
    global _REF
    if _REF is None:
        L = C.CDLL(str(REF_SO))
        L.ref_tree_build.restype = _P
        L.ref_tree_build.argtypes = [_P, _P, _P, C.c_uint32, _P]
        L.ref_tree_free.argtypes = [_P]
        for f in ("ref_tree_num_nodes", "ref_tree_height", "ref_tree_num_triangles"):
            getattr(L, f).restype = C.c_uint64
            getattr(L, f).argtypes = [_P]
        L.ref_tree_export.argtypes = [_P] * 4
        L.ref_intersect.argtypes = [_P, _P, C.c_uint64] + [_P] * 4 + [C.c_int]
        L.ref_camera_delta_x.restype = C.c_float
        L.ref_camera_delta_x.argtypes = [C.c_float, C.c_float]
        L.ref_render.argtypes = [_P, C.POINTER(RefCamera), C.POINTER(RefParams), _P, _P]
        L.ref_write_p3.restype = C.c_uint64
        L.ref_write_p3.argtypes = [_P, C.c_uint32, C.c_uint32, _P, C.c_uint64]
        _REF = L
    return _REF


def _ptr(a):
    return None if a is None else a.ctypes.data


class Scene:
    """Oracle scene: FlatNode words, 48-float triangle records, box."""

    def __init__(self, nodes: np.ndarray, tris: np.ndarray, box: np.ndarray):
        self.nodes = np.ascontiguousarray(nodes, np.uint64)
        self.tris = np.ascontiguousarray(tris, np.float32).reshape(-1, 48)
        self.box = np.ascontiguousarray(box, np.float32)
        self._h = lib().orc_scene_create(_ptr(self.nodes), self.nodes.size, _ptr(self.tris), self.tris.shape[0],
                                         _ptr(self.box))

    def __del__(self):
        if getattr(self, "_h", None) and _ORC is not None:
            _ORC.orc_scene_free(self._h)
            self._h = None

    def intersect(self, o: np.ndarray, d: np.ndarray, threads: int = 0, counts: bool = False):
        """o, d: (3, n). Returns id, r, s, t (and [node visits, triangle tests])."""
        rays = np.ascontiguousarray(np.concatenate([o, d], 0).T, np.float32)
        n = rays.shape[0]
        hid = np.empty(n, np.uint32)
        r = np.empty(n, np.float32)
        s = np.empty(n, np.float32)
        t = np.empty(n, np.float32)
        cnt = np.zeros(2, np.uint64)
        lib().orc_intersect(self._h, _ptr(rays), n, _ptr(hid), _ptr(r), _ptr(s), _ptr(t), _ptr(cnt),
                            threads or os.cpu_count())
        return (hid, r, s, t, cnt) if counts else (hid, r, s, t)

    def render(self, camera, light, width: int, height: int, spp: int, max_depth: int, mc: int = 1,
               seed: int = 1, exposure: float = 1.0, inverse_gamma: float = 0.454545, gamma: bool = True,
               background=(0.0, 0.0, 0.0), sampling: int = 0, tone_map: bool = True, threads: int = 0,
               rows: tuple[int, int] | None = None, renderer: int = 0, shadow_intensity: float = 0.5,
               max_visibility: float = 2.0, row_step: int = 1):
        """Returns (image (h, w, 4) float32, stats [rays, primary, shadow, closest-hit node visits,
        closest-hit triangle tests, shadow node visits, shadow triangle tests]).
        renderer: 0 path tracer, 1 Whitted raytracer, 2 raycaster. rows=(a, b)
        with row_step k renders rows a, a + k, a + 2k, ... below b (the
        other rows stay zero); threads take one row at a time."""
        cam = OrcCamera()
        cam.position[:] = list(camera.position)
        cam.trafo[:] = list(camera.trafo)
        cam.delta_x = camera.delta_x
        cam.aspect = camera.aspect
        p = OrcParams()
        p.width, p.height, p.pixel_samples = width, height, spp
        p.max_depth, p.monte_carlo_samples = max_depth, mc
        p.exposure = exposure
        p.inverse_gamma = np.float32(inverse_gamma)
        p.gamma_correction = 1 if gamma else 0
        p.background[:] = list(background)
        p.seed = seed
        p.n_lights = 1 if light is not None else 0
        if light is not None:
            p.light_position[:] = list(light.position)
            p.light_color[:] = list(light.color)
        p.sampling = sampling
        p.tone_map = 1 if tone_map else 0
        p.renderer = renderer
        p.shadow_intensity = shadow_intensity
        p.max_visibility = max_visibility
        img = np.zeros((height, width, 4), np.float32)
        stats = np.zeros(7, np.uint64)
        r0, r1 = rows if rows else (0, 0)
        lib().orc_render(self._h, C.byref(cam), C.byref(p), _ptr(img), _ptr(stats), threads or os.cpu_count(),
                         r0, r1, row_step)
        return img, stats


def write_p3(rgba: np.ndarray) -> str:
    a = np.ascontiguousarray(rgba, np.float32)
    h, w = a.shape[:2]
    n = lib().orc_write_p3(_ptr(a), w, h, None, 0)
    buf = C.create_string_buffer(n)
    lib().orc_write_p3(_ptr(a), w, h, buf, n)
    return buf.raw[:n].decode()


def xorshift_floats(seed: int, n: int) -> np.ndarray:
    out = np.empty(n, np.float32)
    lib().orc_xorshift_floats(seed, n, _ptr(out))
    return out


def from_to(n3) -> np.ndarray:
    a = np.asarray(n3, np.float32)
    m = np.empty(9, np.float32)
    lib().orc_from_to(_ptr(a), _ptr(m))
    return m.reshape(3, 3)


def ray_box(ray6, box6):
    r = np.asarray(ray6, np.float32)
    b = np.asarray(box6, np.float32)
    t = np.empty(2, np.float32)
    hit = lib().orc_ray_box(_ptr(r), _ptr(b), _ptr(t))
    return bool(hit), t


def tone(rgba: np.ndarray, exposure: float, inverse_gamma: float, gamma: bool = True) -> np.ndarray:
    a = np.ascontiguousarray(rgba, np.float32)
    out = np.empty_like(a)
    lib().orc_tone(_ptr(a), a.size // 4, exposure, inverse_gamma, 1 if gamma else 0, _ptr(out))
    return out


# ----------------------------------------------------------- reference
class RefTree:
    """The reference's KDTree built by oracle/_ref (checker only)."""

    def __init__(self, vertices: np.ndarray, normals=None, diffuse=None, reflective=None):
        v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 9)
        self.n = v.shape[0]
        nr = None if normals is None else np.ascontiguousarray(normals, np.float32).reshape(-1, 9)
        d = None if diffuse is None else np.ascontiguousarray(diffuse, np.float32).reshape(-1, 4)
        rf = None if reflective is None else np.ascontiguousarray(reflective, np.float32).reshape(-1, 5)
        self._keep = (v, nr, d, rf)
        self._h = ref_lib().ref_tree_build(_ptr(v), _ptr(nr), _ptr(d), self.n, _ptr(rf))

    def __del__(self):
        if getattr(self, "_h", None) and _REF is not None:
            _REF.ref_tree_free(self._h)
            self._h = None

    def height(self) -> int:
        return ref_lib().ref_tree_height(self._h)

    def num_nodes(self) -> int:
        return ref_lib().ref_tree_num_nodes(self._h)

    def export(self):
        nodes = np.empty(self.num_nodes(), np.uint64)
        tris = np.empty((self.n, 48), np.float32)
        box = np.empty(6, np.float32)
        ref_lib().ref_tree_export(self._h, _ptr(nodes), _ptr(tris), _ptr(box))
        return nodes, tris, box

    def intersect(self, o: np.ndarray, d: np.ndarray, threads: int = 0):
        rays = np.ascontiguousarray(np.concatenate([o, d], 0).T, np.float32)
        n = rays.shape[0]
        hid = np.empty(n, np.uint32)
        r = np.empty(n, np.float32)
        s = np.empty(n, np.float32)
        t = np.empty(n, np.float32)
        ref_lib().ref_intersect(self._h, _ptr(rays), n, _ptr(hid), _ptr(r), _ptr(s), _ptr(t), threads or os.cpu_count())
        return hid, r, s, t

    def render(self, position, trafo, hfov, aspect, light, width, height, spp, max_depth, mc=1, seed=1,
               exposure=1.0, inverse_gamma=0.454545, gamma=True, background=(0.0, 0.0, 0.0), threads=0,
               renderer=0, shadow_intensity=0.5, max_visibility=2.0):
        """renderer: 0 pathtracer.cpp, 1 raytracer.cpp, 2 raycaster.cpp."""
        cam = RefCamera()
        cam.position[:] = list(position)
        cam.trafo[:] = list(trafo)
        cam.hfov = hfov
        cam.aspect = aspect
        p = RefParams()
        p.width, p.height, p.pixel_samples = width, height, spp
        p.max_depth, p.monte_carlo_samples = max_depth, mc
        p.exposure = exposure
        p.inverse_gamma = np.float32(inverse_gamma)
        p.gamma_correction = 1 if gamma else 0
        p.background[:] = list(background)
        p.seed = seed
        p.n_lights = 1 if light is not None else 0
        if light is not None:
            p.light_position[:] = list(light.position)
            p.light_color[:] = list(light.color)
        p.threads = threads or os.cpu_count()
        p.renderer = renderer
        p.shadow_intensity = shadow_intensity
        p.max_visibility = max_visibility
        img = np.zeros((height, width, 4), np.float32)
        stats = np.zeros(2, np.uint64)
        ref_lib().ref_render(self._h, C.byref(cam), C.byref(p), _ptr(img), _ptr(stats))
        return img, stats


def ref_delta_x(hfov: float, aspect: float) -> float:
    return ref_lib().ref_camera_delta_x(hfov, aspect)


def ref_write_p3(rgba: np.ndarray) -> str:
    a = np.ascontiguousarray(rgba, np.float32)
    h, w = a.shape[:2]
    n = ref_lib().ref_write_p3(_ptr(a), w, h, None, 0)
    buf = C.create_string_buffer(int(n))
    ref_lib().ref_write_p3(_ptr(a), w, h, buf, n)
    return buf.raw[:n].decode()
