"""Python mirror of the GB300 path-tracing core's C ABI (include/turner_gpu.h).

The native library turner_gb300/lib/libturner_gb300.so is the product; this
module only binds it with ctypes. There is no Python or CPU fallback: if the
library is missing or the GPU is not an sm_103 device, calls raise.

Names follow the reference (turner-renderer/turner): a `KDTree` is built from
triangles and uploaded as a scene; `Context.intersect` is the batched
`KDTreeIntersection::intersect` (lib/kdtree.cpp:516-607); `Context.render` is
the `pathtracer` render loop (main.cpp:181-236 around pathtracer.cpp:14-102).
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

LIB_DIR = Path(__file__).resolve().parent / "lib"
LIB_PATH = LIB_DIR / "libturner_gb300.so"

OK = 0
ERR_INVALID_ARG = -1
ERR_CUDA = -2
ERR_OUT_OF_MEMORY = -3
ERR_BAD_SCENE = -4
ERR_TIMEOUT = -5
ERR_DEVICE_BOUNDS = -6
ERR_UNSUPPORTED = -7
ERR_NO_DEVICE = -8
ERR_TOO_LARGE = -9

MISS = 0x40000000
HOST_BUFFERS = 0
DEVICE_BUFFERS = 1
TRAVERSAL_PARITY = 0
TRAVERSAL_FAST = 1
SAMPLING_UNIFORM = 0
SAMPLING_COSINE = 1
SAMPLING_GUIDED = 2

SCENE_ROOM = 0
SCENE_SPHERE_ROOM = 1
SCENE_SOUP = 2
SCENE_BAFFLE_ROOM = 3
SCENE_BAFFLE_SPHERE = 4
SCENE_MIRROR_ROOM = 5

TRIANGLE_FLOATS = 48  # turner_triangle: Triangle::serialize order

GRAPH_AUTO, GRAPH_ALWAYS, GRAPH_NEVER = 0, 1, 2
RAYS_PRIMARY, RAYS_BOUNCE, RAYS_SHADOW_PRIMARY, RAYS_SHADOW, RAYS_INTERSECT = 0, 1, 2, 3, 4
PACKET_CAMERA, PACKET_BATCHED = 1, 2
RENDERER_PATH, RENDERER_RAYTRACE, RENDERER_RAYCAST = 0, 1, 2
KERNEL_NAMES = ("k_camera", "k_trace", "k_shade", "k_shadow", "k_resolve", "k_intersect", "k_guide_features",
                "k_mlp_forward", "guide_train")
KERNEL_KINDS = len(KERNEL_NAMES)


class TurnerError(RuntimeError):
    def __init__(self, status: int, what: str = ""):
        self.status = status
        msg = _lib().turner_strerror(status).decode() if _LIB is not None else str(status)
        super().__init__(f"{what}: {msg} ({status})" if what else f"{msg} ({status})")


class Camera(C.Structure):
    _fields_ = [("position", C.c_float * 3), ("trafo", C.c_float * 9), ("delta_x", C.c_float),
                ("aspect", C.c_float)]


class Light(C.Structure):
    _fields_ = [("position", C.c_float * 3), ("color", C.c_float * 4)]


class Job(C.Structure):
    _fields_ = [("scene_id", C.c_uint32), ("width", C.c_uint32), ("height", C.c_uint32),
                ("pixel_samples", C.c_uint32), ("max_depth", C.c_int32), ("monte_carlo_samples", C.c_int32),
                ("exposure", C.c_float), ("inverse_gamma", C.c_float), ("gamma_correction", C.c_int32),
                ("background", C.c_float * 3), ("seed", C.c_uint64), ("n_lights", C.c_int32),
                ("light", Light), ("camera", Camera), ("sampling", C.c_int32), ("traversal", C.c_int32),
                ("linear_output", C.c_int32), ("renderer", C.c_int32), ("shadow_intensity", C.c_float),
                ("max_visibility", C.c_float), ("row_begin", C.c_uint32), ("row_end", C.c_uint32)]

    @property
    def rows(self) -> int:
        """Rows this job renders (its output's height): [row_begin, row_end)."""
        return (self.row_end or self.height) - self.row_begin


class Tuning(C.Structure):
    _fields_ = [("persistent", C.c_int32), ("blocks_per_sm", C.c_uint32), ("block", C.c_uint32),
                ("stack", C.c_uint32), ("chunk_paths", C.c_uint32), ("mailbox", C.c_uint32),
                ("min_blocks", C.c_uint32), ("ms", C.c_double), ("candidates", C.c_uint32),
                ("refill_camera", C.c_uint32), ("refill_bounce", C.c_uint32), ("packets", C.c_uint32)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class Stats(C.Structure):
    _fields_ = [("rays", C.c_uint64), ("primary_rays", C.c_uint64), ("shadow_rays", C.c_uint64),
                ("device_ms", C.c_double)]


_LIB = None
_P = C.c_void_p


def _lib() -> C.CDLL:
    """Loads the native library; raises if it has not been built."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not LIB_PATH.exists():
        raise ImportError(f"{LIB_PATH} is missing: run `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(str(LIB_PATH))
    sig = {
        "turner_strerror": (C.c_char_p, [C.c_int]),
        "turner_create": (C.c_int, [C.POINTER(_P), C.c_int]),
        "turner_destroy": (None, [_P]),
        "turner_last_device_error": (C.c_int, [_P]),
        "turner_last_error_message": (C.c_char_p, [_P]),
        "turner_launch_count": (C.c_uint64, [_P]),
        "turner_set_chunk_paths": (C.c_int, [_P, C.c_uint32]),
        "turner_set_profiling": (C.c_int, [_P, C.c_int]),
        "turner_set_graph_mode": (C.c_int, [_P, C.c_int]),
        "turner_autotune": (C.c_int, [_P, C.POINTER(Job), C.c_uint32, C.c_int, C.POINTER(Tuning)]),
        "turner_set_tuning": (C.c_int, [_P, C.POINTER(Tuning)]),
        "turner_guide_set_objective": (C.c_int, [_P, C.c_int]),
        "turner_get_tuning": (C.c_int, [_P, C.POINTER(Tuning)]),
        "turner_graph_launch_count": (C.c_uint64, [_P]),
        "turner_set_traversal_launch": (C.c_int, [_P, C.c_int, C.c_uint32]),
        "turner_set_traversal_refill": (C.c_int, [_P, C.c_int, C.c_uint32]),
        "turner_set_traversal_ring": (C.c_int, [_P, C.c_uint32]),
        "turner_set_traversal_speculative": (C.c_int, [_P, C.c_int]),
        "turner_set_traversal_packet": (C.c_int, [_P, C.c_int]),
        "turner_kernel_times": (C.c_int, [_P, _P, _P, C.c_int]),
        "turner_upload_scene": (C.c_int, [_P, _P, C.c_uint32, _P, C.c_uint32, _P, C.POINTER(C.c_uint32)]),
        "turner_free_scene": (C.c_int, [_P, C.c_uint32]),
        "turner_validate_nodes": (C.c_int, [_P, C.c_uint32, C.c_uint32, C.POINTER(C.c_uint32)]),
        "turner_intersect": (C.c_int, [_P, C.c_uint32] + [_P] * 6 + [C.c_uint64] + [_P] * 4 + [C.c_int, C.c_uint32]),
        "turner_probe_gather": (C.c_int, [_P, C.c_uint64, C.c_uint32, C.c_uint32, C.POINTER(C.c_double)]),
        "turner_occluded": (C.c_int, [_P, C.c_uint32] + [_P] * 7 + [C.c_uint64, _P, C.c_uint32]),
        "turner_intersect_noalloc": (C.c_int, [_P, C.c_uint32] + [_P] * 6 + [C.c_uint64] + [_P] * 4 + [C.c_int]),
        "turner_render": (C.c_int, [_P, C.POINTER(Job), C.c_uint32, C.POINTER(_P), C.POINTER(Stats), C.c_uint32]),
        "turner_render_accumulate": (C.c_int, [_P, C.POINTER(Job), C.c_uint32, _P, C.POINTER(C.c_uint64),
                                               C.c_uint32]),
        "turner_guide_create": (C.c_int, [_P, C.c_uint64, C.POINTER(_P)]),
        "turner_set_guide": (C.c_int, [_P, _P, C.c_int, C.c_float, C.c_uint32]),
        "turner_set_guide_steps": (C.c_int, [_P, C.c_uint32]),
        "turner_set_guide_depth": (C.c_int, [_P, C.c_uint32]),
        "turner_set_guide_weighting": (C.c_int, [_P, C.c_int]),
        "turner_guide_stats": (C.c_int, [_P, C.POINTER(C.c_uint64), C.POINTER(C.c_float), C.POINTER(C.c_double)]),
        "turner_guide_destroy": (None, [_P]),
        "turner_guide_params": (C.c_int, [_P, _P, C.c_int]),
        "turner_guide_forward": (C.c_int, [_P, _P, C.c_uint32, _P]),
        "turner_guide_gradient": (C.c_int, [_P, _P, _P, _P, C.c_uint32, _P, C.POINTER(C.c_float)]),
        "turner_guide_train": (C.c_int, [_P, _P, _P, _P, C.c_uint32, C.c_float, C.c_uint32, C.POINTER(C.c_float)]),
        "turner_kdtree_build": (C.c_int, [_P, _P, _P, C.c_uint32, C.c_int, C.POINTER(_P)]),
        "turner_kdtree_num_nodes": (C.c_uint32, [_P]),
        "turner_kdtree_num_triangles": (C.c_uint32, [_P]),
        "turner_kdtree_height": (C.c_uint32, [_P]),
        "turner_kdtree_export": (C.c_int, [_P, _P, _P, _P]),
        "turner_upload_kdtree": (C.c_int, [_P, _P, C.POINTER(C.c_uint32)]),
        "turner_kdtree_free": (None, [_P]),
        "turner_mesh_key": (C.c_uint64, [_P, _P, _P, C.c_uint32]),
        "turner_kdtree_build_gpu": (C.c_int, [_P, _P, _P, _P, C.c_uint32, C.POINTER(_P)]),
        "turner_kdtree_save": (C.c_int, [_P, C.c_uint64, C.c_char_p]),
        "turner_kdtree_load": (C.c_int, [C.c_char_p, C.c_uint64, C.POINTER(_P)]),
        "turner_kdtree_build_cached": (C.c_int, [_P, _P, _P, C.c_uint32, C.c_int, C.c_char_p, C.POINTER(_P),
                                                 C.POINTER(C.c_int)]),
        "turner_tree_file_map": (C.c_int, [C.c_char_p, C.c_uint64, C.c_int, C.POINTER(_P)]),
        "turner_tree_file_nodes": (_P, [_P, C.POINTER(C.c_uint32)]),
        "turner_tree_file_triangles": (_P, [_P, C.POINTER(C.c_uint32)]),
        "turner_tree_file_box": (_P, [_P]),
        "turner_tree_file_key": (C.c_uint64, [_P]),
        "turner_tree_file_unmap": (None, [_P]),
        "turner_scene_make": (C.c_int, [C.c_int, C.c_uint32, C.c_uint32, C.c_uint64, C.c_float, C.POINTER(_P)]),
        "turner_mesh_num_triangles": (C.c_uint32, [_P]),
        "turner_mesh_vertices": (C.POINTER(C.c_float), [_P]),
        "turner_mesh_normals": (C.POINTER(C.c_float), [_P]),
        "turner_mesh_diffuse": (C.POINTER(C.c_float), [_P]),
        "turner_mesh_reflective": (C.POINTER(C.c_float), [_P]),
        "turner_kdtree_set_reflective": (C.c_int, [_P, _P]),
        "turner_mesh_camera": (None, [_P, C.POINTER(Camera), C.POINTER(C.c_float)]),
        "turner_mesh_light": (C.c_int, [_P, C.POINTER(Light)]),
        "turner_mesh_free": (None, [_P]),
        "turner_make_rays": (C.c_int, [C.c_uint64, _P, C.c_uint64] + [_P] * 6),
        "turner_write_p3": (C.c_uint64, [_P, C.c_uint32, C.c_uint32, _P, C.c_uint64]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def _check(status: int, what: str) -> None:
    if status != OK:
        raise TurnerError(status, what)


def _ptr(a: np.ndarray | None) -> int | None:
    return None if a is None else a.ctypes.data


# ------------------------------------------------------------------ scenes
@dataclass
class Mesh:
    """Triangles of a synthetic scene plus its camera and light."""
    vertices: np.ndarray  # (n, 9) float32
    normals: np.ndarray   # (n, 9) float32
    diffuse: np.ndarray   # (n, 4) float32
    camera: Camera
    hfov: float
    light: Light | None
    reflective: np.ndarray | None = None   # (n, 5) float32: reflective rgba, reflectivity

    @property
    def n_triangles(self) -> int:
        return self.vertices.shape[0]


def make_scene(kind: int, detail: int = 0, count: int = 0, seed: int = 1, aspect: float = 1.0) -> Mesh:
    lib = _lib()
    h = _P()
    _check(lib.turner_scene_make(kind, detail, count, seed, aspect, C.byref(h)), "turner_scene_make")
    try:
        n = lib.turner_mesh_num_triangles(h)
        v = np.ctypeslib.as_array(lib.turner_mesh_vertices(h), (n, 9)).copy()
        nr = np.ctypeslib.as_array(lib.turner_mesh_normals(h), (n, 9)).copy()
        d = np.ctypeslib.as_array(lib.turner_mesh_diffuse(h), (n, 4)).copy()
        rf = np.ctypeslib.as_array(lib.turner_mesh_reflective(h), (n, 5)).copy()
        cam = Camera()
        hfov = C.c_float()
        lib.turner_mesh_camera(h, C.byref(cam), C.byref(hfov))
        light = Light()
        nl = lib.turner_mesh_light(h, C.byref(light))
    finally:
        lib.turner_mesh_free(h)
    return Mesh(v, nr, d, cam, hfov.value, light if nl else None, rf if rf.any() else None)


def make_rays(n: int, box, seed: int) -> tuple[np.ndarray, np.ndarray]:
    """Hit-test rays: origins uniform in `box`, directions uniform on S^2."""
    o = np.empty((3, n), np.float32)
    d = np.empty((3, n), np.float32)
    b = np.asarray(box, np.float32)
    _check(_lib().turner_make_rays(n, _ptr(b), seed, _ptr(o[0]), _ptr(o[1]), _ptr(o[2]), _ptr(d[0]), _ptr(d[1]),
                                   _ptr(d[2])), "turner_make_rays")
    return o, d


def _mesh_arrays(vertices, normals, diffuse):
    v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 9)
    nr = None if normals is None else np.ascontiguousarray(normals, np.float32).reshape(-1, 9)
    d = None if diffuse is None else np.ascontiguousarray(diffuse, np.float32).reshape(-1, 4)
    return v, nr, d


def mesh_key(vertices: np.ndarray, normals: np.ndarray | None = None, diffuse: np.ndarray | None = None) -> int:
    """64-bit content key of a triangle set (the key of its tree file)."""
    v, nr, d = _mesh_arrays(vertices, normals, diffuse)
    return _lib().turner_mesh_key(_ptr(v), None if nr is None else _ptr(nr), None if d is None else _ptr(d),
                                  v.shape[0])


class KDTree:
    """KDTree::KDTree(Triangles) (lib/kdtree.cpp:474-490) on host threads.

    cache_dir: build through a directory of content-keyed tree files (load
    when one is valid for these triangles, else build and write it)."""

    def __init__(self, vertices: np.ndarray, normals: np.ndarray | None = None, diffuse: np.ndarray | None = None,
                 threads: int = 0, cache_dir: str | None = None):
        lib = _lib()
        v, nr, d = _mesh_arrays(vertices, normals, diffuse)
        self._h = _P()
        hit = C.c_int(0)
        _check(lib.turner_kdtree_build_cached(_ptr(v), None if nr is None else _ptr(nr),
                                              None if d is None else _ptr(d), v.shape[0], threads,
                                              None if cache_dir is None else str(cache_dir).encode(),
                                              C.byref(self._h), C.byref(hit)), "turner_kdtree_build_cached")
        self.from_cache = bool(hit.value)

    @classmethod
    def from_mesh(cls, mesh: Mesh, threads: int = 0, cache_dir: str | None = None) -> "KDTree":
        t = cls(mesh.vertices, mesh.normals, mesh.diffuse, threads, cache_dir)
        if mesh.reflective is not None:
            t.set_reflective(mesh.reflective)
        return t

    def set_reflective(self, reflective: np.ndarray) -> None:
        """Reflective colour (rgba) and reflectivity per triangle, (n, 5)."""
        r = np.ascontiguousarray(reflective, np.float32).reshape(-1, 5)
        if r.shape[0] != self.num_triangles():
            raise ValueError("one row per triangle")
        _check(_lib().turner_kdtree_set_reflective(self._h, _ptr(r)), "turner_kdtree_set_reflective")

    @classmethod
    def build_gpu(cls, ctx: "Context", mesh: Mesh) -> "KDTree":
        """Binned-SAH kd-tree built on the context's GPU (same FlatNode format
        and triangle records; not the reference's node words)."""
        v, nr, d = _mesh_arrays(mesh.vertices, mesh.normals, mesh.diffuse)
        t = cls.__new__(cls)
        t._h = _P()
        _check(_lib().turner_kdtree_build_gpu(ctx._h, _ptr(v), _ptr(nr), _ptr(d), v.shape[0], C.byref(t._h)),
               "turner_kdtree_build_gpu")
        t.from_cache = False
        if mesh.reflective is not None:
            t.set_reflective(mesh.reflective)
        return t

    @classmethod
    def load(cls, path, key: int = 0) -> "KDTree":
        """Reads a tree file (key != 0 must match the stored one)."""
        t = cls.__new__(cls)
        t._h = _P()
        _check(_lib().turner_kdtree_load(str(path).encode(), key, C.byref(t._h)), "turner_kdtree_load")
        t.from_cache = True
        return t

    def save(self, path, key: int = 0) -> None:
        _check(_lib().turner_kdtree_save(self._h, key, str(path).encode()), "turner_kdtree_save")

    def __del__(self):
        if getattr(self, "_h", None) and _LIB is not None:
            _LIB.turner_kdtree_free(self._h)
            self._h = None

    def height(self) -> int:
        return _lib().turner_kdtree_height(self._h)

    def num_nodes(self) -> int:
        return _lib().turner_kdtree_num_nodes(self._h)

    def num_triangles(self) -> int:
        return _lib().turner_kdtree_num_triangles(self._h)

    def export(self) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
        """(nodes uint64[n_nodes], triangles float32[n_tris, 48], box float32[6])."""
        nodes = np.empty(self.num_nodes(), np.uint64)
        tris = np.empty((self.num_triangles(), TRIANGLE_FLOATS), np.float32)
        box = np.empty(6, np.float32)
        _check(_lib().turner_kdtree_export(self._h, _ptr(nodes), _ptr(tris), _ptr(box)), "turner_kdtree_export")
        return nodes, tris, box


class TreeFile:
    """A tree file mapped read-only: nodes, triangles and box are zero-copy
    views of the mapping, valid until close()."""

    def __init__(self, path, key: int = 0, verify: bool = True):
        lib = _lib()
        self._h = _P()
        _check(lib.turner_tree_file_map(str(path).encode(), key, 1 if verify else 0, C.byref(self._h)),
               "turner_tree_file_map")
        nn, nt = C.c_uint32(), C.c_uint32()
        pn = lib.turner_tree_file_nodes(self._h, C.byref(nn))
        pt = lib.turner_tree_file_triangles(self._h, C.byref(nt))
        pb = lib.turner_tree_file_box(self._h)
        self.key = lib.turner_tree_file_key(self._h)
        self.nodes = np.ctypeslib.as_array(C.cast(pn, C.POINTER(C.c_uint64)), (nn.value,))
        self.triangles = np.ctypeslib.as_array(C.cast(pt, C.POINTER(C.c_float)), (nt.value, TRIANGLE_FLOATS))
        self.box = np.ctypeslib.as_array(C.cast(pb, C.POINTER(C.c_float)), (6,))

    def close(self) -> None:
        if getattr(self, "_h", None) and _LIB is not None:
            self.nodes = self.triangles = self.box = None
            _LIB.turner_tree_file_unmap(self._h)
            self._h = None

    def __del__(self):
        self.close()


def validate_nodes(nodes: np.ndarray, n_tris: int) -> tuple[int, int]:
    """(status, stack depth) of the host-side node-array check."""
    n = np.ascontiguousarray(nodes, np.uint64)
    depth = C.c_uint32(0)
    st = _lib().turner_validate_nodes(_ptr(n), n.size, n_tris, C.byref(depth))
    return st, depth.value


# ---------------------------------------------------------------- context
class Context:
    """One GPU, one stream, the scenes uploaded to it."""

    def __init__(self, device: int = 0):
        lib = _lib()
        self._h = _P()
        _check(lib.turner_create(C.byref(self._h), device), "turner_create")

    def close(self) -> None:
        if getattr(self, "_h", None) and _LIB is not None:
            _LIB.turner_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self) -> int:
        return self._h.value

    def launch_count(self) -> int:
        return _lib().turner_launch_count(self._h)

    def set_chunk_paths(self, paths: int) -> None:
        _check(_lib().turner_set_chunk_paths(self._h, paths), "turner_set_chunk_paths")

    def set_traversal_launch(self, persistent: bool = True, blocks_per_sm: int = 0) -> None:
        _check(_lib().turner_set_traversal_launch(self._h, 1 if persistent else 0, blocks_per_sm),
               "turner_set_traversal_launch")

    def probe_gather(self, buffer_bytes: int = 64 << 20, load_bytes: int = 8, repeats: int = 5) -> float:
        """GB/s of independent random loads of load_bytes over a buffer of
        buffer_bytes (the traversal's gather roof when the buffer fits L2)."""
        v = C.c_double()
        _check(_lib().turner_probe_gather(self._h, buffer_bytes, load_bytes, repeats, C.byref(v)),
               "turner_probe_gather")
        return v.value

    def set_traversal_refill(self, kind: int, lanes: int) -> None:
        """A warp of the persistent traversal takes new rays of this kind
        (RAYS_*) only once `lanes` of its lanes are idle."""
        _check(_lib().turner_set_traversal_refill(self._h, kind, lanes), "turner_set_traversal_refill")

    def set_traversal_packet(self, mode: int) -> None:
        """Where warps of fresh rays with one direction octant traverse as
        packets (same results): a mask of PACKET_CAMERA (renders' camera
        rays, the default) and PACKET_BATCHED (intersect / occluded)."""
        _check(_lib().turner_set_traversal_packet(self._h, int(mode)), "turner_set_traversal_packet")

    def set_traversal_speculative(self, on: bool) -> None:
        """Speculative traversal rounds (same results)."""
        _check(_lib().turner_set_traversal_speculative(self._h, 1 if on else 0), "turner_set_traversal_speculative")

    def set_traversal_ring(self, entries: int) -> None:
        """0, 4 or 8: how many of each thread's newest traversal-stack entries
        live in shared memory (the rest in local memory)."""
        _check(_lib().turner_set_traversal_ring(self._h, entries), "turner_set_traversal_ring")

    def set_profiling(self, on: bool) -> None:
        _check(_lib().turner_set_profiling(self._h, 1 if on else 0), "turner_set_profiling")

    def kernel_times(self, reset: bool = False) -> dict:
        """{kind: (milliseconds, launches)} measured with CUDA events."""
        ms = np.zeros(KERNEL_KINDS, np.float64)
        n = np.zeros(KERNEL_KINDS, np.uint64)
        _check(_lib().turner_kernel_times(self._h, _ptr(ms), _ptr(n), 1 if reset else 0), "turner_kernel_times")
        return {name: (float(ms[k]), int(n[k])) for k, name in enumerate(KERNEL_NAMES)}

    def upload(self, nodes: np.ndarray, tris: np.ndarray, box: np.ndarray) -> int:
        n = np.ascontiguousarray(nodes, np.uint64)
        t = np.ascontiguousarray(tris, np.float32).reshape(-1, TRIANGLE_FLOATS)
        b = np.ascontiguousarray(box, np.float32)
        sid = C.c_uint32()
        _check(_lib().turner_upload_scene(self._h, _ptr(n), n.size, _ptr(t), t.shape[0], _ptr(b), C.byref(sid)),
               "turner_upload_scene")
        return sid.value

    def upload_tree(self, tree: KDTree) -> int:
        sid = C.c_uint32()
        _check(_lib().turner_upload_kdtree(self._h, tree._h, C.byref(sid)), "turner_upload_kdtree")
        return sid.value

    def free_scene(self, scene_id: int) -> None:
        _check(_lib().turner_free_scene(self._h, scene_id), "turner_free_scene")

    def intersect(self, scene_id: int, o: np.ndarray, d: np.ndarray, mode: int = TRAVERSAL_PARITY):
        """Host-buffer batch intersect. o, d: (3, n) float32. Returns id, r, s, t."""
        o = np.ascontiguousarray(o, np.float32)
        d = np.ascontiguousarray(d, np.float32)
        n = o.shape[1]
        hid = np.empty(n, np.uint32)
        r = np.empty(n, np.float32)
        s = np.empty(n, np.float32)
        t = np.empty(n, np.float32)
        _check(_lib().turner_intersect(self._h, scene_id, _ptr(o[0]), _ptr(o[1]), _ptr(o[2]), _ptr(d[0]), _ptr(d[1]),
                                       _ptr(d[2]), n, _ptr(hid), _ptr(r), _ptr(s), _ptr(t), mode, HOST_BUFFERS),
               "turner_intersect")
        return hid, r, s, t

    def occluded(self, scene_id: int, o: np.ndarray, d: np.ndarray, tmax: np.ndarray) -> np.ndarray:
        """Host-buffer shadow-ray test: o, d (3, n), tmax (n,) float32. Returns
        blocked (n,) bool: some valid intersection with r <= tmax
        (pathtracer.cpp:44-58: lit iff no hit or r_closest > distance)."""
        o = np.ascontiguousarray(o, np.float32)
        d = np.ascontiguousarray(d, np.float32)
        tm = np.ascontiguousarray(tmax, np.float32).reshape(-1)
        n = o.shape[1]
        assert tm.size == n
        out = np.empty(n, np.uint8)
        _check(_lib().turner_occluded(self._h, scene_id, _ptr(o[0]), _ptr(o[1]), _ptr(o[2]), _ptr(d[0]), _ptr(d[1]),
                                      _ptr(d[2]), _ptr(tm), n, _ptr(out), HOST_BUFFERS), "turner_occluded")
        return out.astype(bool)

    def intersect_device(self, scene_id: int, ptrs: list[int], n: int, out_ptrs: list[int],
                         mode: int = TRAVERSAL_PARITY) -> None:
        # ptrs: ox, oy, oz, dx, dy, dz; out_ptrs: id, r, s, t (device addresses)
        """Device-buffer batch intersect (six ray pointers, four output pointers)."""
        _check(_lib().turner_intersect(self._h, scene_id, *ptrs, n, *out_ptrs, mode, DEVICE_BUFFERS),
               "turner_intersect")

    def autotune(self, jobs: list[Job], force: bool = False) -> Tuning:
        """Times launch configurations on `jobs` and applies the fastest."""
        arr = (Job * len(jobs))(*jobs)
        t = Tuning()
        _check(_lib().turner_autotune(self._h, arr, len(jobs), 1 if force else 0, C.byref(t)), "turner_autotune")
        return t

    def get_tuning(self) -> Tuning:
        t = Tuning()
        _check(_lib().turner_get_tuning(self._h, C.byref(t)), "turner_get_tuning")
        return t

    def set_tuning(self, t: Tuning) -> None:
        _check(_lib().turner_set_tuning(self._h, C.byref(t)), "turner_set_tuning")

    def set_guide(self, guide: "Guide | None", train: bool = False, lr: float = 1e-3, records: int = 0,
                  steps_per_pass: int = 16) -> None:
        _check(_lib().turner_set_guide(self._h, guide._h if guide is not None else None, 1 if train else 0, lr,
                                       records), "turner_set_guide")
        _check(_lib().turner_set_guide_steps(self._h, steps_per_pass), "turner_set_guide_steps")

    def guide_stats(self) -> tuple[int, float, float]:
        """(Adam steps of the bound proposal, its last mean loss, training device ms in renders)."""
        steps, loss, ms = C.c_uint64(), C.c_float(), C.c_double()
        _check(_lib().turner_guide_stats(self._h, C.byref(steps), C.byref(loss), C.byref(ms)), "turner_guide_stats")
        return steps.value, loss.value, ms.value

    def set_graph_mode(self, mode) -> None:
        """True / GRAPH_ALWAYS, False / GRAPH_AUTO, or GRAPH_NEVER."""
        m = GRAPH_ALWAYS if mode is True else GRAPH_AUTO if mode is False else int(mode)
        _check(_lib().turner_set_graph_mode(self._h, m), "turner_set_graph_mode")

    def graph_launch_count(self) -> int:
        return _lib().turner_graph_launch_count(self._h)

    def accumulate(self, job: Job, passes: int, readback: bool = True) -> tuple[np.ndarray | None, int]:
        """FP64 running mean of linear radiance after `passes` more passes of
        job.pixel_samples samples each: ((h, w, 4) float64, total samples).
        readback=False keeps the sum on the device and returns (None, total)."""
        out = np.empty((max(0, job.rows), job.width, 4), np.float64) if readback else None
        total = C.c_uint64(0)
        _check(_lib().turner_render_accumulate(self._h, C.byref(job), passes, _ptr(out), C.byref(total),
                                               HOST_BUFFERS), "turner_render_accumulate")
        return out, total.value

    def set_guide_weighting(self, mode: int) -> None:
        """Training-record weights: 0 incident radiance, 1 also by path throughput, 2 by its square root."""
        _check(_lib().turner_set_guide_weighting(self._h, mode), "turner_set_guide_weighting")

    def set_guide_depth(self, depth: int) -> None:
        """Guided jobs sample from the proposal at hits of depth < depth."""
        _check(_lib().turner_set_guide_depth(self._h, depth), "turner_set_guide_depth")

    def render(self, jobs: list[Job], outs: list[int] | None = None, flags: int = HOST_BUFFERS):
        """Renders jobs; returns (images, stats). With flags=DEVICE_BUFFERS,
        `outs` are device pointers and images is None."""
        arr = (Job * len(jobs))(*jobs)
        stats = (Stats * len(jobs))()
        images = None
        if flags == HOST_BUFFERS:
            # a bad row range is the library's to refuse: no negative shapes here
            images = [np.empty((max(0, j.rows), j.width, 4), np.float32) for j in jobs]
            outs = [_ptr(im) for im in images]
        ptrs = (_P * len(jobs))(*outs)
        _check(_lib().turner_render(self._h, arr, len(jobs), ptrs, stats, flags), "turner_render")
        return images, list(stats)


GUIDE_PARAMS = 20264
GUIDE_OBJECTIVE_KL, GUIDE_OBJECTIVE_VARIANCE = 0, 1


class Guide:
    """The learned bounce proposal (BF16 MLP on tcgen05, vMF-mixture head)."""

    def __init__(self, ctx: Context, seed: int = 1):
        self._ctx = ctx   # keeps the context alive
        self._h = _P()
        _check(_lib().turner_guide_create(ctx._h, seed, C.byref(self._h)), "turner_guide_create")

    def close(self) -> None:
        if getattr(self, "_h", None) and _LIB is not None:
            _LIB.turner_guide_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    @property
    def handle(self) -> int:
        return self._h.value

    def set_objective(self, objective: int) -> None:
        """GUIDE_OBJECTIVE_KL (default) or GUIDE_OBJECTIVE_VARIANCE (the 50/50 estimator's second moment)."""
        _check(_lib().turner_guide_set_objective(self._h, objective), "turner_guide_set_objective")

    def get_params(self) -> np.ndarray:
        p = np.empty(GUIDE_PARAMS, np.float32)
        _check(_lib().turner_guide_params(self._h, _ptr(p), 0), "turner_guide_params")
        return p

    def set_params(self, p: np.ndarray) -> None:
        q = np.ascontiguousarray(p, np.float32)
        assert q.size == GUIDE_PARAMS
        _check(_lib().turner_guide_params(self._h, _ptr(q), 1), "turner_guide_params")

    def forward(self, features: np.ndarray) -> np.ndarray:
        f = np.ascontiguousarray(features, np.float32).reshape(-1, 9)
        out = np.empty((f.shape[0], 40), np.float32)
        _check(_lib().turner_guide_forward(self._h, _ptr(f), f.shape[0], _ptr(out)), "turner_guide_forward")
        return out

    def gradient(self, features, dirs, weights):
        f = np.ascontiguousarray(features, np.float32).reshape(-1, 9)
        d = np.ascontiguousarray(dirs, np.float32).reshape(-1, 3)
        w = np.ascontiguousarray(weights, np.float32).reshape(-1)
        g = np.empty(GUIDE_PARAMS, np.float32)
        loss = C.c_float()
        _check(_lib().turner_guide_gradient(self._h, _ptr(f), _ptr(d), _ptr(w), f.shape[0], _ptr(g), C.byref(loss)),
               "turner_guide_gradient")
        return g, loss.value

    def train(self, features, dirs, weights, lr: float = 1e-3, steps: int = 1) -> float:
        f = np.ascontiguousarray(features, np.float32).reshape(-1, 9)
        d = np.ascontiguousarray(dirs, np.float32).reshape(-1, 3)
        w = np.ascontiguousarray(weights, np.float32).reshape(-1)
        loss = C.c_float()
        _check(_lib().turner_guide_train(self._h, _ptr(f), _ptr(d), _ptr(w), f.shape[0], lr, steps, C.byref(loss)),
               "turner_guide_train")
        return loss.value


def look_at_camera(position, target, aspect: float, vfov_deg: float = 40.0, up=(0.0, 1.0, 0.0)) -> Camera:
    """Pinhole camera at `position` looking at `target` (lib/types.h:88-123
    conventions: the camera looks down -z of its frame, so the rotation's
    columns are right, up and -forward; delta_x = tan(vfov / 2) * aspect)."""
    pos = np.asarray(position, np.float64)
    f = np.asarray(target, np.float64) - pos
    f /= np.linalg.norm(f)
    r = np.cross(f, np.asarray(up, np.float64))
    r /= np.linalg.norm(r)
    u = np.cross(r, f)
    rot = np.stack([r, u, -f], axis=1)   # column-wise
    cam = Camera()
    for k in range(3):
        cam.position[k] = pos[k]
    for k, v in enumerate(rot.reshape(-1)):
        cam.trafo[k] = v
    cam.aspect = aspect
    cam.delta_x = float(np.tan(np.radians(vfov_deg) / 2) * aspect)
    return cam


def make_job(scene_id: int, mesh: Mesh, width: int, height: int | None = None, pixel_samples: int = 1,
             max_depth: int = 3, monte_carlo_samples: int = 1, seed: int = 1, exposure: float = 1.0,
             inverse_gamma: float = 0.454545, gamma_correction: bool = True, background=(0.0, 0.0, 0.0),
             sampling: int = SAMPLING_UNIFORM, traversal: int = TRAVERSAL_PARITY, renderer: int = RENDERER_PATH,
             shadow_intensity: float = 0.5, max_visibility: float = 2.0,
             rows: tuple[int, int] | None = None) -> Job:
    """A job with the reference's defaults (config.h, pathtracer.h,
    raytracer.h, raycaster.h). rows=(y0, y1) renders only image rows
    [y0, y1) (the reference's unit of work is one row, main.cpp:193-226)."""
    j = Job()
    j.scene_id = scene_id
    j.width = width
    j.height = height if height is not None else int(np.float32(width) / np.float32(mesh.camera.aspect))
    j.pixel_samples = pixel_samples
    j.max_depth = max_depth
    j.monte_carlo_samples = monte_carlo_samples
    j.exposure = exposure
    j.inverse_gamma = np.float32(inverse_gamma)
    j.gamma_correction = 1 if gamma_correction else 0
    for k in range(3):
        j.background[k] = background[k]
    j.seed = seed
    j.n_lights = 1 if mesh.light is not None else 0
    if mesh.light is not None:
        j.light = mesh.light
    j.camera = mesh.camera
    j.sampling = sampling
    j.traversal = traversal
    j.renderer = renderer
    j.shadow_intensity = shadow_intensity
    j.max_visibility = max_visibility
    if rows is not None:
        j.row_begin, j.row_end = int(rows[0]), int(rows[1])
    return j


def write_p3(rgba: np.ndarray) -> str:
    """P3 text of an (h, w, 4) float32 image (lib/raster.h:79-100)."""
    a = np.ascontiguousarray(rgba, np.float32)
    h, w = a.shape[:2]
    lib = _lib()
    n = lib.turner_write_p3(_ptr(a), w, h, None, 0)
    buf = C.create_string_buffer(n)
    lib.turner_write_p3(_ptr(a), w, h, buf, n)
    return buf.raw[:n].decode()
