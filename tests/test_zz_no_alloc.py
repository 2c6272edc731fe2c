"""turner_intersect_noalloc: the batched intersect for callers that must not
allocate device memory while they run (a per-frame loop where cudaMalloc could
stall the device, or a host framework whose pool owns all device memory).

The entry point is called through the C ABI with rays and outputs in device
memory owned by the caller (torch tensors here), twice in a row, and compared
with turner_intersect on the same rays. Hit ids, r, s and t must be equal as
bit patterns: the tolerance of every hit test in this suite is exact. The file
is named so that pytest collects it last."""
import ctypes as C

import numpy as np
import pytest

import turner_gb300 as tg

pytestmark = pytest.mark.gpu


def _device_rays(torch, o, d):
    return [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (*o, *d)]


def _outputs(torch, n):
    return [torch.empty(n, dtype=torch.int32, device="cuda")] + \
        [torch.empty(n, dtype=torch.float32, device="cuda") for _ in range(3)]


def test_noalloc_intersect_matches_turner_intersect():
    torch = pytest.importorskip("torch")
    lib = tg._lib()
    mesh = tg.make_scene(tg.SCENE_SPHERE_ROOM, detail=5)
    tree = tg.KDTree.from_mesh(mesh)
    nodes, tris, box = tree.export()
    with tg.Context(0) as ctx:
        sid = ctx.upload(nodes, tris, box)
        n = 300_000
        o, d = tg.make_rays(n, box, seed=77)
        d[1, ::11] = 0   # zero components exercise the EPS direction fix
        rays = _device_rays(torch, o, d)
        ray_ptrs = [t.data_ptr() for t in rays]

        for mode in (tg.TRAVERSAL_PARITY, tg.TRAVERSAL_FAST):
            # the existing entry point, device buffers, same mode
            want = _outputs(torch, n)
            ctx.intersect_device(sid, ray_ptrs, n, [t.data_ptr() for t in want], mode=mode)
            torch.cuda.synchronize()
            want_np = [w.cpu().numpy().view(np.uint32) for w in want]
            assert (want_np[0] != tg.MISS).any()
            for call in range(2):   # two calls in a row: the static scratch must be reset each time
                got = _outputs(torch, n)
                st = lib.turner_intersect_noalloc(ctx.handle, sid, *ray_ptrs, n, *[g.data_ptr() for g in got], mode)
                assert st == tg.OK, tg.TurnerError(st)
                got_np = [g.cpu().numpy().view(np.uint32) for g in got]
                for a, b in zip(got_np, want_np):
                    assert np.array_equal(a, b), (mode, call)

        # more rays than the 32-bit work counter allows are refused before any launch
        st = lib.turner_intersect_noalloc(ctx.handle, sid, *ray_ptrs, tg_max_rays() + 1,
                                          *[g.data_ptr() for g in got], tg.TRAVERSAL_PARITY)
        assert st == tg.ERR_TOO_LARGE
        assert lib.turner_intersect_noalloc(ctx.handle, 999, *ray_ptrs, n, *[g.data_ptr() for g in got],
                                            tg.TRAVERSAL_PARITY) == tg.ERR_INVALID_ARG


def tg_max_rays():
    return 1 << 30
