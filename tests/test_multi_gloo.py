"""Multi-rank host logic on the CPU (gloo, world size 2, 127.0.0.1).

Each rank renders its rows of one frame with the oracle standing in for its
GPU; the gathered image must equal a single-process render bit for bit,
because per-pixel seeds depend only on (pixel, sample). A rank that fails
before the gather must be reported to the other rank as an error (process
group timeout), not as a hang."""
import datetime
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from turner_gb300.shard import frame_seed, row_range

W, H, SPP, DEPTH, SEED = 24, 19, 2, 2, 5


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _scene():
    import turner_gb300 as tg
    from oracle import oracle as orc

    m = tg.make_scene(tg.SCENE_SPHERE_ROOM, detail=2)
    nodes, tris, box = tg.KDTree.from_mesh(m).export()
    return m, orc.Scene(nodes, tris, box)


def _worker(rank, world, port, out_dir, fail_rank):
    import torch.distributed as dist

    from turner_gb300.shard import gather_rows

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=datetime.timedelta(seconds=10))
    try:
        m, sc = _scene()
        y0, y1 = row_range(H, rank, world)
        img, _ = sc.render(m.camera, m.light, W, H, SPP, DEPTH, seed=SEED, threads=2, rows=(y0, y1))
        if rank == fail_rank:
            raise RuntimeError("injected failure before the gather")
        full = gather_rows(img[y0:y1], H)
        np.save(os.path.join(out_dir, f"rank{rank}.npy"), full)
        dist.barrier()
    except RuntimeError as e:
        with open(os.path.join(out_dir, f"rank{rank}.err"), "w") as f:
            f.write(str(e))
    finally:
        try:
            dist.destroy_process_group()
        except Exception:
            pass


def test_row_range_partitions_exactly():
    for height in (1, 7, 19, 1080):
        for world in (1, 2, 3, 8):
            rows = [row_range(height, r, world) for r in range(world)]
            assert rows[0][0] == 0 and rows[-1][1] == height
            assert all(a[1] == b[0] for a, b in zip(rows, rows[1:]))
            sizes = [b - a for a, b in rows]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        row_range(10, 2, 2)
    assert [frame_seed(1, r) for r in range(4)] == [1, 2, 3, 4]


def test_two_ranks_rebuild_the_single_process_image(tmp_path):
    port = _free_port()
    mp.spawn(_worker, args=(2, port, str(tmp_path), -1), nprocs=2, join=True)
    m, sc = _scene()
    ref, _ = sc.render(m.camera, m.light, W, H, SPP, DEPTH, seed=SEED, threads=2)
    for r in range(2):
        got = np.load(tmp_path / f"rank{r}.npy")
        assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))


def test_failed_rank_is_reported_not_hung(tmp_path):
    port = _free_port()
    mp.spawn(_worker, args=(2, port, str(tmp_path), 1), nprocs=2, join=True)
    assert (tmp_path / "rank1.err").read_text().startswith("injected failure")
    # rank 0 waited in the gather and was released by the timeout with an error
    assert (tmp_path / "rank0.err").exists()
    assert not (tmp_path / "rank0.npy").exists()


def _gpu_worker(rank, world, port, out_dir):
    import torch.distributed as dist

    import turner_gb300 as tg
    from turner_gb300.shard import gather_rows

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=datetime.timedelta(seconds=60))
    try:
        m = tg.make_scene(tg.SCENE_SPHERE_ROOM, detail=3)
        with tg.Context(0) as ctx:
            sid = ctx.upload_tree(tg.KDTree.from_mesh(m))
            y0, y1 = row_range(GH, rank, world)
            job = tg.make_job(sid, m, GW, GH, pixel_samples=SPP, max_depth=DEPTH, seed=SEED, rows=(y0, y1))
            (img,), _ = ctx.render([job])
        full = gather_rows(img, GH)
        np.save(os.path.join(out_dir, f"gpu_rank{rank}.npy"), full)
        dist.barrier()
    finally:
        dist.destroy_process_group()


GW, GH = 40, 27


@pytest.mark.gpu
def test_two_ranks_render_their_rows_on_the_gpu(tmp_path):
    """The product path of the row partition: two ranks (processes, gloo on
    the host) each render their rows through turner_render's row range and
    all-gather them; the frame equals one single-process GPU render bit for
    bit. Both ranks share one GPU; their kernels never wait on each other
    (only the host-side gather does)."""
    import turner_gb300 as tg

    port = _free_port()
    mp.spawn(_gpu_worker, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    m = tg.make_scene(tg.SCENE_SPHERE_ROOM, detail=3)
    with tg.Context(0) as ctx:
        sid = ctx.upload_tree(tg.KDTree.from_mesh(m))
        (ref,), _ = ctx.render([tg.make_job(sid, m, GW, GH, pixel_samples=SPP, max_depth=DEPTH, seed=SEED)])
    for r in range(2):
        got = np.load(tmp_path / f"gpu_rank{r}.npy")
        assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))
