"""Host-side partition of render work over ranks (one process per GPU).

Every (pixel, sample) path is independent, so frames shard with no
collective on the data path:

  - frames per rank (what bench.py measures, weak scaling): rank r renders
    its own frame with seed base + r; nothing is exchanged.
  - rows per rank (one frame over several GPUs): rank r renders the rows
    row_range(height, r, world) of the same frame; per-pixel seeds depend only
    on (pixel, sample), so the rows are exactly those of a single-GPU render.
    The tiles are gathered once at the end.
"""
from __future__ import annotations

import numpy as np


def frame_seed(base: int, rank: int) -> int:
    return base + rank


def row_range(height: int, rank: int, world: int) -> tuple[int, int]:
    """Contiguous, balanced rows [y0, y1) of rank `rank` out of `world`."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    base, extra = divmod(height, world)
    y0 = rank * base + min(rank, extra)
    return y0, y0 + base + (1 if rank < extra else 0)


def gather_rows(tile: np.ndarray, height: int, group=None) -> np.ndarray:
    """All-gathers every rank's rows (tile: (rows, width, 4) float32) into the
    full (height, width, 4) image on every rank (torch.distributed)."""
    import torch
    import torch.distributed as dist

    world = dist.get_world_size(group)
    width = tile.shape[1]
    rows_max = max(row_range(height, r, world)[1] - row_range(height, r, world)[0] for r in range(world))
    pad = np.zeros((rows_max, width, 4), np.float32)
    pad[: tile.shape[0]] = tile
    parts = [torch.zeros((rows_max, width, 4), dtype=torch.float32) for _ in range(world)]
    dist.all_gather(parts, torch.from_numpy(pad), group=group)
    out = np.empty((height, width, 4), np.float32)
    for r, p in enumerate(parts):
        y0, y1 = row_range(height, r, world)
        out[y0:y1] = p.numpy()[: y1 - y0]
    return out
