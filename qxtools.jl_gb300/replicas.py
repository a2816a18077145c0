"""Replica parallelism over bitstrings (one process per GPU).

The reference splits the output bitstrings across MPI ranks and each rank contracts its own
(docs/src/users_guide.md:11-13; qxrun.jl's --mpi).  Bitstrings are independent, so here every
rank runs its own programme on a contiguous shard and the only cross-rank step is a host-side
gather of the amplitudes at the end -- no collective on the data path.
"""
from __future__ import annotations

import numpy as np

__all__ = ["shard_bounds", "shard", "gather_amplitudes"]


def shard_bounds(n: int, rank: int, world: int):
    """[begin, end) of rank's contiguous share of n items (the first n % world ranks get one more)."""
    if world <= 0 or not 0 <= rank < world:
        raise ValueError("bad rank/world size")
    q, r = divmod(n, world)
    begin = rank * q + min(rank, r)
    return begin, begin + q + (1 if rank < r else 0)


def shard(items, rank: int, world: int):
    b, e = shard_bounds(len(items), rank, world)
    return list(items[b:e])


def gather_amplitudes(local: np.ndarray, n_total: int, rank: int, world: int, group=None):
    """Gather every rank's (n_local, out_size) complex128 block to rank 0 (torch.distributed on
    the host).  Returns the full (n_total, out_size) array on rank 0, None elsewhere."""
    import torch
    import torch.distributed as dist
    if world == 1:
        return local
    out_size = local.shape[1]
    maxn = max(shard_bounds(n_total, r, world)[1] - shard_bounds(n_total, r, world)[0] for r in range(world))
    buf = torch.zeros((maxn, out_size, 2), dtype=torch.float64)
    buf[: local.shape[0]] = torch.from_numpy(np.ascontiguousarray(local).view(np.float64).reshape(-1, out_size, 2))
    parts = [torch.zeros_like(buf) for _ in range(world)] if rank == 0 else None
    dist.gather(buf, parts, dst=0, group=group)
    if rank != 0:
        return None
    rows = []
    for r in range(world):
        b, e = shard_bounds(n_total, r, world)
        rows.append(parts[r][: e - b].numpy().reshape(e - b, out_size * 2).view(np.complex128))
    return np.concatenate(rows, axis=0)
