"""Rank-level host logic: which k-points a rank owns and how the local sums
are combined.

The reference distributes k round robin (mpi_ki_selector,
src/mpi_comm.f90:80-99: rank r of P owns 1-based ki = r+1, r+1+P, ...), counts
k with MPI_ALLREDUCE (src/core.f90:276) and sums every *_loc tensor to the root
with MPI_REDUCE (src/core.f90:328, :467-531).  Here one process drives one
GPU; the share is passed to mepi_run as (k_begin = rank, k_stride = P) and the
local sums are combined with torch.distributed (gloo or NCCL) in FP64.
"""
from __future__ import annotations

from typing import Callable

import numpy as np

LOC_KEYS = ("Ne_sum", "ahc", "mep_ic", "mep_lc", "mep_cs", "kubo_mep_ic", "kubo_mep_lc", "kubo_mep_cs")


def rank_share(rank: int, world: int):
    """(k_begin, k_stride) of mpi_ki_selector for 0-based k indices."""
    if world <= 0 or not (0 <= rank < world):
        raise ValueError("bad rank/world")
    return rank, world


def reduce_loc(loc: dict, group=None) -> dict:
    """Sum the local sums of all ranks (every rank gets the total)."""
    import torch
    import torch.distributed as dist
    out = {}
    for k in LOC_KEYS + tuple(x for x in ("velo_ahc", "kubo_ohc") if x in loc):
        a = np.asarray(loc[k])
        cplx = np.iscomplexobj(a)
        flat = a.ravel(order="F")
        flat = np.stack([flat.real, flat.imag], axis=1).ravel() if cplx else flat.astype(np.float64)
        t = torch.from_numpy(np.ascontiguousarray(flat).copy())
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
        r = t.numpy()
        r = r[0::2] + 1j * r[1::2] if cplx else r
        out[k] = r.reshape(a.shape, order="F")
    n = torch.tensor([int(loc["n_k"])], dtype=torch.int64)
    dist.all_reduce(n, op=dist.ReduceOp.SUM, group=group)
    out["n_k"] = int(n.item())
    return out


def run_ranked(compute: Callable[[int, int], dict], rank: int, world: int, group=None) -> dict:
    """compute(k_begin, k_stride) -> local sums; returns the global sums."""
    k_begin, k_stride = rank_share(rank, world)
    loc = compute(k_begin, k_stride)
    return reduce_loc(loc, group) if world > 1 else loc
