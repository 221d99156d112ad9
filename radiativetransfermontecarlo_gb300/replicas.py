"""Replica parallelism: one process per GPU, each on its own range of particle ids.

The reference reduces packet histograms with a parfor sum (`E = E + E_local`,
radiativeTransfer.m:88).  Here every rank transports a disjoint range of global
particle ids (the Philox stream is keyed by the global id, so the union is the same set
of trajectories as one process running them all) and the int64 histograms are summed:
integer addition, exact and independent of the order and of the number of ranks.

With NCCL the sum runs in place on the device histogram the library keeps
(rtmc_histogram_device), and the result crosses to the host once; with gloo (CPU
ranks, or ranks that share a GPU) it runs on the host copy.
"""
from __future__ import annotations

import numpy as np


def shard(n_particles: int, rank: int, world: int) -> tuple[int, int]:
    """(first global particle id, particle count) of `rank` among `world` replicas."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank must lie in [0, world)")
    base, rem = divmod(int(n_particles), world)
    count = base + (1 if rank < rem else 0)
    first = rank * base + min(rank, rem)
    return first, count


def allreduce_histogram(hist: np.ndarray, group=None) -> np.ndarray:
    """Sum a host int64 histogram over the ranks of a gloo group (in place, returned)."""
    import torch
    import torch.distributed as dist
    if hist.dtype != np.int64:
        raise TypeError("histograms are int64")
    if dist.get_backend(group) == "nccl":
        raise ValueError("NCCL ranks reduce the device histogram: use allreduce_device_histogram")
    t = torch.from_numpy(hist)
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return hist


class _DeviceArray:
    """__cuda_array_interface__ view of a library-owned device buffer (no copy)."""

    def __init__(self, ptr: int, n: int):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": "<i8", "data": (ptr, False), "version": 3,
                                         "strides": None}


def allreduce_device_histogram(ctx, group=None) -> int:
    """Sum, over the ranks of an NCCL group, the int64 histogram that rtmc_forward_device
    left in the library context ctx: in place on the device, no host round trip.  Returns
    its length."""
    import torch
    import torch.distributed as dist
    ptr, n = ctx.histogram_device()
    t = torch.as_tensor(_DeviceArray(ptr, n), device=f"cuda:{torch.cuda.current_device()}")
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    torch.cuda.current_stream().synchronize()
    return n


def radiative_transfer_replica(geometry, source, material, observation, options=None, group=None) -> dict:
    """radiativeTransfer on this rank's share of the particles, histograms summed over all
    ranks, normalised with the global particle count.  Needs torch.distributed set up."""
    import torch.distributed as dist

    from .radiative_transfer import build_problem, get_context, normalise
    opt = dict(options or {})
    rank, world = dist.get_rank(group), dist.get_world_size(group)
    prob, grid, n_total = build_problem(geometry, source, material, observation, opt)
    first, count = shard(n_total, rank, world)
    prob.pid0 = int(opt.get("pid0", 0)) + first
    prob.n_particles = count
    ctx = get_context(int(opt.get("device", 0)))
    P, keep = prob.to_ctypes()
    if dist.get_backend(group) == "nccl":
        # the library's stream has finished when forward_device returns
        stats = ctx.forward_device(P, prob.tables)
        allreduce_device_histogram(ctx, group)
        hist = ctx.copy_histogram(np.empty(prob.hist_len, dtype=np.int64))
    else:
        hist, stats = ctx.forward(P, prob.tables)
        allreduce_histogram(hist, group)
    obs = dict(grid.obs)
    obs["energyDensity"], obs["energy"] = normalise(hist, grid, n_total, prob.hist_shift)
    obs["stats"] = stats
    obs["E"] = hist
    return obs
