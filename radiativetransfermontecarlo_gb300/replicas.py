"""Replica parallelism: one process per GPU, each on its own range of particle ids.

The reference reduces packet histograms with a parfor sum (`E = E + E_local`,
radiativeTransfer.m:88).  Here every rank transports a disjoint range of global
particle ids (the Philox stream is keyed by the global id, so the union is the same set
of trajectories as one process running them all) and the int64 histograms are summed:
integer addition, exact and independent of the order and of the number of ranks.
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
    """Sum an int64 histogram over the ranks of torch.distributed (in place, returned)."""
    import torch
    import torch.distributed as dist
    if hist.dtype != np.int64:
        raise TypeError("histograms are int64")
    backend = dist.get_backend(group)
    if backend == "nccl":
        t = torch.from_numpy(hist).cuda()
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
        hist[...] = t.cpu().numpy()
    else:
        t = torch.from_numpy(hist)
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return hist


def radiative_transfer_replica(geometry, source, material, observation, options=None, group=None) -> dict:
    """radiativeTransfer on this rank's share of the particles, histograms summed over all
    ranks, normalised with the global particle count.  Needs torch.distributed set up."""
    import torch.distributed as dist

    from .radiative_transfer import build_problem, normalise, run_transport
    opt = dict(options or {})
    rank, world = dist.get_rank(group), dist.get_world_size(group)
    prob, grid, n_total = build_problem(geometry, source, material, observation, opt)
    first, count = shard(n_total, rank, world)
    prob.pid0 = int(opt.get("pid0", 0)) + first
    prob.n_particles = count
    hist, stats = run_transport(prob, int(opt.get("device", 0)))
    allreduce_histogram(hist, group)
    obs = dict(grid.obs)
    obs["energyDensity"], obs["energy"] = normalise(hist, grid, n_total, prob.hist_shift)
    obs["stats"] = stats
    return obs
