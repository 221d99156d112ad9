"""Replica parallelism on CPU ranks (gloo, world size 2): every rank transports its own
range of particle ids and the int64 histograms are summed.  Counter-based Philox keyed
by the global id makes the sum equal, bin for bin, to one process running all the
particles.  On CPU ranks the per-rank transport is the oracle; the GPU test runs the
product's radiative_transfer_replica on two ranks that share GPU 0 (their kernels never
wait on one another; the sum is on the host, over gloo)."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

N = 6000


def _problem():
    from radiativetransfermontecarlo_gb300 import build_problem
    from radiativetransfermontecarlo_gb300 import workloads as W
    geo, src, mat, obs, opts = W.c1_acoustic3d(n=N, precision="fp64")
    prob, grid, n = build_problem(geo, src, mat, obs, dict(opts, exact_count=True))
    return prob


def _rank(rank, world, port, out):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import torch.distributed as dist

    from oracle import oracle as O
    from radiativetransfermontecarlo_gb300.replicas import allreduce_histogram, shard
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    prob = _problem()
    first, count = shard(prob.n_particles, rank, world)
    hist, _, _ = O.run(prob, O.table_knots(prob.tables), scheme="event", n_particles=count, pid0=first, nthreads=1)
    allreduce_histogram(hist)
    if rank == 0:
        np.save(out, hist)
    dist.barrier()
    dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_cpu_ranks_sum_to_the_single_run(tmp_path):
    out = str(tmp_path / "hist.npy")
    mp.start_processes(_rank, args=(2, _free_port(), out), nprocs=2, join=True, start_method="spawn")
    from oracle import oracle as O
    prob = _problem()
    ref, _, _ = O.run(prob, O.table_knots(prob.tables), scheme="event")
    got = np.load(out)
    assert np.array_equal(got, ref)


def _gpu_rank(rank, world, port, out):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import torch.distributed as dist

    from radiativetransfermontecarlo_gb300 import workloads as W
    from radiativetransfermontecarlo_gb300.replicas import radiative_transfer_replica
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    geo, src, mat, obs, opts = W.c1_acoustic3d(n=30000, precision="fp32")
    res = radiative_transfer_replica(geo, src, mat, obs, dict(opts, exact_count=True))
    if rank == 0:
        np.save(out, res["E"])
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.gpu
def test_gpu_replicas_sum_to_the_single_run(tmp_path):
    """Two gloo ranks sharing GPU 0, each transporting its half of the particle ids on the
    GPU (independent kernels), histograms summed on the host: bin for bin the single run."""
    out = str(tmp_path / "hist_gpu.npy")
    mp.start_processes(_gpu_rank, args=(2, _free_port(), out), nprocs=2, join=True, start_method="spawn")
    from radiativetransfermontecarlo_gb300 import build_problem, get_context
    from radiativetransfermontecarlo_gb300 import workloads as W
    geo, src, mat, obs, opts = W.c1_acoustic3d(n=30000, precision="fp32")
    prob, grid, n = build_problem(geo, src, mat, obs, dict(opts, exact_count=True))
    P, keep = prob.to_ctypes()
    ref, _ = get_context(0).forward(P, prob.tables)
    assert np.array_equal(np.load(out), ref)
