"""Batched radiative transfer: many independent problems on one GPU in one persistent,
CUDA-graph-captured launch (rtmc_batch_* of librtmc).

A parameter sweep over materials (the reference drives radiativeTransfer.m once per
material) becomes one launch: instances share the observation grid, each has its own
tables, particle count and seed; blocks pull (instance, particle range) work items,
largest expected cost first.
"""
from __future__ import annotations

import ctypes as C
import os
import time
from concurrent.futures import ThreadPoolExecutor

import numpy as np

from . import _lib
from .material import MaterialClass
from .radiative_transfer import build_problem, get_context, normalise


class Batch:
    def __init__(self, instances, device: int = 0):
        """instances: list of (geometry, source, material, observation, options)."""
        self.ctx = get_context(device)
        self.problems, self.grids, self.N = [], [], []
        # tables first, on host threads (the FP64 builder releases the GIL)
        todo = [(mat, int(geo["dimension"])) for geo, src, mat, obs, opt in instances if mat.invcdf is None]
        if todo:
            with ThreadPoolExecutor(max_workers=min(len(todo), os.cpu_count() or 1)) as ex:
                list(ex.map(lambda md: MaterialClass.prepareSigma(*md), todo))
        for geo, src, mat, obs, opt in instances:
            prob, grid, n = build_problem(geo, src, mat, obs, opt)
            self.problems.append(prob)
            self.grids.append(grid)
            self.N.append(n)
        self._keep = []
        arr = (_lib.RtmcProblem * len(self.problems))()
        for i, p in enumerate(self.problems):
            P, keep = p.to_ctypes()
            arr[i] = P
            self._keep.append(keep)
        self._arr = arr
        tabs = (C.c_void_p * len(self.problems))(*[p.tables.handle.value for p in self.problems])
        h = C.c_void_p()
        _lib.check(self.ctx.lib.rtmc_batch_create(self.ctx.handle, len(self.problems), arr, tabs, C.byref(h)),
                   self.ctx.handle)
        self.handle = h
        self.hist_len = self.problems[0].hist_len

    def set_launch(self, block: int = 0, ring_cap: int = 0, chunk: int = 0):
        _lib.check(self.ctx.lib.rtmc_batch_set_launch(self.handle, block, ring_cap, chunk), self.ctx.handle)

    def set_em_histogram(self, shared: int = -1):
        """rtmc_batch_set_em_histogram: 1 shared-memory, 0 (default) or -1 device-memory
        histogram for the event-major instances."""
        _lib.check(self.ctx.lib.rtmc_batch_set_em_histogram(self.handle, shared), self.ctx.handle)

    def run(self) -> dict:
        st = _lib.RtmcStats()
        _lib.check(self.ctx.lib.rtmc_batch_run(self.handle, C.byref(st)), self.ctx.handle)
        return st.as_dict()

    def schedule(self) -> np.ndarray:
        """1 for the instances the event-major kernel runs, 0 for the lockstep kernel's."""
        out = np.zeros(len(self.problems), dtype=np.int32)
        _lib.check(self.ctx.lib.rtmc_batch_schedule(self.handle, out.ctypes.data_as(C.POINTER(C.c_int32))),
                   self.ctx.handle)
        return out

    def set_schedule(self, event_major=None):
        """rtmc_batch_set_schedule: event_major[i] = 1 runs instance i on the event-major
        kernel, 0 on the lockstep kernel; None restores the automatic choice."""
        if event_major is None:
            ptr = None
        else:
            em = np.ascontiguousarray(event_major, dtype=np.int32)
            if em.shape != (len(self.problems),):
                raise ValueError("event_major needs one entry per instance")
            ptr = em.ctypes.data_as(C.POINTER(C.c_int32))
        _lib.check(self.ctx.lib.rtmc_batch_set_schedule(self.handle, ptr), self.ctx.handle)

    def expected_events(self) -> np.ndarray:
        """Expected scatterings per particle of each instance over the observed time (the
        quantity the automatic kernel choice compares with the observation instants)."""
        out = np.zeros(len(self.problems))
        for i in range(len(self.problems)):
            P = self._arr[i]
            rates = [1.0 / P.mft[m] for m in range(1 if P.acoustics else 2) if np.isfinite(P.mft[m]) and P.mft[m] > 0]
            out[i] = (max(rates) if rates else 0.0) * P.h * P.n_sub * P.n_obs
        return out

    def histograms(self, first: int = 0, count: int | None = None) -> np.ndarray:
        count = len(self.problems) - first if count is None else count
        out = np.empty((count, self.hist_len), dtype=np.int64)
        _lib.check(self.ctx.lib.rtmc_batch_histograms(self.handle, first, count,
                                                      out.ctypes.data_as(C.POINTER(C.c_int64))), self.ctx.handle)
        return out

    def results(self) -> list[dict]:
        """obs structs (energyDensity, energy, grid fields) of every instance."""
        H = self.histograms()
        out = []
        for i, (grid, n, prob) in enumerate(zip(self.grids, self.N, self.problems)):
            obs = dict(grid.obs)
            obs["energyDensity"], obs["energy"] = normalise(H[i], grid, n, prob.hist_shift)
            out.append(obs)
        return out

    def close(self):
        if getattr(self, "handle", None) and self.handle.value:
            self.ctx.lib.rtmc_batch_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def autotune(batch: Batch, blocks=(256, 512), rings=(4, 8), chunks=(4096, 16384, 65536),
             split_chunks=(4096,), repeats: int = 2):
    """Time every launch shape of the grid on the batch itself and keep the fastest
    (block, ring capacity, particles per work item); (0, -1, chunk) is the split kernel.
    Returns (best shape, {shape: ms})."""
    shapes = [(0, -1, c) for c in split_chunks] + [(b, r, c) for b in blocks for r in rings for c in chunks]
    times = {}
    for shape in shapes:
        try:
            batch.set_launch(*shape)
        except _lib.RtmcError:
            continue
        batch.run()  # warm-up
        times[shape] = min(batch.run()["kernel_ms"] for _ in range(repeats))
    shape = min(times, key=times.get)
    batch.set_launch(*shape)
    return shape, times


def tune_schedule(batch: Batch, factors=(2, 4, 8, 16, 32), repeats: int = 2):
    """Time the split of the instances between the two kernels on the batch itself: an
    instance runs event-major when factor x its expected events per particle >= its
    observation instants (4 is the automatic choice).  Keeps the fastest and returns
    (best factor, {factor: ms})."""
    ev = batch.expected_events()
    n_obs = np.array([batch._arr[i].n_obs for i in range(len(batch.problems))], dtype=np.float64)
    times, seen = {}, {}
    for f in factors:
        em = (f * ev >= n_obs).astype(np.int32)
        key = em.tobytes()
        if key in seen:  # the same split as an earlier factor
            times[f] = times[seen[key]]
            continue
        seen[key] = f
        batch.set_schedule(em)
        batch.run()  # warm-up
        times[f] = min(batch.run()["kernel_ms"] for _ in range(repeats))
    best = min(times, key=times.get)
    batch.set_schedule((best * ev >= n_obs).astype(np.int32))
    return best, times


def radiative_transfer_batch(instances, device: int = 0, tune: bool = False) -> list[dict]:
    """radiativeTransfer for every instance in one batched launch."""
    b = Batch(instances, device)
    if tune:
        autotune(b)
        tune_schedule(b)
    b.run()
    res = b.results()
    b.close()
    return res
