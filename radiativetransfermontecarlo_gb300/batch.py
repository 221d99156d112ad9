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
             split_chunks=(2048, 4096, 8192), repeats: int = 2):
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


def radiative_transfer_batch(instances, device: int = 0, tune: bool = False) -> list[dict]:
    """radiativeTransfer for every instance in one batched launch."""
    b = Batch(instances, device)
    if tune:
        autotune(b)
    b.run()
    res = b.results()
    b.close()
    return res
