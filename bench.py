#!/usr/bin/env python3
"""Benchmark: particle scattering events/s of the transport hot path on one GB300.

Workload: 3D elastic isotropic unbounded medium, 1e7 particles, cartesian 60^3 x 8
directions x 251 times x 2 modes (867,456,000 int64 bins, 6.9 GB), FP32 propagation,
int64 fixed-point histogram (2^-40).  One step = one whole simulation of that workload
(histogram clear + particle init + transport + binning) with the tables resident.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
  python bench.py --workload c1|c3|c4|c5   (3D acoustic FP64 / half-space / batched sweep / gradient;
                                            one extra JSON line each)

Prints one JSON line.  `value` is device time (CUDA events on the library's stream);
`e2e` times rtmc_forward through the C ABI with host buffers (tables uploaded and the
histogram copied to pinned host memory every step).  `--impl reference` times the CPU
restatement of the reference's own sub-step algorithm on the host cores, on a problem and
tables set up by the oracle itself (oracle/reference_problem.py), so it loads no product code.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "particle scattering events/s on 1 GB300, FP32 vs plain FP64 at ≤0.5% rel-L2 energyDensity"
UNIT = "scattering events/s"
WORKLOAD = ("3D elastic isotropic unbounded (vp=2, vs=1.155, cv=0.1x3, gauss lc=0.2, f=5, Q=Inf), point source, "
            "1e7 particles, cartesian x=y=z=-5:1/6:5 x 8 directions x 251 times x 2 modes, int64 fixed point 2^-40")


def log(*a):
    print(*a, file=sys.stderr, flush=True)


# ---------------------------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.file = None

    def __enter__(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.file, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if self.proc is None or self.file is None:
            return None
        rows = []
        with open(self.file.name) as f:
            for line in f:
                p = [x.strip() for x in line.split(",")]
                if len(p) < 9:
                    continue
                try:
                    rows.append(dict(sm=float(p[1]), smax=float(p[2]), power=float(p[3]),
                                     hw=p[5], hwt=p[6], swt=p[7], swp=p[8]))
                except ValueError:
                    continue
        os.unlink(self.file.name)
        if not rows:
            return None
        load = [r for r in rows if r["power"] > 0.25 * max(x["power"] for x in rows)] or rows
        reasons = set()
        for r in load:
            for k, name in (("hw", "hw_slowdown"), ("hwt", "hw_thermal_slowdown"), ("swt", "sw_thermal_slowdown"),
                            ("swp", "sw_power_cap")):
                if r[k].lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": float(np.median([r["sm"] for r in load])), "sm_max_mhz": max(r["smax"] for r in rows),
                "reasons": sorted(reasons), "samples": len(load)}


# ---------------------------------------------------------------------------------- helpers
def measured_peak_hbm():
    p = ROOT / "MEASURED_PEAKS.json"
    try:
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def load_traffic(field: str = "dram_bytes_full_launch"):
    """Per kernel, a figure of one full-size launch of this workload from one-pass ncu
    captures summarised in profiles/c2_traffic.json: DRAM bytes read + written (default),
    or the L2 reduction requests of the fold ("l2_reduction_requests",
    lts__t_requests_srcunit_tex_op_red.sum); {} when absent."""
    p = ROOT / "profiles" / "c2_traffic.json"
    try:
        d = json.loads(p.read_text())
        return {k: v[field] for k, v in d["kernels"].items() if field in v}
    except Exception:
        return {}


# Algorithmic work per unit (the roofline basis): issue slots of one lane per scattering
# event and per particle start (Philox block, logarithm, sine/cosine pairs, table lookup,
# rotation and renormalisation), and per (particle, observation instant) on the cartesian
# path (three multiply-adds, three floors and range tests, the index, one store); a warp
# instruction issues 32 lanes.  Peak issue: 4 warp instructions per clock per SM.
ISSUE_PER_EVENT, ISSUE_PER_START, ISSUE_PER_OBS = 100.0, 120.0, 12.0


def issue_peak(clocks, sms: int = 152) -> float:
    """Warp instructions per second the GPU can issue at the sampled SM clock."""
    mhz = (clocks or {}).get("sm_mhz") or 2070.0
    return 4.0 * sms * mhz * 1e6


def cpu_histogram(prob):
    """The oracle's histogram for timing runs, allocated and written once; returns it and
    the seconds that took (the one fixed cost of a run over the whole workload)."""
    t0 = time.perf_counter()
    hist = np.zeros(prob.hist_len, dtype=np.int64)
    hist.fill(0)
    return hist, time.perf_counter() - t0


def cpu_sample(prob, knots, target_s: float = 12.0, threads: int | None = None, hist=None, fixed: float = 0.0,
               particles: int | None = None):
    """Reference-order sub-step oracle on a bounded particle sample of the same workload.

    The rate is the whole workload's: its events over (the fixed seconds of allocating and
    zeroing its histogram + its particles x the sample's seconds per particle).  Timed runs
    add into one histogram that is already resident, so a sample is not charged the
    first-touch page faults of the whole histogram (the 6.9 GB of C2) over and over."""
    from oracle import oracle as O
    nth = threads or (os.cpu_count() or 1)
    if hist is None:
        hist, fixed = cpu_histogram(prob)
    n2 = particles
    if n2 is None:
        n = 4000
        while True:  # calibrate the time per particle
            t0 = time.perf_counter()
            O.run(prob, knots, scheme="substep", ufloat=False, nthreads=nth, n_particles=n, pid0=0, hist=hist)
            dt = time.perf_counter() - t0
            if dt > 1.0 or n >= 1_000_000:
                break
            n *= 4
        n2 = int(min(4_000_000, max(n, target_s * n / dt)))
    t0 = time.perf_counter()
    _, st, _ = O.run(prob, knots, scheme="substep", ufloat=False, nthreads=nth, n_particles=n2, pid0=10_000_000,
                     hist=hist)
    dt = time.perf_counter() - t0
    N = int(prob.n_particles)
    full_s = fixed + dt / n2 * N
    full_events = st["scatter_events"] / n2 * N
    return {"value": full_events / full_s, "unit": UNIT, "cores": nth, "kind": "port",
            "sample": f"{n2} of the workload's {N} particles over all 250 time steps, reference sub-step order "
                      f"(h={prob.h:.5g}, {prob.n_sub * prob.n_obs} sub-steps/particle), {dt:.1f} s; rate of the whole "
                      f"workload = its events / ({fixed:.2f} s to allocate and zero its histogram + {N} x the "
                      f"sample's time per particle)",
            "events": st["scatter_events"], "seconds": dt, "full_events": full_events, "full_seconds": full_s,
            "fixed_seconds": fixed, "particles": n2}


def baseline_fields(sample: dict) -> dict:
    """The cpu_baseline object of a bench line from a cpu_sample result."""
    return {k: sample[k] for k in ("value", "unit", "cores", "kind", "sample")}


def rel_l2_density(a: np.ndarray, b: np.ndarray, grid, chunk_bins: int) -> float:
    """relative L2 of energyDensity between two count arrays of the same grid (same weights)."""
    dpsi = np.asarray(grid.obs["dpsi"], float)
    nb = grid.shape[:4]
    per_psi = nb[0] * nb[1] * nb[2]
    num = den = 0.0
    n = a.size
    for s in range(0, n, chunk_bins):
        e = min(n, s + chunk_bins)
        idx = np.arange(s, e)
        w = 1.0 / dpsi[(idx // per_psi) % nb[3]]
        x = a[s:e].astype(np.float64) * w
        y = b[s:e].astype(np.float64) * w
        num += float(np.dot(x - y, x - y))
        den += float(np.dot(y, y))
    return math.sqrt(num / den) if den > 0 else float("nan")


# ---------------------------------------------------------------------------------- arms
def run_reference_arm(args, rank, world):
    if rank != 0:
        return None
    # the oracle's own problem set-up and table builder: this arm loads no product code
    from oracle import reference_problem
    prob, knots = reference_problem.c2_problem()
    nth = os.cpu_count() or 1
    per_step = args.ref_seconds or max(2.0, 120.0 / max(1, args.steps + args.warmup))
    hist, fixed = cpu_histogram(prob)
    times, full_events, full_seconds, nparts, particles = [], 0.0, 0.0, 0, None
    for i in range(args.warmup + args.steps):
        s = cpu_sample(prob, knots, target_s=per_step, threads=nth, hist=hist, fixed=fixed, particles=particles)
        particles = s["particles"]  # calibrated by the first warm-up step
        if i >= args.warmup:
            times.append(s["seconds"])
            full_events += s["full_events"]
            full_seconds += s["full_seconds"]
            nparts += particles
    value = full_events / full_seconds
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000 * float(np.mean(times)), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "sample_particles_per_step": nparts // max(1, args.steps)},
            "impl": "reference",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": nth, "kind": "port",
                             "sample": "each step: a particle sample of the workload sized to a few seconds, "
                                       "reference sub-step algorithm (C restatement), all host threads; rate of "
                                       f"the whole workload = its events / ({fixed:.2f} s to allocate and zero its "
                                       "histogram + its particles x each sample's time per particle)"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    return line


def run_our_arm(args, rank, world, dist):
    from oracle import oracle as O
    from radiativetransfermontecarlo_gb300 import _lib, build_problem, get_context
    from radiativetransfermontecarlo_gb300 import workloads as W
    device = int(os.environ.get("LOCAL_RANK", 0))
    n = args.particles
    geo, src, mat, obs, opts = W.c2_elastic3d(n=n, precision="fp32", t_end=args.t_end)
    prob, grid, N = build_problem(geo, src, mat, obs, dict(opts, exact_count=True, pid0=rank * n))
    ctx = get_context(device)
    if args.block or args.ring or args.index_mb:
        ctx.set_launch(args.block, args.ring, args.index_mb)
    if args.chunks or args.k1_bps:
        ctx.set_pipeline(args.chunks, args.k1_bps)
    if args.schedule >= 0:
        ctx.set_schedule(args.schedule)
    if args.fold:
        ctx.set_fold(args.fold)
    P32, keep32 = prob.to_ctypes()

    def barrier():
        if dist is not None:
            dist.barrier()

    def step(P):
        st = ctx.forward_device(P, prob.tables)
        return st

    for _ in range(args.warmup):
        step(P32)
    # timed region: device time of each step from CUDA events on the library stream
    dev_ms, kern_ms, fold_ms, ev_ms, cv_ms, events, obs_n = [], [], [], [], [], 0, 0
    barrier()
    with ClockSampler(device) as clk:
        t_wall = time.perf_counter()
        for _ in range(args.steps):
            ctx.flush_l2()
            st = step(P32)
            if dist is not None:
                # the replicas' histograms summed in place on the devices (NCCL), timed with
                # the step: the parfor sum E = E + E_local of the reference
                import torch
                from radiativetransfermontecarlo_gb300.replicas import allreduce_device_histogram
                t0 = torch.cuda.Event(enable_timing=True)
                t1 = torch.cuda.Event(enable_timing=True)
                t0.record()
                allreduce_device_histogram(ctx)
                t1.record()
                t1.synchronize()
                st["total_ms"] += t0.elapsed_time(t1)
            dev_ms.append(st["total_ms"])
            kern_ms.append(st["kernel_ms"])
            fold_ms.append(st["fold_ms"])
            ev_ms.append(st["events_ms"])
            cv_ms.append(st["convert_ms"])
            launches_per_step = ctx.last_timing()[1]
            events += st["scatter_events"]
            obs_n += st["observations"]
        t_wall = time.perf_counter() - t_wall
    clocks = clk.summary()
    barrier()
    total_s = sum(dev_ms) / 1000.0
    if dist is not None:
        import torch
        tt = torch.tensor([total_s], dtype=torch.float64, device=f"cuda:{device}")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        ev = torch.tensor([events], dtype=torch.float64, device=f"cuda:{device}")
        dist.all_reduce(ev)
        total_s, events_all = float(tt.item()), float(ev.item())
    else:
        events_all = events
    value = events_all / total_s
    ms_per_step = 1000.0 * total_s / args.steps
    result = {}
    if rank == 0:
        peak, peak_kind = measured_peak_hbm()
        kmean, fmean, emean = float(np.mean(kern_ms)), float(np.mean(fold_ms)), float(np.mean(ev_ms))
        cmean = float(np.mean(cv_ms))
        entries = N * prob.n_obs  # (particle, observation instant) pairs of one step
        obs_per_step = obs_n / args.steps
        ev_step = events / args.steps
        ipk = issue_peak(clocks)
        traffic = load_traffic()
        # rt_events and rt_observe: bound by instruction issue (the algorithmic issue slots
        # above); rt_observe also writes the 4-byte bin index of every (particle, instant)
        ev_inst = (ev_step * ISSUE_PER_EVENT + N * ISSUE_PER_START) / 32.0
        ob_inst = entries * ISSUE_PER_OBS / 32.0
        omean = max(kmean - emean, 1e-9)
        kernels = {
            "rt_events": {"ms": emean, "bound": "issue", "algorithmic_warp_inst": ev_inst,
                          "achieved": ev_inst / max(emean, 1e-9) / 1e6, "peak": ipk / 1e9, "unit": "Ginst/s",
                          "frac": ev_inst / max(emean, 1e-9) * 1e3 / ipk, "traffic": traffic.get("rt_events")},
            "rt_observe": {"ms": omean, "bound": "issue", "algorithmic_warp_inst": ob_inst,
                           "achieved": ob_inst / omean / 1e6, "peak": ipk / 1e9, "unit": "Ginst/s",
                           "frac": ob_inst / omean * 1e3 / ipk, "index_write_gbs": 4.0 * entries / omean / 1e6,
                           "traffic": traffic.get("rt_observe")},
        }
        if cmean > 0:
            # time-blocked fold: rt_fold_tb reads the index array once (its FP32 vector
            # reductions land in the L2); rt_tb_convert reads the FP32 accumulator (4 B per
            # bin and instant) and writes the 8-byte histogram
            tmean = max(fmean - cmean, 1e-9)
            fb, cb = 4.0 * entries, 12.0 * prob.hist_len
            kernels["rt_fold_tb"] = {"ms": tmean, "bound": "hbm", "algorithmic_bytes": fb,
                                     "achieved": fb / tmean / 1e6, "peak": peak, "unit": "GB/s",
                                     "frac": fb / tmean / 1e6 / peak,
                                     "observations_per_s": obs_per_step / tmean * 1e3,
                                     "traffic": traffic.get("rt_fold_tb")}
            # its actual bound: the L2's rate of 16-byte vector reductions, measured here by
            # rtmc_probe_l2_reductions; the requests per launch come from a one-pass capture
            reds = load_traffic("l2_reduction_requests").get("rt_fold_tb")
            red_peak = ctx.probe_l2_reductions()
            kernels["rt_fold_tb"]["l2_reductions"] = {
                "per_launch": reds, "peak_per_s": red_peak, "unit": "red.global.add.v4.f32 per second",
                "achieved_per_s": reds / tmean * 1e3 if reds else None,
                "frac": reds / tmean * 1e3 / red_peak if reds and red_peak else None}
            kernels["rt_tb_convert"] = {"ms": cmean, "bound": "hbm", "algorithmic_bytes": cb,
                                        "achieved": cb / cmean / 1e6, "peak": peak, "unit": "GB/s",
                                        "frac": cb / cmean / 1e6 / peak, "traffic": traffic.get("rt_tb_convert")}
        else:
            # 64-bit slice fold: reads the index array and, slice by slice in the L2, reads
            # and writes the histogram once (its 64-bit reductions stay in the L2)
            k2_bytes = 4.0 * entries + 16.0 * prob.hist_len
            kernels["rt_bin_slices"] = {"ms": fmean, "bound": "hbm", "algorithmic_bytes": k2_bytes,
                                        "achieved": k2_bytes / max(fmean, 1e-9) / 1e6, "peak": peak, "unit": "GB/s",
                                        "frac": k2_bytes / max(fmean, 1e-9) / 1e6 / peak,
                                        "l2_reductions_per_s": obs_per_step / max(fmean, 1e-9) * 1e3,
                                        "traffic": traffic.get("rt_bin_slices")}
        dom = max(kernels, key=lambda k: kernels[k]["ms"])
        kd = kernels[dom]
        result = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                  "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
                  "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                  "config": {"workload": WORKLOAD, "particles_per_gpu": n, "histogram_bins": int(prob.hist_len),
                             "l2": "512 MB device write between steps; the 6.9 GB histogram exceeds L2",
                             "wall_s_timed": t_wall},
                  "roofline": {"bound": kd["bound"], "achieved": kd["achieved"], "peak": kd["peak"], "unit": kd["unit"],
                               "frac": kd["frac"], "traffic": kd["traffic"], "kernel": dom, "kernel_ms": kd["ms"],
                               "basis": "rt_events: 100 issue slots per event + 120 per particle start; rt_observe: 12 "
                                        "per (particle, instant); issue peak 4 warp instructions/clk/SM at the sampled "
                                        "clock; rt_fold_tb: the 4 B index entry of every (particle, instant) read once; "
                                        "rt_tb_convert: 4 B of FP32 count read and the 8 B bin written per (bin, instant); "
                                        "rt_bin_slices (slice fold): the index read + the 8 B histogram read and written "
                                        f"once; HBM peak {peak_kind}; traffic: DRAM bytes of one full-size launch "
                                        "(ncu, one pass)",
                               "kernels": kernels},
                  "gpu_launches": args.steps * launches_per_step, "clocks": clocks,
                  "events_per_step": events / args.steps, "observations_per_step": obs_per_step,
                  "observations_per_s": obs_per_step * args.steps / total_s,
                  "transport_ms": kmean, "fold_ms": fmean, "convert_ms": cmean, "sink": int(st["sink"])}
    # end to end through the C ABI with host buffers
    # (first, while the host holds no other histogram-sized buffer; the accuracy check below
    # reuses its pinned buffer)
    buf = _lib.PinnedBuffer(prob.hist_len * 8) if rank == 0 and not (args.no_e2e and args.no_fp64) else None
    if rank == 0 and not args.no_e2e:
        # the reference's uint32 E (rtmc_forward_u32: counts narrowed on the device after the
        # int64 fixed-point accumulation), then the int64 fixed-point histogram itself
        def e2e_leg(call, out):
            ctx.set_table_cache(False)
            call(P32, prob.tables, out)
            times, dev, kern, ev, h2d, d2h = [], [], [], 0, 0.0, 0.0
            with ClockSampler(device) as clk:
                call(P32, prob.tables, out)  # untimed: the sampler's start-up runs beside it
                for _ in range(max(3, args.steps // 2)):
                    ctx.flush_l2()
                    t0 = time.perf_counter()
                    _, st = call(P32, prob.tables, out)
                    times.append(time.perf_counter() - t0)
                    dev.append(st["total_ms"])
                    kern.append(st["kernel_ms"] + st["fold_ms"])
                    ev += st["scatter_events"]
                    h2d, d2h = st["h2d_bytes"], st["d2h_bytes"]
            ctx.set_table_cache(True)
            return {"value": ev / sum(times), "unit": UNIT, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "ms_per_step": 1000 * float(np.mean(times)),
                    "ms_per_step_median": 1000 * float(np.median(times)),
                    "ms_steps": [round(1000 * t, 2) for t in times],
                    # the same calls' CUDA-event time from their first to their last queued
                    # operation (copies included): a step slow here too was slow on the device
                    # or the host link, not in host code; and the transport + fold share of it
                    # (the copies overlap the folds): a step slow there was slow in the kernels
                    "device_ms_steps": [round(t, 2) for t in dev],
                    "kernel_ms_steps": [round(t, 2) for t in kern], "clocks": clk.summary()}
        result["e2e"] = dict(e2e_leg(ctx.forward_u32, buf.array(np.uint32, prob.hist_len)),
                             api="rtmc_forward_u32 (uint32 counts, the reference's E type)")
        # the same call into pageable host memory, which is what a MEX gateway receives from
        # mxCreateNumericMatrix (the first, untimed call touches its pages)
        pageable = np.empty(prob.hist_len, dtype=np.uint32)
        result["e2e_pageable"] = dict(e2e_leg(ctx.forward_u32, pageable),
                                      api="rtmc_forward_u32 into pageable host memory (a MEX gateway's mxArray)")
        del pageable
        result["e2e_int64"] = dict(e2e_leg(ctx.forward, buf.array(np.int64, prob.hist_len)),
                                   api="rtmc_forward (int64 fixed point, 2^-40)")
        # the host link alone: one plain device-to-host copy of the histogram, as a yardstick
        # for the end-to-end figures (each is transport + the first fold group + its bytes
        # at this rate when the link bounds it)
        out = buf.array(np.int64, prob.hist_len)
        ctx.copy_histogram(out)
        ts = []
        for _ in range(3):
            t0 = time.perf_counter()
            ctx.copy_histogram(out)
            ts.append(time.perf_counter() - t0)
        result["host_link_d2h_gbs"] = prob.hist_len * 8 / min(ts) / 1e9
    # FP64 leg (same seed: the same trajectories up to rounding), then the accuracy check
    if rank == 0 and not args.no_fp64:
        geo, src, mat, obs, opts = W.c2_elastic3d(n=n, precision="fp64", t_end=args.t_end)
        prob64, _, _ = build_problem(geo, src, mat, obs, dict(opts, exact_count=True, pid0=0))
        prob64.tables = prob.tables
        P64, keep64 = prob64.to_ctypes()
        step(P64)
        ms64, ev64 = [], 0
        for _ in range(max(2, args.steps // 10)):
            ctx.flush_l2()
            st = step(P64)
            ms64.append(st["total_ms"])
            ev64 += st["scatter_events"]
        v64 = ev64 / (sum(ms64) / 1000.0)
        result["fp64"] = {"value": v64, "unit": UNIT, "ms_per_step": float(np.mean(ms64))}
        result["fp32_over_fp64"] = value / v64
        if not args.no_accuracy:
            b64 = ctx.copy_histogram(np.empty(prob.hist_len, dtype=np.int64))
            step(P32)
            a32 = ctx.copy_histogram(buf.array(np.int64, prob.hist_len))
            result["rel_l2_energy_density_fp32_vs_fp64"] = rel_l2_density(a32, b64, grid, 1 << 26)
            del b64
    if rank == 0 and not args.no_cpu:
        knots = O.table_knots(prob.tables)
        hist, fixed = cpu_histogram(prob)
        result["cpu_baseline"] = baseline_fields(cpu_sample(prob, knots, hist=hist, fixed=fixed))
        one = cpu_sample(prob, knots, target_s=4.0, threads=1, hist=hist, fixed=fixed)
        result["cpu_baseline"]["single_core"] = {"value": one["value"], "sample": one["sample"]}
    return result


def run_c4(args):
    """256 independent 3D acoustic instances (lc, cv, f, Q, N drawn per instance), shared
    spherical 120 x 251 grid, one persistent CUDA-graph launch per step."""
    from oracle import oracle as O
    from radiativetransfermontecarlo_gb300 import workloads as W
    from radiativetransfermontecarlo_gb300.batch import Batch, autotune, tune_schedule
    t0 = time.perf_counter()
    batch = Batch([W.c4_instance(i) for i in range(args.instances)])
    setup_s = time.perf_counter() - t0
    if args.no_tune:
        shape, tune, factor, tune_f = (0, 0, 0), {}, 4, {}
    else:
        shape, tune = autotune(batch, repeats=1)
        factor, tune_f = tune_schedule(batch, repeats=1)
    n_em = int(batch.schedule().sum())
    for _ in range(args.warmup):
        batch.run()
    ms, ev = [], 0
    with ClockSampler(0) as clk:
        for _ in range(args.steps):
            batch.ctx.flush_l2()
            st = batch.run()
            ms.append(st["kernel_ms"])
            ev += st["scatter_events"]
    value = ev / (sum(ms) / 1000.0)
    # end to end: launch + every instance's histogram back to the host
    times, ev2 = [], 0
    for _ in range(max(3, args.steps // 4)):
        t1 = time.perf_counter()
        st = batch.run()
        H = batch.histograms()
        times.append(time.perf_counter() - t1)
        ev2 += st["scatter_events"]
    n_total = int(sum(batch.N))
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": float(np.mean(ms)), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"{args.instances}-instance 3D acoustic sweep: lc log-U[0.02,1], cv U[0.01,0.2], "
                                   "f log-U[1,20], Q in {Inf,100,500}, N log-U[1e4,1e7]; spherical 120 x 251 grid",
                       "particles_total": n_total, "launch_shape": list(shape), "table_setup_s": setup_s,
                       "event_major_factor": factor, "event_major_instances": n_em,
                       "l2": "512 MB device write between steps"},
            "gpu_launches": args.steps, "clocks": clk.summary(),
            "events_per_step": ev / args.steps,
            "e2e": {"value": ev2 / sum(times), "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": int(H.nbytes), "ms_per_step": 1000 * float(np.mean(times))},
            "autotune_ms": {f"{b}x{r}x{c}": t for (b, r, c), t in tune.items()},
            "schedule_tune_ms": {str(f): t for f, t in tune_f.items()}}
    if not args.no_cpu:
        prob = batch.problems[int(np.argmax(batch.N))]
        line["cpu_baseline"] = baseline_fields(cpu_sample(prob, O.table_knots(prob.tables), target_s=args.cpu_seconds))
        line["cpu_baseline"]["sample"] = "the largest instance, " + line["cpu_baseline"]["sample"]
    batch.close()
    return line


def run_c1(args):
    """3D acoustic isotropic unbounded, 1e6 particles, spherical 120 r x 251 t, FP64 as the
    reference runs it (and FP32); the CPU port runs the whole workload."""
    from oracle import oracle as O
    from radiativetransfermontecarlo_gb300 import build_problem, get_context, normalise
    from radiativetransfermontecarlo_gb300 import workloads as W
    n = args.particles if args.particles != 10_000_000 else 1_000_000
    ctx = get_context(0)
    out = {}
    for prec in ("fp64", "fp32"):
        geo, src, mat, obs, opts = W.c1_acoustic3d(n=n, precision=prec)
        prob, grid, N = build_problem(geo, src, mat, obs, dict(opts, exact_count=True))
        P, keep = prob.to_ctypes()
        for _ in range(args.warmup):
            ctx.forward_device(P, prob.tables)
        ms, ev = [], 0
        with ClockSampler(0) as clk:
            for _ in range(args.steps):
                ctx.flush_l2()
                st = ctx.forward_device(P, prob.tables)
                ms.append(st["total_ms"])
                ev += st["scatter_events"]
        h, st1 = ctx.forward(P, prob.tables)
        dens, energy = normalise(h, grid, N)
        out[prec] = {"value": ev / (sum(ms) / 1000.0), "ms": float(np.mean(ms)), "clocks": clk.summary(),
                     "energy": energy, "density": dens, "obs": st1["observations"], "sink": st1["sink"],
                     "prob": prob}
    e64, e32 = out["fp64"]["energy"], out["fp32"]["energy"]
    d64, d32 = out["fp64"]["density"], out["fp32"]["density"]
    line = {"metric": METRIC, "value": out["fp64"]["value"], "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": out["fp64"]["ms"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "3D acoustic isotropic unbounded, exp lc=0.1 cv=0.05/0.05 f=10 v=1, point source "
                                   "lambda=0.05, 1e6 particles, spherical 120 r x 251 t", "particles": n},
            "gpu_launches": args.steps, "clocks": out["fp64"]["clocks"], "sink": out["fp64"]["sink"],
            "fp32": {"value": out["fp32"]["value"], "ms_per_step": out["fp32"]["ms"]},
            "fp32_over_fp64": out["fp32"]["value"] / out["fp64"]["value"],
            "rel_l2_energy_density_fp32_vs_fp64": float(np.linalg.norm(d32 - d64) / np.linalg.norm(d64)),
            "energy_conserved_fp64": bool(np.all(e64[1:, 0] == 1.0)), "energy_conserved_fp32": bool(np.all(e32[1:, 0] == 1.0))}
    if not args.no_cpu:
        prob = out["fp64"]["prob"]
        nth = os.cpu_count() or 1
        t0 = time.perf_counter()
        _, st, _ = O.run(prob, O.table_knots(prob.tables), scheme="substep", ufloat=False, nthreads=nth)
        dt = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": st["scatter_events"] / dt, "unit": UNIT, "cores": nth, "kind": "port",
                                "sample": f"the whole workload ({n} particles, 250 sub-steps each), reference sub-step "
                                          f"order, {dt:.1f} s"}
    return line


def run_c3(args):
    """2D elastic P-SV half-space, free surface with Zoeppritz reflection, Q = 200, 1e8
    particles, cylindrical 200 r x 401 t; FP32 vs FP64 (1e7 particles, the same ids)."""
    from oracle import oracle as O
    from radiativetransfermontecarlo_gb300 import build_problem, get_context, normalise
    from radiativetransfermontecarlo_gb300 import workloads as W
    import warnings
    n = args.particles if args.particles != 10_000_000 else 100_000_000
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        geo, src, mat, obs, opts = W.c3_halfspace2d(n=n, precision="fp32")
        prob, grid, N = build_problem(geo, src, mat, obs, dict(opts, exact_count=True))
        n64 = min(n, 10_000_000)
        geo, src, mat, obs, opts = W.c3_halfspace2d(n=n64, precision="fp64")
        prob64, _, _ = build_problem(geo, src, mat, obs, dict(opts, exact_count=True))
    prob64.tables = prob.tables
    ctx = get_context(0)
    if args.block or args.ring or args.index_mb:
        ctx.set_launch(args.block, args.ring, args.index_mb)
    if args.schedule >= 0:
        ctx.set_schedule(args.schedule)
    P32, k32 = prob.to_ctypes()
    for _ in range(args.warmup):
        ctx.forward_device(P32, prob.tables)
    ms, ev = [], 0
    with ClockSampler(0) as clk:
        for _ in range(args.steps):
            ctx.flush_l2()
            st = ctx.forward_device(P32, prob.tables)
            ms.append(st["total_ms"])
            ev += st["scatter_events"]
    value = ev / (sum(ms) / 1000.0)
    # FP64 and FP32 on the same 1e7 particle ids: speed ratio and the per-bin error
    P64, k64 = prob64.to_ctypes()
    h64, s64 = ctx.forward(P64, prob.tables)
    P32s, k32s = prob.to_ctypes()
    P32s.n_particles = n64
    h32, s32 = ctx.forward(P32s, prob.tables)
    e32 = normalise(h32, grid, n64)[0]
    e64 = normalise(h64, grid, n64)[0]
    m = e64 > 0
    rel = np.abs(e32[m] - e64[m]) / e64[m]
    sig = np.sqrt(np.maximum(h64.reshape(grid.shape, order="F")[m], 1))  # Monte Carlo error of a bin, in counts
    z = (h32.reshape(grid.shape, order="F")[m] - h64.reshape(grid.shape, order="F")[m]) / sig
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": float(np.mean(ms)), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic",
            "config": {"workload": "2D elastic P-SV half-space, free surface y=0 (Zoeppritz), source at depth 1, "
                                   "exp lc=0.5 f=8 cv=0.2x3, vp=2 vs=1.155 rho=1000, Q=200, cylindrical 200 r x 401 t",
                       "particles": n, "l2": "512 MB device write between steps"},
            "gpu_launches": args.steps * int(st["launches"]), "clocks": clk.summary(), "events_per_step": ev / args.steps,
            "boundary_hits_per_step": st["boundary_hits"], "kills_per_step": st["kills"], "sink": st["sink"],
            "fp64_vs_fp32_same_1e7_ids": {"fp64_ms": s64["kernel_ms"], "fp32_ms": s32["kernel_ms"],
                                          "fp32_over_fp64": s64["kernel_ms"] / s32["kernel_ms"],
                                          "rel_l2_energy_density": float(np.linalg.norm(e32 - e64) / np.linalg.norm(e64)),
                                          "per_bin_rel_error_median": float(np.median(rel)),
                                          "per_bin_rel_error_p99": float(np.quantile(rel, 0.99)),
                                          "per_bin_diff_over_sqrt_count_p99": float(np.quantile(np.abs(z), 0.99)),
                                          "bins": int(m.sum())}}
    if not args.no_cpu:
        line["cpu_baseline"] = baseline_fields(cpu_sample(prob, O.table_knots(prob.tables), target_s=args.cpu_seconds))
    return line


def run_c5(args):
    """Gradient of L = sum (E - E_t)^2 / E_t over (lc, cv_kappa, cv_rho, Q) at lc 0.1,
    cv [0.05 0.05], Q 400 against a target at lc 0.12, cv [0.06 0.04], Q 300, 3D acoustic,
    1e7 particles, C1's grid; checked against central differences with common random numbers."""
    from radiativetransfermontecarlo_gb300 import MaterialClass
    from radiativetransfermontecarlo_gb300 import adjoint as A
    from radiativetransfermontecarlo_gb300 import workloads as W
    n = args.particles  # 1e7, the configuration's count, unless asked otherwise
    geo, src, mat0, obs, opts = W.c1_acoustic3d(n=n, precision="fp32")
    tgt = MaterialClass(geo, 10, True, 1, [0.06, 0.04], 0, "exp", 0.12)
    tgt.Q = 300
    o = dict(opts, exact_count=True, precision="fp32")
    Et = A.forward_weighted(geo, src, tgt, obs, dict(o, seed=77))[0]
    mat = MaterialClass(geo, 10, True, 1, [0.05, 0.05], 0, "exp", 0.1)
    mat.Q = 400
    params = ("lc", "cv_kappa", "cv_rho", "Q", "mfp")
    o = dict(o, seed=5)
    if args.block or args.ring or args.index_mb or args.schedule >= 0:
        from radiativetransfermontecarlo_gb300 import get_context
        get_context(0).set_launch(args.block, args.ring, args.index_mb)
        if args.schedule >= 0:  # 0 or 1: the lockstep ring replay; 2: the split replay
            get_context(0).set_schedule(args.schedule)
    for _ in range(args.warmup):
        A.radiativeTransferGradient(geo, src, mat, obs, Et, params, o)
    fwd, adj, wall, ev = [], [], [], 0
    with ClockSampler(0) as clk:
        for _ in range(args.steps):
            t0 = time.perf_counter()
            res = A.radiativeTransferGradient(geo, src, mat, obs, Et, params, o)
            wall.append(time.perf_counter() - t0)
            fwd.append(res["forward_stats"]["total_ms"])
            adj.append(res["adjoint_stats"]["total_ms"])
            ev += res["forward_stats"]["scatter_events"] + res["adjoint_stats"]["scatter_events"]
    dev_s = (sum(fwd) + sum(adj)) / 1000.0
    scale = {"lc": 0.1, "cv_kappa": 0.05, "cv_rho": 0.05, "Q": 400.0, "mfp": float(mat.meanFreePath)}
    if args.no_fd:  # timing or profiling only
        return {"metric": "gradient evaluations/s (forward + adjoint replay)", "value": args.steps / dev_s,
                "unit": "gradients/s", "forward_ms": float(np.mean(fwd)), "adjoint_ms": float(np.mean(adj)),
                "gradient": res["grad"], "particles": n}
    fd = {p: A.finite_difference(geo, src, mat, obs, Et, p, 1e-3, o) for p in params}
    fd2 = {p: A.finite_difference(geo, src, mat, obs, Et, p, 1e-2, o) for p in params if p != "Q"}
    g = np.array([res["grad"][p] * scale[p] for p in params])
    f = np.array([fd[p] * scale[p] for p in params])
    f2 = np.array([(fd2[p] if p != "Q" else fd[p]) * scale[p] for p in params])
    line = {"metric": "gradient evaluations/s (forward + adjoint replay), " + UNIT + " alongside",
            "value": args.steps / dev_s, "unit": "gradients/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000 * dev_s / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 (FP64 gradient accumulation)", "data": "synthetic",
            "config": {"workload": "3D acoustic exp lc=0.1 cv=[.05 .05] f=10 Q=400, 1e7 particles, spherical 120 x 251, "
                                   "target lc=0.12 cv=[.06 .04] Q=300 (1e7 particles, another seed)",
                       "bins_in_misfit": res["bins"], "min_target_count": 1000},
            "scattering_events_per_s": ev / dev_s, "forward_ms": float(np.mean(fwd)), "adjoint_ms": float(np.mean(adj)),
            "wall_ms": 1000 * float(np.mean(wall)), "gpu_launches": 2 * args.steps, "clocks": clk.summary(),
            "L": res["L"], "gradient": res["grad"],
            "finite_differences_1e-3": fd, "finite_differences_1e-2": fd2,
            "rel_error_scaled_vector_1e-3": float(np.linalg.norm(g - f) / np.linalg.norm(f)),
            "rel_error_scaled_vector_1e-2": float(np.linalg.norm(g - f2) / np.linalg.norm(f2)),
            "rel_error_per_param_1e-3": {p: abs(res["grad"][p] - fd[p]) / abs(fd[p]) for p in params},
            "rel_error_per_param_1e-2": {p: abs(res["grad"][p] - (fd2.get(p, fd[p]))) / abs(fd2.get(p, fd[p]))
                                         for p in params},
            "weights_centred": bool(res.get("centred"))}
    return line


def sub_records(args):
    """Compact records of the other four workloads (C1 3D acoustic FP64 and FP32, C3
    half-space, C4 batched sweep, C5 gradient), each measured as its own --workload run
    does with fewer steps and shorter CPU samples."""
    import copy
    out = {}
    keep = ("value", "unit", "ms_per_step", "clocks", "fp32", "fp32_over_fp64", "rel_l2_energy_density_fp32_vs_fp64",
            "energy_conserved_fp64", "energy_conserved_fp32", "events_per_step", "fp64_vs_fp32_same_1e7_ids",
            "cpu_baseline", "e2e", "launch_shape", "forward_ms", "adjoint_ms", "rel_error_scaled_vector_1e-3",
            "rel_error_per_param_1e-3", "scattering_events_per_s", "metric", "config")
    for name, fn, steps in (("c1", run_c1, 5), ("c3", run_c3, 2), ("c4", run_c4, 3), ("c5", run_c5, 2)):
        a = copy.copy(args)
        a.steps, a.warmup, a.cpu_seconds = steps, 2, 4.0
        a.particles = 10_000_000  # each workload's own default count
        t0 = time.perf_counter()
        try:
            line = fn(a)
            rec = {k: line[k] for k in keep if k in line}
            if "cpu_baseline" in rec:
                rec["cpu_baseline"] = {k: rec["cpu_baseline"][k] for k in ("value", "unit", "cores", "kind")}
            rec["seconds"] = time.perf_counter() - t0
            out[name] = rec
        except Exception as e:  # one failing record must not take the headline line with it
            out[name] = {"error": f"{type(e).__name__}: {e}"}
        log(f"sub-record {name}: {time.perf_counter() - t0:.1f} s")
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--particles", type=int, default=10_000_000)
    ap.add_argument("--t-end", type=float, default=5.0, help="last observation time (profiling cases only)")
    ap.add_argument("--block", type=int, default=0, help="threads per block (0: automatic)")
    ap.add_argument("--ring", type=int, default=0, help="segments per lane (0: automatic)")
    ap.add_argument("--index-mb", type=int, default=0, help="index-array budget in MB (0: automatic, -1: global atomics)")
    ap.add_argument("--chunks", type=int, default=0, help="transport/fold pipeline chunks (0: automatic, 1: off)")
    ap.add_argument("--schedule", type=int, default=-1, help="-1 automatic, 0 lockstep warp batches, 1 particle per thread")
    ap.add_argument("--k1-bps", type=int, default=0, help="transport blocks per SM while pipelined (0: automatic)")
    ap.add_argument("--fold", type=int, default=0,
                    help="fold of the index path: 0 automatic, 1 64-bit slice fold, 2 time-blocked, 3 rolling")
    ap.add_argument("--ref-seconds", type=float, default=0.0,
                    help="reference arm: seconds of CPU work per step (0: about 120 s over all steps)")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-accuracy", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="seconds of each CPU-baseline sample")
    ap.add_argument("--no-tune", action="store_true", help="c4: the default launch shape, no autotuning")
    ap.add_argument("--instances", type=int, default=256, help="c4: instances of the sweep (the first n of its draw)")
    ap.add_argument("--no-fd", action="store_true", help="c5: skip the finite-difference check (timing only)")
    ap.add_argument("--no-sub", action="store_true",
                    help="skip the compact C1/C3/C4/C5 records that the default C2 line carries")
    ap.add_argument("--workload", default="c2", choices=["c1", "c2", "c3", "c4", "c5"],
                    help="c2: the headline line (default); c1: 3D acoustic FP64; c3: 2D half-space; "
                         "c4: batched sweep; c5: gradient")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    if args.impl == "reference" and args.workload == "c2":
        # the reference arm runs the oracle alone: build it, and nothing of the product
        from oracle import oracle as O
        O.build()
        line = run_reference_arm(args, rank, world)
        if line is not None:
            print(json.dumps(line), flush=True)
        return
    import __graft_entry__
    __graft_entry__.build()
    if args.workload != "c2":
        if rank == 0:
            line = {"c1": run_c1, "c3": run_c3, "c4": run_c4, "c5": run_c5}[args.workload](args)
            print(json.dumps(line), flush=True)
        return
    dist = None
    if world > 1:
        import torch
        import torch.distributed as td
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
        td.init_process_group("nccl")
        dist = td
    line = run_our_arm(args, rank, world, dist)
    if rank == 0 and not args.no_sub and world == 1:
        line["workloads"] = sub_records(args)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
