#!/usr/bin/env python3
"""Benchmark: particle scattering events/s of the transport hot path on one GB300.

Workload: 3D elastic isotropic unbounded medium, 1e7 particles, cartesian 60^3 x 8
directions x 251 times x 2 modes (867,456,000 int64 bins, 6.9 GB), FP32 propagation,
int64 fixed-point histogram (2^-40).  One step = one whole simulation of that workload
(histogram clear + particle init + transport + binning) with the tables resident.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line.  `value` is device time (CUDA events on the library's stream);
`e2e` times rtmc_forward through the C ABI with host buffers (tables uploaded and the
histogram copied to pinned host memory every step).  `--impl reference` times the CPU
restatement of the reference's own sub-step algorithm on the host cores.
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


def load_traffic():
    """DRAM bytes per launch of each kernel (read + write) from the last ncu capture of this
    workload, summarised in profiles/c2_traffic.json; {} when absent."""
    p = ROOT / "profiles" / "c2_traffic.json"
    try:
        d = json.loads(p.read_text())
        return {k: v["dram_read_bytes"] + v["dram_write_bytes"] for k, v in d["kernels"].items()}
    except Exception:
        return {}


def cpu_sample(prob, knots, target_s: float = 12.0, threads: int | None = None):
    """Reference-order sub-step oracle on a bounded particle sample of the same workload."""
    from oracle import oracle as O
    nth = threads or (os.cpu_count() or 1)
    n, dt = 4000, 0.0
    while True:  # calibrate on a sample long enough to hide the fixed per-call overhead
        t0 = time.perf_counter()
        _, st, _ = O.run(prob, knots, scheme="substep", u24=False, nthreads=nth, n_particles=n, pid0=0)
        dt = time.perf_counter() - t0
        if dt > 2.0 or n >= 1_000_000:
            break
        n *= 4
    n2 = int(min(4_000_000, max(n, n * target_s / max(dt, 1e-3))))
    t0 = time.perf_counter()
    _, st, _ = O.run(prob, knots, scheme="substep", u24=False, nthreads=nth, n_particles=n2, pid0=10_000_000)
    dt = time.perf_counter() - t0
    return {"value": st["scatter_events"] / dt, "unit": UNIT, "cores": nth, "kind": "port",
            "sample": f"{n2} of the workload's particles over all 250 time steps, reference sub-step order "
                      f"(h={prob.h:.5g}, {prob.n_sub * prob.n_obs} sub-steps/particle), {dt:.1f} s",
            "events": st["scatter_events"], "seconds": dt}


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
    from oracle import oracle as O
    from radiativetransfermontecarlo_gb300 import build_problem
    from radiativetransfermontecarlo_gb300 import workloads as W
    geo, src, mat, obs, opts = W.c2_elastic3d(precision="fp64")
    prob, grid, N = build_problem(geo, src, mat, obs, dict(opts, exact_count=True))
    knots = O.table_knots(prob.tables)
    nth = os.cpu_count() or 1
    per_step = max(2.0, 120.0 / max(1, args.steps + args.warmup))
    vals, times, events, nparts = [], [], 0, 0
    for i in range(args.warmup + args.steps):
        s = cpu_sample(prob, knots, target_s=per_step, threads=nth)
        if i >= args.warmup:
            vals.append(s["value"])
            times.append(s["seconds"])
            events += s["events"]
            nparts += int(s["sample"].split()[0])
    value = events / sum(times)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000 * float(np.mean(times)), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "sample_particles_per_step": nparts // max(1, args.steps)},
            "impl": "reference",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": nth, "kind": "port",
                             "sample": "each step: a particle sample of the workload sized to a few seconds, "
                                       "reference sub-step algorithm (C restatement), all host threads"},
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
    dev_ms, kern_ms, fold_ms, events, obs_n = [], [], [], 0, 0
    barrier()
    with ClockSampler(device) as clk:
        t_wall = time.perf_counter()
        for _ in range(args.steps):
            ctx.flush_l2()
            st = step(P32)
            dev_ms.append(st["total_ms"])
            kern_ms.append(st["kernel_ms"])
            fold_ms.append(st["fold_ms"])
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
        kmean, fmean = float(np.mean(kern_ms)), float(np.mean(fold_ms))
        entries = N * prob.n_obs  # (particle, observation instant) pairs of one step
        obs_per_step = obs_n / args.steps
        # algorithmic bytes per launch: K1 writes one 4-byte bin index per (particle, instant);
        # K2 reads it back and does one int64 read-modify-write (16 B) per counted observation
        k1_bytes = 4.0 * entries
        k2_bytes = 4.0 * entries + 16.0 * obs_per_step
        traffic = load_traffic()
        kernels = {
            "rt_transport": {"ms": kmean, "algorithmic_bytes": k1_bytes, "achieved_gbs": k1_bytes / kmean / 1e6,
                             "traffic": traffic.get("rt_transport")},
            "rt_bin_slices": {"ms": fmean, "algorithmic_bytes": k2_bytes, "achieved_gbs": k2_bytes / max(fmean, 1e-9) / 1e6,
                              "traffic": traffic.get("rt_bin_slices")},
        }
        dom = max(kernels, key=lambda k: kernels[k]["ms"])
        kd = kernels[dom]
        result = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                  "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
                  "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                  "config": {"workload": WORKLOAD, "particles_per_gpu": n, "histogram_bins": int(prob.hist_len),
                             "l2": "512 MB device write between steps; the 6.9 GB histogram exceeds L2",
                             "wall_s_timed": t_wall},
                  "roofline": {"bound": "hbm", "achieved": kd["achieved_gbs"], "peak": peak, "unit": "GB/s",
                               "frac": kd["achieved_gbs"] / peak, "traffic": kd["traffic"], "kernel": dom,
                               "kernel_ms": kd["ms"], "algorithmic_bytes_per_launch": kd["algorithmic_bytes"],
                               "basis": "K1: 4 B index written per (particle, instant); K2: 4 B read per (particle, "
                                        f"instant) + 16 B int64 read-modify-write per counted observation; peak {peak_kind}",
                               "kernels": kernels},
                  "gpu_launches": args.steps * launches_per_step, "clocks": clocks,
                  "events_per_step": events / args.steps, "observations_per_step": obs_per_step,
                  "transport_ms": kmean, "fold_ms": fmean, "sink": int(st["sink"])}
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
            buf = _lib.PinnedBuffer(prob.hist_len * 8)
            b64 = ctx.copy_histogram(np.empty(prob.hist_len, dtype=np.int64))
            step(P32)
            a32 = ctx.copy_histogram(buf.array(np.int64, prob.hist_len))
            result["rel_l2_energy_density_fp32_vs_fp64"] = rel_l2_density(a32, b64, grid, 1 << 26)
            del b64
    # end to end through the C ABI with host buffers
    if rank == 0 and not args.no_e2e:
        buf = _lib.PinnedBuffer(prob.hist_len * 8)
        out = buf.array(np.int64, prob.hist_len)
        ctx.set_table_cache(False)
        ctx.forward(P32, prob.tables, out)
        times, ev, h2d, d2h = [], 0, 0.0, 0.0
        for _ in range(max(3, args.steps // 4)):
            ctx.flush_l2()
            t0 = time.perf_counter()
            _, st = ctx.forward(P32, prob.tables, out)
            times.append(time.perf_counter() - t0)
            ev += st["scatter_events"]
            h2d, d2h = st["h2d_bytes"], st["d2h_bytes"]
        ctx.set_table_cache(True)
        result["e2e"] = {"value": ev / sum(times), "unit": UNIT, "h2d_bytes_per_step": h2d,
                         "d2h_bytes_per_step": d2h, "ms_per_step": 1000 * float(np.mean(times))}
    if rank == 0 and not args.no_cpu:
        knots = O.table_knots(prob.tables)
        result["cpu_baseline"] = {k: v for k, v in cpu_sample(prob, knots).items() if k not in ("events", "seconds")}
    return result


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
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-accuracy", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    import __graft_entry__
    __graft_entry__.build()
    if args.impl == "reference":
        line = run_reference_arm(args, rank, world)
        if line is not None:
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
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
