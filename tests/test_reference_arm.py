"""The reference arm's problem (oracle/reference_problem.py) matches the product's set-up
of the same workload, so the timed CPU baseline runs the benchmark configuration, yet
loads no product code."""
import subprocess
import sys
import warnings
from pathlib import Path

import numpy as np

from oracle import reference_problem as RP

ROOT = Path(__file__).resolve().parents[1]


def test_reference_problem_matches_product_setup():
    from radiativetransfermontecarlo_gb300 import build_problem
    from radiativetransfermontecarlo_gb300 import workloads as W
    prob, knots = RP.c2_problem()
    geo, src, mat, obs, opts = W.c2_elastic3d(precision="fp64")
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        ours, grid, N = build_problem(geo, src, mat, obs, dict(opts, exact_count=True))
    for k in ("d", "frame", "acoustics", "src_dir", "polarization", "n_sub", "n_obs", "n_particles", "seed",
              "axis_mode", "axis_stride", "time_stride", "mode_stride", "hist_len", "hist_shift"):
        assert getattr(prob, k) == getattr(ours, k), k
    for k in ("h", "p2p", "s2s", "src_lambda"):
        assert abs(getattr(prob, k) - getattr(ours, k)) <= 1e-12 * abs(getattr(ours, k)), k
    assert np.allclose(prob.mft, ours.mft, rtol=1e-9)
    for a in range(4):
        assert np.allclose(prob.axis_edges[a], ours.axis_edges[a], rtol=0, atol=1e-12)
    mine = [ours.tables.knots(i) for i in range(4)]
    for (c, t), (c2, t2) in zip(knots, mine):
        assert abs(c.size - c2.size) <= 2
        u = np.linspace(0.01, 0.99, 999)
        from oracle.tables_ref import invcdf
        assert np.max(np.abs(invcdf(c, t, u) - invcdf(c2, t2, u))) < 1e-6


def test_reference_arm_loads_no_product_code():
    """--impl reference on a tiny sample maps only the oracle's library."""
    code = ("import sys, json;"
            "sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '0', '--ref-seconds', '0.5'];"
            "import bench;"
            "bench.main();"
            "maps = open('/proc/self/maps').read();"
            "assert 'librtmc' not in maps, 'product library mapped';"
            "assert 'radiativetransfermontecarlo_gb300' not in sys.modules")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    line = [ln for ln in r.stdout.splitlines() if ln.startswith("{")][-1]
    import json
    d = json.loads(line)
    assert d["impl"] == "reference" and d["value"] > 0
