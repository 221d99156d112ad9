"""Generate the golden fixtures of tests/golden/ from the CPU oracle.

The reference (MATLAB) cannot run here, so the fixtures record the oracle's event-order
restatement on three small cases of the benchmark configurations (3D acoustic, 3D
elastic with the 4-axis histogram, 2D elastic half-space with Q): sparse histograms and
the final state of the first particles, for both uniform widths (32-bit: the FP64 GPU
stream; 24-bit: the FP32 GPU stream).  Run from the repository root:

    python tests/golden/make_golden.py
"""
import platform
import sys
import warnings
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import oracle as O  # noqa: E402
from radiativetransfermontecarlo_gb300 import build_problem  # noqa: E402
from radiativetransfermontecarlo_gb300 import workloads as W  # noqa: E402

CASES = {
    "c1": (lambda: W.c1_acoustic3d(precision="fp64"), 2000),
    "c2": (lambda: W.c2_elastic3d(precision="fp64"), 1000),
    "c3": (lambda: W.c3_halfspace2d(precision="fp64", t_end=1.0), 500),
}
N_STATES = 200


def case_problem(name, precision):
    make, n = CASES[name]
    geo, src, mat, obs, opts = make()
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        prob, grid, N = build_problem(geo, dict(src, numberParticles=n), mat, obs,
                                      dict(opts, exact_count=True, precision=precision))
    return prob, grid


def main():
    out = {}
    for name in CASES:
        for precision in ("fp64", "fp32"):
            prob, grid = case_problem(name, precision)
            hist, stats, states = O.run(prob, O.table_knots(prob.tables), scheme="event", want_state=True, nthreads=1)
            nz = np.nonzero(hist)[0]
            key = f"{name}_{precision}"
            out[key + "_idx"] = nz.astype(np.int64)
            out[key + "_val"] = hist[nz]
            out[key + "_states"] = states[:N_STATES]
            out[key + "_stats"] = np.array([stats[k] for k in O.ST_NAMES], dtype=np.int64)
    out["machine"] = np.array(platform.machine())
    np.savez_compressed(Path(__file__).resolve().parent / "oracle_event.npz", **out)


if __name__ == "__main__":
    main()
