"""Generate the golden fixtures of tests/golden/ from the CPU oracle.

The reference (MATLAB) cannot run here, so the fixtures record the oracle's event-order
restatement on small cases of the benchmark configurations (3D acoustic, 3D elastic with
the 4-axis histogram, 2D elastic half-space with Q, a sweep instance) and of the
cylinder boundary, the plane-wave and radial sources and the large-time-step scheme:
sparse histograms and
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
from radiativetransfermontecarlo_gb300 import MaterialClass, build_problem, colon  # noqa: E402
from radiativetransfermontecarlo_gb300 import workloads as W  # noqa: E402


def _cylinder():
    geo = {"dimension": 3, "frame": "cylindrical", "bnd": [{"dir": 4, "val": 1.0}, {"dir": 3, "val": -0.5}]}
    mat = MaterialClass(geo, 5, False, [2, 1.155], [0.2, 0.2, 0.2], [0, 0, 0], "exp", 0.2)
    mat.rho = 1000.0
    mat.Q = 100
    obs = {"x": colon(0, 0.05, 1.0), "z": colon(-0.5, 0.25, 2.0), "time": colon(0, 0.05, 1.5)}
    return geo, {"lambda": 0.05, "position": [0.3, 0, 0], "polarization": "S"}, mat, obs, {"seed": 21}


def _plane():
    geo = {"dimension": 3, "frame": "cartesian"}
    mat = MaterialClass(geo, 10, True, 1, [0.2, 0.2], 0, "exp", 0.1)
    src = {"type": "plane", "direction": [1.0, 2.0, -2.0], "extent": [1.0, 0.5], "lambda": 0.1}
    return geo, src, mat, {"x": colon(-2, 0.1, 3), "y": colon(-2, 0.25, 2), "time": colon(0, 0.05, 1.5)}, {"seed": 22}


def _radial():
    geo = {"dimension": 2, "frame": "cylindrical"}
    mat = MaterialClass(geo, 8, True, 1, [0.2, 0.2], 0, "exp", 0.1)
    src = {"lambda": 0.05, "radial": ([0.0, 0.2, 0.4], [1.0, 0.5, 0.0])}
    return geo, src, mat, {"x": colon(0, 0.05, 3), "time": colon(0, 0.05, 1.5)}, {"seed": 23}


def _large_dt():
    geo, src, mat, obs, opts = W.c1_acoustic3d(precision="fp64")
    mat = MaterialClass(geo, 10, True, 1, [0.2, 0.2], 0, "exp", 0.1)
    mat.timeSteps = 1
    return geo, src, mat, dict(obs, time=colon(0, 0.05, 1.5)), dict(opts, seed=24)


CASES = {
    "c1": (lambda: W.c1_acoustic3d(precision="fp64"), 2000),
    "c2": (lambda: W.c2_elastic3d(precision="fp64"), 1000),
    "c3": (lambda: W.c3_halfspace2d(precision="fp64", t_end=1.0), 500),
    "c4_7": (lambda: W.c4_instance(7), 1000),
    "cylinder": (_cylinder, 1000),
    "plane_source": (_plane, 1000),
    "radial_source": (_radial, 1000),
    "large_dt": (_large_dt, 1000),
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
