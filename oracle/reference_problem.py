"""The 3D elastic benchmark problem (1e7 particles, cartesian 60^3 x 8 directions x 251
times x 2 modes) set up for the oracle without the product library.

TEST INFRASTRUCTURE ONLY: bench.py's reference arm times the oracle on this problem, so
the arm loads no product code at all.  The tables come from tables_ref.prepare_sigma
(the NumPy restatement of prepareSigma, MaterialClass.m:2379-2463); the observation grid
restates initializeObservation.m:9-133 for a cartesian 3D frame with the direction axis
(psi edges = cos(directions) reversed, :64-66) and the mode axis; the sub-step restates
propagateParticleSmallDt.m:4-7 (h = dt / ceil(dt / min(0.01 min(mft), dt))).
"""
from __future__ import annotations

import math
from types import SimpleNamespace

import numpy as np

from . import tables_ref as T


def matlab_colon(a: float, step: float, b: float) -> np.ndarray:
    """a:step:b as MATLAB builds it: both ends exact, the middle symmetric."""
    n = int(math.floor((b - a) / step + 1e-10))
    k = np.arange(n + 1, dtype=float)
    return np.where(k < n / 2, a + k * step, (a + n * step) - (n - k) * step)


def c2_problem(n_particles: int = 10_000_000, seed: int = 1, hist_shift: int = 40):
    """(problem namespace for oracle.run, knots [(cdf, theta)] x 4) of the 3D elastic case:
    vp 2, vs 1.155, cv 0.1 x 3, corr 0, gaussian lc 0.2, f 5, Q Inf, P point source at the
    origin with lambda 0.05, edges -5:1/6:5 on x, y, z, directions 0:pi/8:pi, time 0:0.02:5."""
    tab = T.prepare_sigma(3, False, 5.0, [2.0, 1.155], [0.1, 0.1, 0.1], [0.0, 0.0, 0.0], "gaussian", 0.2)
    mft = tuple(float(x) for x in tab["meanFreeTime"])
    e = matlab_colon(-5.0, 1.0 / 6.0, 5.0)
    psi = np.cos(matlab_colon(0.0, math.pi / 8, math.pi))[::-1].copy()
    time = matlab_colon(0.0, 0.02, 5.0)
    Nt = time.size  # t = 0 is part of the grid and never filled (radiativeTransfer.m:72)
    dt = float(np.mean(np.diff(time)))
    n_sub = int(math.ceil(dt / min(0.01 * min(mft), dt)))
    nb = [e.size - 1, e.size - 1, e.size - 1, psi.size - 1]
    stride = [1, nb[0], nb[0] * nb[1], nb[0] * nb[1] * nb[2]]
    time_stride = stride[3] * nb[3]
    mode_stride = time_stride * Nt
    prob = SimpleNamespace(
        d=3, frame=0, acoustics=False, precision=1, src_dir=0, polarization=0, n_sub=n_sub, n_obs=Nt - 1,
        n_particles=n_particles, pid0=0, seed=seed, src_pos=(0.0, 0.0, 0.0), src_lambda=0.05, v=(2.0, 1.155),
        mft=mft, p2p=float(tab["P2P"]), s2s=float(tab["S2S"]), qrate=(0.0, 0.0), h=dt / n_sub,
        axis_mode=[2, 2, 2, 2], axis_edges=[e, e, e, psi], axis_stride=stride, time_stride=time_stride,
        mode_stride=mode_stride, hist_len=2 * mode_stride, hist_shift=hist_shift, bnd=[], zoe_rpp=None,
        zoe_rsvsv=None, src_type=0, src_aperture=0, src_radial=None)
    return prob, tab["tables"]
