"""ctypes wrapper of the C oracle (oracle/rtmc_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline leg, as the checker.  The product library never calls it.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "rtmc_oracle.c"
LIB = HERE / "_build" / "liboracle.so"

ST_NAMES = ("scatter_events", "boundary_hits", "kills", "absorbed", "observations", "conversions")


def build(force: bool = False) -> Path:
    """gcc -O2 -fopenmp; FMA contraction off so x86 and Arm builds give the same bits."""
    if not force and LIB.exists() and LIB.stat().st_mtime >= SRC.stat().st_mtime:
        return LIB
    LIB.parent.mkdir(exist_ok=True)
    tmp = LIB.with_suffix(".tmp.so")
    subprocess.run(["gcc", "-O2", "-std=c11", "-D_GNU_SOURCE", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared",
                    str(SRC), "-o", str(tmp), "-lm"], check=True)
    os.replace(tmp, LIB)
    return LIB


class OracleProblem(C.Structure):
    _fields_ = [("d", C.c_int32), ("frame", C.c_int32), ("acoustics", C.c_int32), ("scheme", C.c_int32),
                ("ufloat", C.c_int32), ("src_dir", C.c_int32), ("polarization", C.c_int32), ("n_sub", C.c_int32),
                ("n_obs", C.c_int32), ("n_bnd", C.c_int32), ("hist_shift", C.c_int32), ("nthreads", C.c_int32),
                ("n_particles", C.c_int64), ("pid0", C.c_int64), ("seed", C.c_uint64),
                ("src_pos", C.c_double * 3), ("src_lambda", C.c_double), ("v", C.c_double * 2),
                ("mft", C.c_double * 2), ("p2p", C.c_double), ("s2s", C.c_double), ("qrate", C.c_double * 2),
                ("h", C.c_double), ("axis_mode", C.c_int32 * 4), ("axis_nedges", C.c_int32 * 4),
                ("axis_edges", C.POINTER(C.c_double) * 4), ("axis_stride", C.c_int64 * 4),
                ("time_stride", C.c_int64), ("mode_stride", C.c_int64), ("hist_len", C.c_int64),
                ("bnd_dir", C.c_int32 * 4), ("bnd_absorb", C.c_int32 * 4), ("bnd_val", C.c_double * 4),
                ("zoe_rpp", C.POINTER(C.c_double)), ("zoe_rsvsv", C.POINTER(C.c_double)),
                ("tab_n", C.c_int64 * 4), ("tab_cdf", C.POINTER(C.c_double) * 4),
                ("tab_theta", C.POINTER(C.c_double) * 4), ("src_type", C.c_int32), ("src_aperture", C.c_int32),
                ("src_radial_n", C.c_int64), ("src_radial_cdf", C.POINTER(C.c_double)),
                ("src_radial_r", C.POINTER(C.c_double)), ("src_normal", C.c_double * 3), ("src_u", C.c_double * 3),
                ("src_v", C.c_double * 3), ("src_extent", C.c_double * 2),
                ("cross_margin", C.POINTER(C.c_double))]


_lib = None


def load():
    global _lib
    if _lib is None:
        lib = C.CDLL(str(build()))
        lib.oracle_run.restype = C.c_int
        lib.oracle_run.argtypes = [C.POINTER(OracleProblem), C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                   C.POINTER(C.c_double)]
        lib.oracle_philox4x32_10.restype = None
        lib.oracle_philox4x32_10.argtypes = [C.POINTER(C.c_uint32)] * 3
        lib.oracle_invcdf.restype = C.c_double
        lib.oracle_invcdf.argtypes = [C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_int64, C.c_double]
        lib.oracle_max_threads.restype = C.c_int
        lib.oracle_gradient.restype = C.c_int
        lib.oracle_gradient.argtypes = [C.POINTER(OracleProblem), C.POINTER(C.c_double), C.POINTER(C.c_double),
                                        C.c_int, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                        C.POINTER(C.c_double), C.POINTER(C.c_int64)]
        lib.oracle_reflect.restype = C.c_int
        lib.oracle_reflect.argtypes = [C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_double, C.c_double, C.c_int,
                                       C.c_int64, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                       C.POINTER(C.c_int32), C.POINTER(C.c_double)]
        _lib = lib
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def philox(ctr, key):
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    load().oracle_philox4x32_10(c, k, o)
    return list(o)


def run(prob, knots, scheme: str = "event", ufloat: bool | None = None, nthreads: int | None = None,
        n_particles: int | None = None, pid0: int | None = None, want_state: bool = False,
        hist: np.ndarray | None = None, margins: np.ndarray | None = None):
    """Run the oracle on a TransportProblem-like object with the given table knots
    [(cdf, theta), ...].  scheme 'substep' (reference order) or 'event' (snap, GPU stream).
    hist, if given, is an int64 array of hist_len that the run adds into (timing runs
    reuse one, so allocation and first-touch page faults stay out of the particles' time).
    margins, if given, is a float64 array of n_particles that the event scheme fills with
    each particle's smallest plane-crossing margin (distance of the deciding sub-step
    position from the plane; inf without crossings).
    Returns (int64 histogram, stats dict, final states [N,16] or None)."""
    lib = load()
    P, keep = _problem(prob, knots, scheme, ufloat, nthreads, n_particles, pid0)
    if margins is not None:
        if margins.dtype != np.float64 or margins.size != P.n_particles or not margins.flags.c_contiguous:
            raise ValueError("margins must be a contiguous float64 array of n_particles")
        P.cross_margin = _dp(margins)
    if hist is None:
        hist = np.zeros(prob.hist_len, dtype=np.int64)
    elif hist.dtype != np.int64 or hist.size != prob.hist_len or not hist.flags.c_contiguous:
        raise ValueError("hist must be a contiguous int64 array of hist_len")
    stats = np.zeros(8, dtype=np.int64)
    fs = np.zeros((P.n_particles, 16)) if want_state else None
    rc = lib.oracle_run(C.byref(P), hist.ctypes.data_as(C.POINTER(C.c_int64)),
                        stats.ctypes.data_as(C.POINTER(C.c_int64)), _dp(fs) if want_state else None)
    if rc:
        raise RuntimeError(f"oracle_run failed ({rc})")
    return hist, dict(zip(ST_NAMES, map(int, stats[:6]))), fs


def gradient(prob, knots, dlogsigma, dlogSigma, adjoint, ufloat: bool | None = None, nthreads: int | None = None):
    """Score-function gradient by the event scheme (the restatement of rtmc_gradient):
    returns (grad [n_params], stats).  prob must be acoustic with qrate = 0."""
    lib = load()
    P, keep = _problem(prob, knots, "event", ufloat, nthreads, None, None)
    dls = np.ascontiguousarray(dlogsigma, dtype=np.float64)
    adj = np.ascontiguousarray(adjoint, dtype=np.float64).ravel()
    hS = prob.h / prob.mft[0] if math.isfinite(prob.mft[0]) else 0.0
    kappa = hS / math.expm1(hS) if hS > 0 else 1.0
    dlS = np.asarray(dlogSigma, dtype=np.float64)
    a_inc = np.ascontiguousarray(dlS * (kappa - 1.0 + hS))
    b_obs = np.ascontiguousarray(-dlS * hS * prob.n_sub)
    grad = np.zeros(dls.shape[0])
    stats = np.zeros(8, dtype=np.int64)
    rc = lib.oracle_gradient(C.byref(P), _dp(adj), _dp(dls), dls.shape[0], dls.shape[1], _dp(a_inc), _dp(b_obs),
                             _dp(grad), stats.ctypes.data_as(C.POINTER(C.c_int64)))
    if rc:
        raise RuntimeError(f"oracle_gradient failed ({rc})")
    return grad, dict(zip(ST_NAMES, map(int, stats[:6])))


def _problem(prob, knots, scheme, ufloat, nthreads, n_particles, pid0):
    lib = load()
    P = OracleProblem()
    P.d, P.frame, P.acoustics = prob.d, prob.frame, int(prob.acoustics)
    P.scheme = 0 if scheme == "substep" else 1
    P.ufloat = int(prob.precision == 0) if ufloat is None else int(ufloat)
    P.src_dir, P.polarization, P.n_sub, P.n_obs = prob.src_dir, prob.polarization, prob.n_sub, prob.n_obs
    P.n_bnd, P.hist_shift = len(prob.bnd), prob.hist_shift
    P.nthreads = nthreads or max(1, lib.oracle_max_threads())
    P.n_particles = prob.n_particles if n_particles is None else n_particles
    P.pid0 = prob.pid0 if pid0 is None else pid0
    P.seed = prob.seed
    for i in range(3):
        P.src_pos[i] = prob.src_pos[i]
    P.src_lambda = prob.src_lambda
    for m in range(2):
        P.v[m] = prob.v[m]
        P.mft[m] = prob.mft[m]
        P.qrate[m] = prob.qrate[m]
    P.p2p, P.s2s, P.h = prob.p2p, prob.s2s, prob.h
    keep = []
    for a in range(4):
        # the oracle range-checks every integrated axis as the reference does
        mode = prob.axis_mode[a]
        e = prob.axis_edges[a]
        if mode == 0 and e is not None and not (prob.d == 2 and a == 2):
            mode = 1
        P.axis_mode[a] = mode
        if mode:
            ea = np.ascontiguousarray(e, dtype=np.float64)
            keep.append(ea)
            P.axis_nedges[a] = ea.size
            P.axis_edges[a] = _dp(ea)
        P.axis_stride[a] = prob.axis_stride[a]
    P.time_stride, P.mode_stride, P.hist_len = prob.time_stride, prob.mode_stride, prob.hist_len
    for b, (bd, bv, ab) in enumerate(prob.bnd):
        P.bnd_dir[b], P.bnd_val[b], P.bnd_absorb[b] = bd, bv, int(ab)
    if prob.zoe_rpp is not None:
        zr = np.ascontiguousarray(prob.zoe_rpp, dtype=np.float64)
        zs = np.ascontiguousarray(prob.zoe_rsvsv, dtype=np.float64)
        keep += [zr, zs]
        P.zoe_rpp, P.zoe_rsvsv = _dp(zr), _dp(zs)
    P.src_type = getattr(prob, "src_type", 0)
    P.src_aperture = getattr(prob, "src_aperture", 0)
    for i in range(3):
        P.src_normal[i] = getattr(prob, "src_normal", (0.0, 0.0, 1.0))[i]
        P.src_u[i] = getattr(prob, "src_u", (1.0, 0.0, 0.0))[i]
        P.src_v[i] = getattr(prob, "src_v", (0.0, 1.0, 0.0))[i]
    P.src_extent[0], P.src_extent[1] = getattr(prob, "src_extent", (0.0, 0.0))
    radial = getattr(prob, "src_radial", None)
    if radial is not None:
        rc = np.ascontiguousarray(radial[0], dtype=np.float64)
        rr = np.ascontiguousarray(radial[1], dtype=np.float64)
        keep += [rc, rr]
        P.src_radial_n = rc.size
        P.src_radial_cdf, P.src_radial_r = _dp(rc), _dp(rr)
    for i, (c, t) in enumerate(knots):
        c = np.ascontiguousarray(c, dtype=np.float64)
        t = np.ascontiguousarray(t, dtype=np.float64)
        keep += [c, t]
        P.tab_n[i] = c.size
        P.tab_cdf[i] = _dp(c)
        P.tab_theta[i] = _dp(t)
    return P, keep


def reflect(zoe_rpp, zoe_rsvsv, vp, vs, k, d, q, mode, u):
    """Elastic reflection of n particles at the plane normal to e_k (k = 0, 1, 2), or at a
    cylinder wall with outward normal e_x (k = 3); test entry of the oracle."""
    d = np.ascontiguousarray(d, dtype=np.float64).copy()
    q = np.ascontiguousarray(q, dtype=np.float64).copy()
    mode = np.ascontiguousarray(mode, dtype=np.int32).copy()
    zr = np.ascontiguousarray(zoe_rpp, dtype=np.float64)
    zs = np.ascontiguousarray(zoe_rsvsv, dtype=np.float64)
    u = np.ascontiguousarray(u, dtype=np.float64)
    rc = load().oracle_reflect(_dp(zr), _dp(zs), vp, vs, k, len(mode), _dp(d), _dp(q),
                               mode.ctypes.data_as(C.POINTER(C.c_int32)), _dp(u))
    if rc:
        raise RuntimeError("oracle_reflect failed")
    return d, q, mode


def table_knots(tables) -> list:
    """[(cdf, theta)] of a product tables handle, to feed both sides the same tables."""
    n = tables.info().n_tables
    return [tables.knots(i) for i in range(n)]
