"""The MATLAB/Octave gateway mex/rtmc_mex.c, compiled against a plain-memory stand-in for
the MEX API (tests/mex_stub), since neither MATLAB nor Octave is installed.

CPU: the gateway compiles and links against librtmc, reads a complete problem struct,
reports missing fields and bad arguments through mexErrMsgIdAndTxt, and frees what it
allocates.  GPU: its E equals rtmc_forward_u32 through ctypes, bin for bin, on a 3D
acoustic case, the 2D elastic half-space (2x2 knot cell, Zoeppritz tables, boundary) and
a plane-wave source; its gradient branch equals rtmc_gradient.
"""
import ctypes as C
import subprocess
import warnings
from pathlib import Path

import numpy as np
import pytest

from radiativetransfermontecarlo_gb300 import _lib, build_problem, get_context
from radiativetransfermontecarlo_gb300 import workloads as W

ROOT = Path(__file__).resolve().parents[1]
STUB = ROOT / "tests" / "mex_stub"
PKG = ROOT / "radiativetransfermontecarlo_gb300"
SO = STUB / "_build" / "rtmc_mex_stub.so"


def _build():
    srcs = [ROOT / "mex" / "rtmc_mex.c", STUB / "mex_stub.c"]
    if SO.exists() and all(s.stat().st_mtime <= SO.stat().st_mtime for s in srcs + [_lib.LIB_PATH]):
        return SO
    SO.parent.mkdir(exist_ok=True)
    _lib.load()  # librtmc.so must exist
    subprocess.run(["gcc", "-std=c11", "-O2", "-Wall", "-Werror", "-fPIC", "-shared", f"-I{STUB}",
                    f"-I{ROOT / 'include'}", *map(str, srcs), f"-L{PKG}", "-lrtmc", f"-Wl,-rpath,{PKG}",
                    "-o", str(SO), "-lm"], check=True)
    return SO


_mex = None


def mex():
    global _mex
    if _mex is None:
        lib = C.CDLL(str(_build()))
        P = C.c_void_p
        for name, res, args in (("mex_stub_cell", P, [C.c_size_t]), ("mex_stub_set_cell", None, [P, C.c_size_t, P]),
                                ("mex_stub_string", P, [C.c_char_p]), ("mex_stub_struct", P, []),
                                ("mex_stub_doubles", P, [C.c_size_t, C.c_size_t, C.POINTER(C.c_double)]),
                                ("mxSetField", None, [P, C.c_size_t, C.c_char_p, P]),
                                ("mxGetField", P, [P, C.c_size_t, C.c_char_p]),
                                ("mex_stub_call", C.c_int, [C.c_int, C.POINTER(P), C.c_int, C.POINTER(P)]),
                                ("mex_stub_error", C.c_char_p, []), ("mex_stub_class", C.c_int, [P]),
                                ("mxGetData", P, [P]), ("mxGetNumberOfElements", C.c_size_t, [P]),
                                ("mxGetScalar", C.c_double, [P]), ("mxDestroyArray", None, [P]),
                                ("mex_stub_run_atexit", None, []), ("mex_stub_live", C.c_long, [])):
            f = getattr(lib, name)
            f.restype, f.argtypes = res, args
        _mex = lib
    return _mex


def mx_doubles(a, rows=None):
    a = np.asarray(a, dtype=np.float64)
    flat = np.ascontiguousarray(a.ravel(order="F"))
    m, n = (a.shape[0], a.shape[1]) if a.ndim == 2 else ((flat.size, 1) if rows is None else (rows, flat.size // max(rows, 1)))
    return mex().mex_stub_doubles(m, n, flat.ctypes.data_as(C.POINTER(C.c_double)))


def mx_problem(prob):
    """P struct for the gateway: the rtmc_problem fields of a TransportProblem (what
    rtmcProblem.m builds in MATLAB)."""
    M = mex()
    s = M.mex_stub_struct()

    def put(name, v):
        M.mxSetField(s, 0, name.encode(), mx_doubles(np.atleast_1d(np.asarray(v, dtype=float))))
    for k in ("d", "frame", "precision", "src_dir", "polarization", "n_sub", "n_obs", "hist_shift", "max_events",
              "n_particles", "pid0", "seed", "src_lambda", "p2p", "s2s", "h", "time_stride", "mode_stride",
              "hist_len", "src_type", "src_aperture"):
        put(k, getattr(prob, k))
    put("acoustics", int(prob.acoustics))
    put("src_pos", prob.src_pos)
    for k in ("v", "mft", "qrate", "axis_mode", "axis_stride", "src_normal", "src_u", "src_v", "src_extent"):
        put(k, list(getattr(prob, k)))
    if prob.bnd:
        put("bnd_dir", [b[0] for b in prob.bnd])
        put("bnd_val", [b[1] for b in prob.bnd])
        put("bnd_absorb", [int(b[2]) for b in prob.bnd])
    if prob.zoe_rpp is not None:
        put("zoe_rpp", prob.zoe_rpp)
        put("zoe_rsvsv", prob.zoe_rsvsv)
    if prob.src_radial is not None:
        put("src_radial_cdf", prob.src_radial[0])
        put("src_radial_r", prob.src_radial[1])
    return s


def mx_edges(prob):
    M = mex()
    c = M.mex_stub_cell(4)
    for a in range(4):
        e = prob.axis_edges[a]
        M.mex_stub_set_cell(c, a, mx_doubles([] if e is None else e))
    return c


def mx_knots(tables):
    """1x1 or 2x2 cell of [cdf theta] matrices; table t = 2 old + new sits at old + 2 new."""
    M = mex()
    n = tables.info().n_tables
    c = M.mex_stub_cell(n)
    for t in range(n):
        cdf, th = tables.knots(t)
        M.mex_stub_set_cell(c, t if n == 1 else (t // 2) + 2 * (t % 2), mx_doubles(np.stack([cdf, th], axis=1)))
    return c


def call(args, nlhs=1):
    M = mex()
    prhs = (C.c_void_p * len(args))(*args)
    plhs = (C.c_void_p * max(1, nlhs))()
    rc = M.mex_stub_call(nlhs, plhs, len(args), prhs)
    return rc, (M.mex_stub_error().decode() if rc else ""), [plhs[i] for i in range(nlhs)]


def _problem(make, n):
    geo, src, mat, obs, opts = make()
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        prob, grid, N = build_problem(geo, dict(src, numberParticles=n), mat, obs, dict(opts, exact_count=True))
    return prob


def _plane():
    from tests.golden.make_golden import _plane as plane
    return plane()


def test_gateway_reads_problem_and_reports_errors():
    M = mex()
    live0 = M.mex_stub_live()
    prob = _problem(lambda: W.c3_halfspace2d(precision="fp32", t_end=1.0), 100)
    P, E, K = mx_problem(prob), mx_edges(prob), mx_knots(prob.tables)
    cmd = M.mex_stub_string(b"forward")
    rc, err, _ = call([cmd, P])
    assert rc == 1 and err.startswith("rtmc:args"), err
    fly = M.mex_stub_string(b"fly")
    rc, err, _ = call([fly, P, K, E])
    assert rc == 1 and "unknown command" in err
    # a missing required field is named
    Q = M.mex_stub_struct()
    M.mxSetField(Q, 0, b"d", mx_doubles([2.0]))
    rc, err, _ = call([cmd, Q, K, E])
    assert rc == 1 and err.startswith("rtmc:field") and "P.frame" in err, err
    # wrong vector length
    M.mxSetField(P, 0, b"v", mx_doubles([1.0, 2.0, 3.0]))
    rc, err, _ = call([cmd, P, K, E])
    assert rc == 1 and "P.v must hold 2 values" in err, err
    for a in (cmd, fly, P, K, E, Q):
        M.mxDestroyArray(a)
    assert M.mex_stub_live() == live0  # the gateway freed everything it made


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["c1", "c3", "plane"])
def test_gateway_forward_equals_forward_u32(case):
    make = {"c1": lambda: W.c1_acoustic3d(precision="fp32"),
            "c3": lambda: W.c3_halfspace2d(precision="fp32", t_end=1.0), "plane": _plane}[case]
    prob = _problem(make, {"c1": 20000, "c3": 4000, "plane": 5000}[case])
    M = mex()
    P, E, K = mx_problem(prob), mx_edges(prob), mx_knots(prob.tables)
    rc, err, out = call([M.mex_stub_string(b"forward"), P, K, E], nlhs=2)
    assert rc == 0, err
    h, stats = out
    assert M.mex_stub_class(h) == 5  # mxUINT32_CLASS
    n = M.mxGetNumberOfElements(h)
    assert n == prob.hist_len
    E_mex = np.ctypeslib.as_array(C.cast(M.mxGetData(h), C.POINTER(C.c_uint32)), shape=(n,)).copy()
    Pc, keep = prob.to_ctypes()
    E_abi, st = get_context(0).forward_u32(Pc, prob.tables)
    assert np.array_equal(E_mex, E_abi)
    assert E_mex.sum() > 0
    assert M.mxGetScalar(M.mxGetField(stats, 0, b"scatter_events")) == st["scatter_events"]
    for a in (P, E, K, h, stats):
        M.mxDestroyArray(a)


@pytest.mark.gpu
def test_gateway_gradient_equals_rtmc_gradient():
    from radiativetransfermontecarlo_gb300 import adjoint as A
    geo, src, mat, obs, opts = W.c1_acoustic3d(precision="fp32")
    prob = _problem(lambda: (geo, src, mat, obs, opts), 20000)
    prob.qrate = (0.0, 0.0)
    dls, dlS = A.score_tables(mat, 3, ["lc", "cv_kappa", "cv_rho", "mfp"])
    w = np.random.default_rng(3).standard_normal(prob.hist_len)
    M = mex()
    S = M.mex_stub_struct()
    M.mxSetField(S, 0, b"dlogsigma", mx_doubles(np.asarray(dls).T))  # n_theta x n_params
    M.mxSetField(S, 0, b"dlogSigma", mx_doubles(np.asarray(dlS)))
    P, E, K, Wm = mx_problem(prob), mx_edges(prob), mx_knots(prob.tables), mx_doubles(w)
    rc, err, out = call([M.mex_stub_string(b"gradient"), P, K, E, Wm, S])
    assert rc == 0, err
    g_mex = np.ctypeslib.as_array(C.cast(M.mxGetData(out[0]), C.POINTER(C.c_double)), shape=(len(dlS),)).copy()
    Pc, keep = prob.to_ctypes()
    g_abi, st = get_context(0).gradient(Pc, prob.tables, dls, dlS, w)
    assert np.array_equal(g_mex, g_abi)
    rc, err, _ = call([M.mex_stub_string(b"reset")], nlhs=0)
    assert rc == 0
    M.mex_stub_run_atexit()
