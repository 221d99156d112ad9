"""ctypes binding of librtmc.so (the C ABI declared in include/rtmc.h).

The library is built in-tree by radiativetransfermontecarlo_gb300.build; loading fails
loudly when it is missing.  There is no CPU fallback for the transport.
"""
from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "librtmc.so"

RTMC_OK = 0
PSDF = {"exp": 0, "gaussian": 1, "power_law": 2, "triangular": 3, "low_pass": 4, "VonKarman": 5, "const": 6}
FRAME = {"cartesian": 0, "cylindrical": 1, "spherical": 2}
AXIS_IGNORED, AXIS_RANGE, AXIS_BINNED = 0, 1, 2
FP32, FP64 = 0, 1
ZOE_N = 181
MAX_BND = 4
MAX_RADIAL = 65536
SOURCE_POINT, SOURCE_PLANE = 0, 1
APERTURE_RECTANGLE, APERTURE_CIRCLE = 0, 1


class RtmcMaterial(C.Structure):
    _fields_ = [("d", C.c_int32), ("acoustics", C.c_int32), ("psdf", C.c_int32), ("reserved", C.c_int32),
                ("freq", C.c_double), ("v", C.c_double * 2), ("cv", C.c_double * 3), ("corr", C.c_double * 3),
                ("lc", C.c_double), ("nu", C.c_double), ("sigma_const", C.c_double * 4), ("n_theta", C.c_int64)]


class RtmcTablesInfo(C.Structure):
    _fields_ = [("n_tables", C.c_int32), ("reserved", C.c_int32), ("n_knots", C.c_int64 * 4),
                ("Sigma", C.c_double * 4), ("Sigmapr", C.c_double * 4), ("mean_free_time", C.c_double * 2),
                ("p2p", C.c_double), ("s2s", C.c_double), ("diffusivity", C.c_double),
                ("transport_mean_free_path", C.c_double * 2), ("g", C.c_double)]


class RtmcProblem(C.Structure):
    _fields_ = [("d", C.c_int32), ("frame", C.c_int32), ("acoustics", C.c_int32), ("precision", C.c_int32),
                ("src_dir", C.c_int32), ("polarization", C.c_int32), ("n_sub", C.c_int32), ("n_obs", C.c_int32),
                ("n_bnd", C.c_int32), ("hist_shift", C.c_int32), ("max_events", C.c_int32), ("reserved", C.c_int32),
                ("n_particles", C.c_int64), ("pid0", C.c_int64), ("seed", C.c_uint64),
                ("src_pos", C.c_double * 3), ("src_lambda", C.c_double), ("v", C.c_double * 2),
                ("mft", C.c_double * 2), ("p2p", C.c_double), ("s2s", C.c_double), ("qrate", C.c_double * 2),
                ("h", C.c_double), ("axis_mode", C.c_int32 * 4), ("axis_nedges", C.c_int32 * 4),
                ("axis_edges", C.POINTER(C.c_double) * 4), ("axis_stride", C.c_int64 * 4),
                ("time_stride", C.c_int64), ("mode_stride", C.c_int64), ("hist_len", C.c_int64),
                ("bnd_dir", C.c_int32 * MAX_BND), ("bnd_absorb", C.c_int32 * MAX_BND),
                ("bnd_val", C.c_double * MAX_BND), ("zoe_rpp", C.c_double * ZOE_N),
                ("zoe_rsvsv", C.c_double * ZOE_N), ("src_type", C.c_int32), ("src_aperture", C.c_int32),
                ("src_radial_n", C.c_int32), ("reserved2", C.c_int32), ("src_radial_cdf", C.POINTER(C.c_double)),
                ("src_radial_r", C.POINTER(C.c_double)), ("src_normal", C.c_double * 3), ("src_u", C.c_double * 3),
                ("src_v", C.c_double * 3), ("src_extent", C.c_double * 2)]


class RtmcStats(C.Structure):
    _fields_ = [("scatter_events", C.c_int64), ("boundary_hits", C.c_int64), ("kills", C.c_int64),
                ("absorbed", C.c_int64), ("observations", C.c_int64), ("conversions", C.c_int64),
                ("device_status", C.c_int64), ("launches", C.c_int32), ("sink", C.c_int32),
                ("kernel_ms", C.c_double), ("fold_ms", C.c_double),
                ("total_ms", C.c_double), ("h2d_bytes", C.c_double), ("d2h_bytes", C.c_double),
                ("events_ms", C.c_double), ("convert_ms", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "reserved"}


MAX_PARAMS = 8


class RtmcScore(C.Structure):
    _fields_ = [("n_params", C.c_int32), ("n_theta", C.c_int32), ("dlogsigma", C.POINTER(C.c_double)),
                ("dlogSigma", C.c_double * MAX_PARAMS)]


# every function declared in include/rtmc.h: name -> (restype, argtypes)
_P = C.c_void_p
SIGNATURES = {
    "rtmc_tables_build": (C.c_int, [C.POINTER(RtmcMaterial), C.POINTER(_P)]),
    "rtmc_tables_from_knots": (C.c_int, [C.c_int32, C.POINTER(C.c_int64), C.POINTER(C.POINTER(C.c_double)),
                                         C.POINTER(C.POINTER(C.c_double)), C.POINTER(_P)]),
    "rtmc_tables_get_info": (C.c_int, [_P, C.POINTER(RtmcTablesInfo)]),
    "rtmc_tables_get_knots": (C.c_int, [_P, C.c_int32, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "rtmc_tables_eval": (C.c_int, [_P, C.c_int32, C.c_int64, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "rtmc_tables_free": (None, [_P]),
    "rtmc_sigma_eval": (C.c_int, [C.POINTER(RtmcMaterial), C.c_int32, C.c_int64, C.POINTER(C.c_double),
                                  C.POINTER(C.c_double)]),
    "rtmc_sigma_total": (C.c_int, [C.POINTER(RtmcMaterial), C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "rtmc_gradient": (C.c_int, [_P, C.POINTER(RtmcProblem), _P, C.POINTER(RtmcScore), C.POINTER(C.c_double),
                                C.POINTER(C.c_double), C.POINTER(RtmcStats)]),
    "rtmc_zoeppritz_fluid": (C.c_int, [C.c_int32, C.POINTER(C.c_double), C.c_double, C.c_double, C.c_double,
                                       C.c_double, C.c_double, C.c_double, C.POINTER(C.c_double)]),
    "rtmc_create": (C.c_int, [C.c_int32, C.POINTER(_P)]),
    "rtmc_destroy": (None, [_P]),
    "rtmc_last_error": (C.c_char_p, [_P]),
    "rtmc_abi_version": (C.c_int32, []),
    "rtmc_abi_sizes": (C.c_int, [C.POINTER(C.c_int64)]),
    "rtmc_forward": (C.c_int, [_P, C.POINTER(RtmcProblem), _P, C.POINTER(C.c_int64), C.POINTER(RtmcStats)]),
    "rtmc_forward_u32": (C.c_int, [_P, C.POINTER(RtmcProblem), _P, C.POINTER(C.c_uint32), C.POINTER(RtmcStats)]),
    "rtmc_forward_trace": (C.c_int, [_P, C.POINTER(RtmcProblem), _P, C.POINTER(C.c_int64), C.POINTER(C.c_double),
                                     C.POINTER(RtmcStats)]),
    "rtmc_forward_device": (C.c_int, [_P, C.POINTER(RtmcProblem), _P, C.POINTER(RtmcStats)]),
    "rtmc_copy_histogram": (C.c_int, [_P, C.POINTER(C.c_int64), C.c_int64]),
    "rtmc_histogram_device": (C.c_int, [_P, C.POINTER(C.c_void_p), C.POINTER(C.c_int64)]),
    "rtmc_forward_noalloc": (C.c_int, [C.POINTER(RtmcProblem), _P, C.c_void_p, C.c_void_p, C.POINTER(RtmcStats)]),
    "rtmc_host_alloc": (C.c_int, [C.c_int64, C.POINTER(_P)]),
    "rtmc_host_free": (C.c_int, [_P]),
    "rtmc_flush_l2": (C.c_int, [_P]),
    "rtmc_set_table_cache": (C.c_int, [_P, C.c_int32]),
    "rtmc_set_fp64_estimate": (C.c_int, [_P, C.c_int32]),
    "rtmc_set_early_copy": (C.c_int, [_P, C.c_int32]),
    "rtmc_set_particle_order": (C.c_int, [_P, C.c_int32]),
    "rtmc_set_launch": (C.c_int, [_P, C.c_int32, C.c_int32, C.c_int32]),
    "rtmc_set_pipeline": (C.c_int, [_P, C.c_int32, C.c_int32]),
    "rtmc_set_schedule": (C.c_int, [_P, C.c_int32]),
    "rtmc_set_fold": (C.c_int, [_P, C.c_int32]),
    "rtmc_batch_create": (C.c_int, [_P, C.c_int32, C.POINTER(RtmcProblem), C.POINTER(_P), C.POINTER(_P)]),
    "rtmc_batch_set_launch": (C.c_int, [_P, C.c_int32, C.c_int32, C.c_int64]),
    "rtmc_batch_set_em_histogram": (C.c_int, [_P, C.c_int32]),
    "rtmc_batch_set_schedule": (C.c_int, [_P, C.POINTER(C.c_int32)]),
    "rtmc_batch_run": (C.c_int, [_P, C.POINTER(RtmcStats)]),
    "rtmc_batch_histograms": (C.c_int, [_P, C.c_int32, C.c_int32, C.POINTER(C.c_int64)]),
    "rtmc_batch_schedule": (C.c_int, [_P, C.POINTER(C.c_int32)]),
    "rtmc_batch_destroy": (None, [_P]),
    "rtmc_last_timing": (C.c_int, [_P, C.POINTER(C.c_double), C.POINTER(C.c_int32)]),
    "rtmc_probe_l2_reductions": (C.c_int, [_P, C.POINTER(C.c_double)]),
}

_lock = threading.Lock()
_lib = None


class RtmcError(RuntimeError):
    pass


def load():
    """Load librtmc.so; raises when it has not been built."""
    global _lib
    with _lock:
        if _lib is None:
            if not LIB_PATH.exists():
                raise RtmcError(f"{LIB_PATH} is missing: build it with "
                                "`python -c 'import __graft_entry__ as g; g.build()'`")
            lib = C.CDLL(str(LIB_PATH))
            for name, (res, args) in SIGNATURES.items():
                f = getattr(lib, name)
                f.restype = res
                f.argtypes = args
            sizes = (C.c_int64 * 4)()
            lib.rtmc_abi_sizes(sizes)
            mine = [C.sizeof(RtmcMaterial), C.sizeof(RtmcTablesInfo), C.sizeof(RtmcProblem), C.sizeof(RtmcStats)]
            if list(sizes) != mine:
                raise RtmcError(f"librtmc ABI mismatch: library {list(sizes)} vs binding {mine}")
            _lib = lib
        return _lib


def check(status: int, ctx=None):
    if status != RTMC_OK:
        msg = load().rtmc_last_error(ctx)
        raise RtmcError(f"librtmc error {status}: {msg.decode() if msg else ''}")


def _need(ok: bool, what: str):
    """Argument check that survives python -O: the library writes through these buffers."""
    if not ok:
        raise ValueError(what)


def dptr(a: np.ndarray):
    _need(a.dtype == np.float64 and a.flags.c_contiguous, "expected a contiguous float64 array")
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Tables:
    """Owning handle of rtmc_tables (host FP64 inverse-CDF knots)."""

    def __init__(self, handle: int):
        self.handle = C.c_void_p(handle)

    @classmethod
    def build(cls, mat: RtmcMaterial) -> "Tables":
        lib = load()
        h = C.c_void_p()
        check(lib.rtmc_tables_build(C.byref(mat), C.byref(h)))
        return cls(h.value)

    @classmethod
    def from_knots(cls, knots) -> "Tables":
        lib = load()
        n = len(knots)
        cs = [np.ascontiguousarray(c, dtype=np.float64) for c, _ in knots]
        ts = [np.ascontiguousarray(t, dtype=np.float64) for _, t in knots]
        _need(all(c.ndim == 1 and c.shape == t.shape for c, t in zip(cs, ts)),
              "each table needs as many theta values as CDF knots")
        nk = (C.c_int64 * n)(*[len(c) for c in cs])
        cp = (C.POINTER(C.c_double) * n)(*[dptr(c) for c in cs])
        tp = (C.POINTER(C.c_double) * n)(*[dptr(t) for t in ts])
        h = C.c_void_p()
        check(lib.rtmc_tables_from_knots(n, nk, cp, tp, C.byref(h)))
        return cls(h.value)

    def info(self) -> RtmcTablesInfo:
        inf = RtmcTablesInfo()
        check(load().rtmc_tables_get_info(self.handle, C.byref(inf)))
        return inf

    def knots(self, t: int):
        n = self.info().n_knots[t]
        c = np.empty(n)
        th = np.empty(n)
        check(load().rtmc_tables_get_knots(self.handle, t, dptr(c), dptr(th)))
        return c, th

    def eval(self, t: int, u) -> np.ndarray:
        u = np.ascontiguousarray(u, dtype=np.float64)
        out = np.empty_like(u)
        check(load().rtmc_tables_eval(self.handle, t, u.size, dptr(u), dptr(out)))
        return out

    def __del__(self):
        if getattr(self, "handle", None) and self.handle.value and _lib is not None:
            _lib.rtmc_tables_free(self.handle)
            self.handle = C.c_void_p()


def zoeppritz_fluid(angles_deg, vp1, vs1, rho1, vp2=343.0, vs2=0.0, rho2=1.0) -> dict:
    a = np.ascontiguousarray(angles_deg, dtype=np.float64)
    out = np.empty(7 * a.size)
    check(load().rtmc_zoeppritz_fluid(a.size, dptr(a), vp1, vs1, rho1, vp2, vs2, rho2, dptr(out)))
    out = out.reshape(7, a.size)
    keys = ("E_Rpp", "E_Rpsv", "E_Tpp", "E_Rsvsv", "E_Rsp", "E_Tsp", "E_Rsh")
    return {k: out[i].copy() for i, k in enumerate(keys)}


class Context:
    """A librtmc context on one CUDA device (owns its stream and device buffers)."""

    def __init__(self, device: int = 0):
        self.lib = load()
        h = C.c_void_p()
        check(self.lib.rtmc_create(device, C.byref(h)))
        self.handle = h
        self.device = device

    def close(self):
        if self.handle and self.handle.value:
            self.lib.rtmc_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def forward(self, problem: RtmcProblem, tables: Tables, out: np.ndarray | None = None):
        """Run the transport; returns (int64 histogram on the host, stats dict)."""
        if out is None:
            out = np.empty(problem.hist_len, dtype=np.int64)
        _need(out.dtype == np.int64 and out.size >= problem.hist_len and out.flags.c_contiguous,
              "out must be a contiguous int64 array of at least hist_len elements")
        st = RtmcStats()
        check(self.lib.rtmc_forward(self.handle, C.byref(problem), tables.handle,
                                    out.ctypes.data_as(C.POINTER(C.c_int64)), C.byref(st)), self.handle)
        return out, st.as_dict()

    def forward_u32(self, problem: RtmcProblem, tables: Tables, out: np.ndarray | None = None):
        """rtmc_forward_u32: (uint32 counts on the host, saturating like the reference's E;
        stats dict)."""
        if out is None:
            out = np.empty(problem.hist_len, dtype=np.uint32)
        _need(out.dtype == np.uint32 and out.size >= problem.hist_len and out.flags.c_contiguous,
              "out must be a contiguous uint32 array of at least hist_len elements")
        st = RtmcStats()
        check(self.lib.rtmc_forward_u32(self.handle, C.byref(problem), tables.handle,
                                        out.ctypes.data_as(C.POINTER(C.c_uint32)), C.byref(st)), self.handle)
        return out, st.as_dict()

    def forward_trace(self, problem: RtmcProblem, tables: Tables):
        """rtmc_forward_trace: (histogram, [n_particles, 16] final states, stats)."""
        out = np.empty(problem.hist_len, dtype=np.int64)
        states = np.empty((problem.n_particles, 16), dtype=np.float64)
        st = RtmcStats()
        check(self.lib.rtmc_forward_trace(self.handle, C.byref(problem), tables.handle,
                                          out.ctypes.data_as(C.POINTER(C.c_int64)), dptr(states), C.byref(st)),
              self.handle)
        return out, states, st.as_dict()

    def gradient(self, problem: RtmcProblem, tables: Tables, dlogsigma: np.ndarray, dlogSigma, adjoint: np.ndarray):
        """rtmc_gradient: score-function adjoint replay.  dlogsigma [n_params, n_theta] on a
        uniform theta grid of [0, pi], dlogSigma [n_params], adjoint [hist_len] (d L / d count).
        Returns (grad [n_params], stats)."""
        dls = np.ascontiguousarray(dlogsigma, dtype=np.float64)
        adj = np.ascontiguousarray(adjoint, dtype=np.float64).ravel()
        _need(dls.ndim == 2 and adj.size == problem.hist_len,
              "dlogsigma must be [n_params, n_theta] and adjoint hold hist_len weights")
        sc = RtmcScore()
        sc.n_params, sc.n_theta = dls.shape
        sc.dlogsigma = dptr(dls)
        for q, v in enumerate(dlogSigma):
            sc.dlogSigma[q] = float(v)
        grad = np.zeros(dls.shape[0], dtype=np.float64)
        st = RtmcStats()
        check(self.lib.rtmc_gradient(self.handle, C.byref(problem), tables.handle, C.byref(sc), dptr(adj), dptr(grad),
                                     C.byref(st)), self.handle)
        return grad, st.as_dict()

    def forward_device(self, problem: RtmcProblem, tables: Tables) -> dict:
        st = RtmcStats()
        check(self.lib.rtmc_forward_device(self.handle, C.byref(problem), tables.handle, C.byref(st)), self.handle)
        return st.as_dict()

    def histogram_device(self):
        """(device address, int64 elements) of the histogram rtmc_forward_device left here."""
        ptr, n = C.c_void_p(), C.c_int64()
        check(self.lib.rtmc_histogram_device(self.handle, C.byref(ptr), C.byref(n)), self.handle)
        return ptr.value, n.value

    def copy_histogram(self, out: np.ndarray):
        _need(out.dtype == np.int64 and out.flags.c_contiguous, "out must be a contiguous int64 array")
        check(self.lib.rtmc_copy_histogram(self.handle, out.ctypes.data_as(C.POINTER(C.c_int64)), out.size),
              self.handle)
        return out

    def set_launch(self, block: int = 0, ring_cap: int = 0, index_mb: int = 0):
        check(self.lib.rtmc_set_launch(self.handle, block, ring_cap, index_mb), self.handle)

    def set_pipeline(self, chunks: int = 0, transport_blocks_per_sm: int = 0):
        """rtmc_set_pipeline: chunks >= 2 overlaps the fold of a chunk with the next chunk's
        transport; 0 = automatic (off), 1 = off."""
        check(self.lib.rtmc_set_pipeline(self.handle, chunks, transport_blocks_per_sm), self.handle)

    def set_fold(self, mode: int = 0):
        """rtmc_set_fold: 0 automatic, 1 64-bit slice fold, 2 time-blocked FP32 fold, 3 the same
        with a rolling accumulator when one chunk covers the call."""
        check(self.lib.rtmc_set_fold(self.handle, mode), self.handle)

    def set_schedule(self, event_major: int = -1):
        """rtmc_set_schedule: -1 automatic, 0 lockstep warp batches, 1 one particle per thread,
        2 split (events kernel, then observation kernel)."""
        check(self.lib.rtmc_set_schedule(self.handle, event_major), self.handle)

    def last_timing(self):
        ms = C.c_double()
        n = C.c_int32()
        check(self.lib.rtmc_last_timing(self.handle, C.byref(ms), C.byref(n)), self.handle)
        return ms.value, n.value

    def set_table_cache(self, enable: bool):
        check(self.lib.rtmc_set_table_cache(self.handle, 1 if enable else 0), self.handle)

    def set_particle_order(self, enable: bool):
        """rtmc_set_particle_order: bin the index path's particles in starting-direction order."""
        check(self.lib.rtmc_set_particle_order(self.handle, 1 if enable else 0), self.handle)

    def set_fp64_estimate(self, enable: bool):
        """rtmc_set_fp64_estimate: FP64 radius-only observations through the exact FP32 estimate."""
        check(self.lib.rtmc_set_fp64_estimate(self.handle, 1 if enable else 0), self.handle)

    def set_early_copy(self, first_percent: int = -1):
        """rtmc_set_early_copy: host-output calls bin the first first_percent of the instants,
        fold them and start their copies before binning the rest (0: off, -1: default)."""
        check(self.lib.rtmc_set_early_copy(self.handle, int(first_percent)), self.handle)

    def flush_l2(self):
        check(self.lib.rtmc_flush_l2(self.handle), self.handle)

    def probe_l2_reductions(self) -> float:
        """rtmc_probe_l2_reductions: the L2's 16-byte vector-reduction rate (per second)."""
        r = C.c_double()
        check(self.lib.rtmc_probe_l2_reductions(self.handle, C.byref(r)), self.handle)
        return r.value


class PinnedBuffer:
    """Page-locked host memory from rtmc_host_alloc, viewed as a numpy array."""

    def __init__(self, nbytes: int):
        self.lib = load()
        p = C.c_void_p()
        check(self.lib.rtmc_host_alloc(nbytes, C.byref(p)))
        self.ptr = p
        self.nbytes = nbytes

    def array(self, dtype, count):
        buf = (C.c_char * self.nbytes).from_address(self.ptr.value)
        return np.frombuffer(buf, dtype=dtype, count=count)

    def __del__(self):
        if getattr(self, "ptr", None) and self.ptr.value:
            self.lib.rtmc_host_free(self.ptr)
            self.ptr = C.c_void_p()
