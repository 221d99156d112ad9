"""The C ABI library loads, exports every function include/rtmc.h declares, and its
structs match the ctypes mirrors.  No GPU needed (no compute calls)."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from radiativetransfermontecarlo_gb300 import _lib

HEADER = Path(__file__).resolve().parents[1] / "include" / "rtmc.h"


def declared_functions():
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    return sorted(set(re.findall(r"\b(rtmc_[a-z0-9_]+)\s*\(", text)))


def test_every_declared_symbol_is_exported_and_bound():
    lib = C.CDLL(str(_lib.LIB_PATH))
    names = declared_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n
        assert n in _lib.SIGNATURES, f"{n} has no ctypes signature"


def test_struct_layout_matches_binding():
    lib = _lib.load()
    sizes = (C.c_int64 * 4)()
    assert lib.rtmc_abi_sizes(sizes) == 0
    assert list(sizes) == [C.sizeof(_lib.RtmcMaterial), C.sizeof(_lib.RtmcTablesInfo),
                           C.sizeof(_lib.RtmcProblem), C.sizeof(_lib.RtmcStats)]
    assert lib.rtmc_abi_version() == 2


def test_host_functions_report_errors():
    lib = _lib.load()
    h = C.c_void_p()
    m = _lib.RtmcMaterial()
    m.d = 4  # invalid dimension
    assert lib.rtmc_tables_build(C.byref(m), C.byref(h)) == 1
    assert b"dimension" in lib.rtmc_last_error(None)
    # knots must be strictly increasing
    c = np.array([0.0, 0.5, 0.5, 1.0])
    t = np.array([0.0, 1.0, 2.0, 3.0])
    nk = (C.c_int64 * 1)(4)
    cp = (C.POINTER(C.c_double) * 1)(_lib.dptr(c))
    tp = (C.POINTER(C.c_double) * 1)(_lib.dptr(t))
    assert lib.rtmc_tables_from_knots(1, nk, cp, tp, C.byref(h)) == 5
    assert b"strictly increasing" in lib.rtmc_last_error(None)
    # forward with a NULL problem is an argument error, not a crash
    assert lib.rtmc_forward(None, None, None, None, None) == 1
    assert lib.rtmc_forward_u32(None, None, None, None, None) == 1
    assert lib.rtmc_forward_noalloc(None, None, None, None, None) == 1


def test_tables_from_knots_roundtrip_and_eval():
    c = np.array([0.0, 0.25, 0.5, 1.0])
    t = np.array([0.0, 1.0, 1.5, 3.0])
    T = _lib.Tables.from_knots([(c, t)])
    cc, tt = T.knots(0)
    assert np.array_equal(cc, c) and np.array_equal(tt, t)
    # griddedInterpolant: linear inside, linear extrapolation outside
    u = np.array([-0.1, 0.0, 0.125, 0.75, 1.0, 1.2])
    assert np.allclose(T.eval(0, u), [-0.4, 0.0, 0.5, 2.25, 3.0, 3.6])


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_has_gpu(), reason="passes a placeholder device pointer: host-only check")
def test_problem_validation_needs_no_gpu():
    """rtmc_forward_noalloc validates the problem before any CUDA call: boundary kinds,
    source shapes, radial profiles and the sub-step budget are refused with a message.
    (Every problem here is invalid, so the placeholder histogram pointer is never used.)"""

    from radiativetransfermontecarlo_gb300 import build_problem
    from radiativetransfermontecarlo_gb300 import workloads as W
    lib = _lib.load()
    geo, src, mat, obs, opts = W.c1_acoustic3d()
    prob, grid, N = build_problem(geo, dict(src, numberParticles=100), mat, obs, dict(opts, exact_count=True))

    def refused(mutate, msg):
        P, keep = prob.to_ctypes()
        extra = mutate(P)
        rc = lib.rtmc_forward_noalloc(C.byref(P), prob.tables.handle, C.c_void_p(256), None, None)
        err = lib.rtmc_last_error(None)
        del extra
        assert rc == 1 and msg.encode() in err, (rc, err)  # RTMC_ERR_ARG

    def bnd(P, d, v):
        P.n_bnd, P.bnd_dir[0], P.bnd_val[0] = 1, d, v
    refused(lambda P: bnd(P, 5, 1.0), "boundary dir")
    refused(lambda P: bnd(P, 4, 0.0), "cylinder radius")
    refused(lambda P: setattr(P, "src_type", 2), "source type")

    def plane(P, d, normal):
        P.src_type, P.d = 1, d
        for i in range(3):
            P.src_normal[i], P.src_u[i], P.src_v[i] = normal[i], (1.0, 0, 0)[i], (0, 1.0, 0)[i]
    refused(lambda P: plane(P, 2, (0, 0, 1.0)), "3D only")
    refused(lambda P: plane(P, 3, (0, 0, 2.0)), "unit vectors")

    def radial(P, c, r):
        c, r = np.ascontiguousarray(c, float), np.ascontiguousarray(r, float)
        P.src_radial_n, P.src_radial_cdf, P.src_radial_r = c.size, _lib.dptr(c), _lib.dptr(r)
        return c, r
    refused(lambda P: radial(P, [0.0], [0.0]), "2 to 65536 knots")
    refused(lambda P: radial(P, [0.0, 0.5, 0.5, 1.0], [0, 1, 2, 3]), "strictly increasing")
    refused(lambda P: setattr(P, "n_sub", 1 << 23), "2^30")
    refused(lambda P: setattr(P, "h", -1.0), "sub-step h")
    refused(lambda P: setattr(P, "mft", (C.c_double * 2)(-1.0, -1.0)), "mean free times")


def test_null_handles_are_argument_errors():
    """Every entry point that takes a context or a batch refuses a NULL handle with
    RTMC_ERR_ARG and a message (no CUDA call, no crash)."""
    lib = _lib.load()
    r = C.c_double()
    em = (C.c_int32 * 4)()
    calls = {
        "rtmc_set_early_copy": (None, 40), "rtmc_set_fp64_estimate": (None, 1), "rtmc_set_particle_order": (None, 1),
        "rtmc_set_fold": (None, 0), "rtmc_set_schedule": (None, -1), "rtmc_set_launch": (None, 0, 0, 0),
        "rtmc_set_pipeline": (None, 0, 0), "rtmc_set_table_cache": (None, 1),
        "rtmc_probe_l2_reductions": (None, C.byref(r)), "rtmc_batch_set_launch": (None, 0, 0, 0),
        "rtmc_batch_set_em_histogram": (None, 1), "rtmc_batch_set_schedule": (None, None),
        "rtmc_batch_schedule": (None, em), "rtmc_batch_run": (None, None), "rtmc_forward_device": (None, None, None, None),
        "rtmc_gradient": (None, None, None, None, None, None, None),
    }
    for name, args in calls.items():
        assert getattr(lib, name)(*args) == 1, name
        assert lib.rtmc_last_error(None), name
