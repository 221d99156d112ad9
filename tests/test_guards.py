"""Guards of the transport and their error statuses.

* the per-particle event cap (rtmc_problem.max_events), a watchdog: a particle that
  reaches it stops, the kernel sets bit 0 of the device status and the call returns
  RTMC_ERR_DEVICE; the context stays usable;
* the 64-bit fixed-point headroom: a bin of one time slice receives at most one count per
  particle, so n_particles << hist_shift must stay below 2^64 (checked on the host before
  any launch);
* the int64 range of rtmc_forward's histogram: a bin of 2^63 or more is reported
  (RTMC_ERR_DEVICE), while rtmc_forward_u32 narrows the unsigned sum exactly, saturating
  like the reference's uint32 E (initializeObservation.m:133);
* tables with NaN knots or angles are refused when the handle is made.

Every failure is made on the host, or by a bounded on-device limit that returns an error
status: nothing here faults, traps or hangs a GPU.
"""
import ctypes as C
import math

import numpy as np
import pytest

from radiativetransfermontecarlo_gb300 import MaterialClass, _lib, build_problem, colon, get_context
from radiativetransfermontecarlo_gb300 import workloads as W

RTMC_ERR_ARG, RTMC_ERR_DEVICE = 1, 4  # enum rtmc_status (include/rtmc.h)


def _small_c1(n, **opts):
    geo, src, mat, obs, o = W.c1_acoustic3d(precision="fp32")
    prob, grid, N = build_problem(geo, dict(src, numberParticles=n), mat, obs, dict(o, exact_count=True, **opts))
    return prob, grid


def _raw_forward(fn, prob, out):
    ctx = get_context(0)
    P, keep = prob.to_ctypes()
    st = _lib.RtmcStats()
    ptr = out.ctypes.data_as(C.POINTER(C.c_uint32 if out.dtype == np.uint32 else C.c_int64))
    rc = fn(ctx.handle, C.byref(P), prob.tables.handle, ptr, C.byref(st))
    msg = ctx.lib.rtmc_last_error(ctx.handle)
    return rc, st.as_dict(), (msg.decode() if msg else "")


def test_nan_tables_are_refused():
    c = np.linspace(0.0, 1.0, 101)
    t = np.linspace(0.0, math.pi, 101)
    for bad_c, bad_t in ((c.copy(), t), (c, t.copy())):
        arr = bad_c if bad_c is not c else bad_t
        arr[50] = np.nan
        with pytest.raises(_lib.RtmcError, match="strictly increasing|finite"):
            _lib.Tables.from_knots([(bad_c, bad_t)])
    c2 = c.copy()
    c2[-1] = np.inf
    t2 = t.copy()
    t2[0] = -np.inf
    with pytest.raises(_lib.RtmcError):
        _lib.Tables.from_knots([(c, t2)])
    assert _lib.Tables.from_knots([(c, t)]).info().n_tables == 1


def test_nan_material_is_refused():
    geo = {"dimension": 3}
    with pytest.raises((_lib.RtmcError, ValueError)):
        mat = MaterialClass(geo, 10, True, 1, [0.05, 0.05], 0, "exp", float("nan"))
        MaterialClass.prepareSigma(mat, 3)


@pytest.mark.gpu
def test_event_cap_returns_device_error_and_context_stays_usable():
    prob, grid = _small_c1(2000)
    prob.max_events = 1  # every scattered particle reaches it (C1: ~2.4 events per particle)
    out = np.zeros(prob.hist_len, dtype=np.int64)
    rc, st, msg = _raw_forward(get_context(0).lib.rtmc_forward, prob, out)
    assert rc == RTMC_ERR_DEVICE, (rc, msg)
    assert st["device_status"] & 1 and "guard" in msg
    prob.max_events = 0
    P, keep = prob.to_ctypes()
    h, st = get_context(0).forward(P, prob.tables)
    assert st["device_status"] == 0 and int(h.sum() >> prob.hist_shift) > 0


@pytest.mark.gpu
def test_fixed_point_headroom_is_checked_before_launch():
    prob, grid = _small_c1(1 << 24, hist_shift=40)  # 2^24 counts of 2^40 reach 2^64
    out = np.zeros(prob.hist_len, dtype=np.int64)
    rc, st, msg = _raw_forward(get_context(0).lib.rtmc_forward, prob, out)
    assert rc == RTMC_ERR_ARG and "hist_shift" in msg, (rc, msg)
    assert st["launches"] == 0


@pytest.mark.gpu
def test_int64_range_reported_and_u32_exact():
    # two particles at the origin, one radial bin: each instant holds 2 counts of 2^62 = 2^63
    geo = {"dimension": 3, "frame": "spherical"}
    mat = MaterialClass(geo, 10, True, 1, [0.05, 0.05], 0, "exp", 0.1)
    src = {"numberParticles": 2, "lambda": 0.0}
    obs = {"x": [0.0, 100.0], "y": [-np.pi, np.pi], "z": [-np.pi / 2, np.pi / 2], "directions": [0, np.pi],
           "time": colon(0, 0.02, 0.2)}
    prob, grid, N = build_problem(geo, src, mat, obs, {"exact_count": True, "precision": "fp32", "hist_shift": 62})
    out = np.zeros(prob.hist_len, dtype=np.int64)
    rc, st, msg = _raw_forward(get_context(0).lib.rtmc_forward, prob, out)
    assert rc == RTMC_ERR_DEVICE and "2^63" in msg, (rc, msg)
    assert st["device_status"] & 2
    P, keep = prob.to_ctypes()
    h32, st32 = get_context(0).forward_u32(P, prob.tables)
    assert st32["device_status"] == 0
    assert h32[0] == 0 and np.all(h32[1:] == 2), h32
    # three particles: 3 * 2^62 is still below 2^64, so the u32 counts stay exact
    prob.n_particles = 3
    P, keep = prob.to_ctypes()
    h32, _ = get_context(0).forward_u32(P, prob.tables)
    assert np.all(h32[1:] == 3)
    prob.n_particles = 4  # 4 * 2^62 = 2^64 would wrap: refused on the host
    rc, st, msg = _raw_forward(get_context(0).lib.rtmc_forward_u32, prob, np.zeros(prob.hist_len, dtype=np.uint32))
    assert rc == RTMC_ERR_ARG


@pytest.mark.gpu
def test_l2_reduction_probe_reports_a_rate():
    """rtmc_probe_l2_reductions times its vector reductions and leaves the context usable:
    a plausible rate (between 1e9 and 1e13 per second), and a forward call afterwards."""
    from radiativetransfermontecarlo_gb300 import get_context
    ctx = get_context(0)
    r = ctx.probe_l2_reductions()
    assert 1e9 < r < 1e13
    geo, src, mat, obs, opts = W.c1_acoustic3d(n=2000, precision="fp32")
    prob, grid, N = build_problem(geo, src, mat, obs, dict(opts, exact_count=True))
    P, keep = prob.to_ctypes()
    h, st = ctx.forward(P, prob.tables)
    assert st["device_status"] == 0 and int(h.sum() >> prob.hist_shift) == st["observations"]
