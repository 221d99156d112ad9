"""rtmc_forward_noalloc: the transport for callers that cannot allocate device memory.

Some hosts cannot call cudaMalloc: an application whose own allocator owns the device
memory, or one that hands the library only buffers it allocated up front.  For them
rtmc_forward_noalloc keeps every buffer it needs in one static device array of a fixed
size (96 MB per GPU) and writes into a device histogram the caller passes.  This test
calls it through the C ABI twice in a row and checks each result against rtmc_forward
on the same problem (integer counts of the same trajectories: equal, bin for bin).
The file sorts last so that a run stopping at the first failure has run the rest.
"""
import ctypes as C

import numpy as np
import pytest

from radiativetransfermontecarlo_gb300 import _lib, build_problem, get_context
from radiativetransfermontecarlo_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [40_000, 1001])
def test_noalloc_matches_forward_on_two_calls(n):
    """40,000 particles run in several chunks through the static array; 1001 in one chunk
    whose index rows are padded to a multiple of 32."""
    torch = pytest.importorskip("torch")
    geo, src, mat, obs, opts = W.c3_halfspace2d()  # 4 elastic tables (~41 MB staged) + 400 time slices
    prob, grid, N = build_problem(geo, dict(src, numberParticles=n), mat, obs,
                                  dict(opts, exact_count=True, precision="fp32"))
    P, keep = prob.to_ctypes()
    ref, ref_stats = get_context(0).forward(P, prob.tables)
    lib = _lib.load()
    out = torch.empty(prob.hist_len, dtype=torch.int64, device="cuda:0")
    for _ in range(2):
        out.fill_(-1)  # the call zeroes the histogram itself
        torch.cuda.synchronize()
        st = _lib.RtmcStats()
        _lib.check(lib.rtmc_forward_noalloc(C.byref(P), prob.tables.handle, C.c_void_p(out.data_ptr()), None,
                                            C.byref(st)))
        got = out.cpu().numpy()
        assert np.array_equal(got, ref)
        assert st.device_status == 0
        assert st.scatter_events == ref_stats["scatter_events"]
        assert st.observations == ref_stats["observations"]
        assert st.launches >= (4 if n > 32_000 else 2)  # several chunks through the static array


def test_noalloc_rejects_problems_beyond_the_static_array():
    """One million observation instants: 32 particles alone would need 128 MB of index
    array, more than the static array holds, so the call refuses before any launch."""
    torch = pytest.importorskip("torch")
    geo, src, mat, obs, opts = W.c1_acoustic3d(n=64, precision="fp32")
    obs = dict(obs, time=np.linspace(0.0, 5.0, 1_000_001))
    prob, grid, N = build_problem(geo, src, mat, obs, dict(opts, exact_count=True))
    P, keep = prob.to_ctypes()
    out = torch.zeros(prob.hist_len, dtype=torch.int64, device="cuda:0")  # a real buffer of the full size
    torch.cuda.synchronize()
    rc = _lib.load().rtmc_forward_noalloc(C.byref(P), prob.tables.handle, C.c_void_p(out.data_ptr()), None, None)
    assert rc == 1  # RTMC_ERR_ARG
    assert b"static scratch" in _lib.load().rtmc_last_error(None)
    assert int(out.abs().sum().item()) == 0  # nothing was written


def test_noalloc_large_slices():
    """C2's 4-axis grid (13.8 MB slices): the fold runs one slice per block row
    (rt_bin_slices) over the whole slice range; equal to rtmc_forward bin for bin."""
    torch = pytest.importorskip("torch")
    geo, src, mat, obs, opts = W.c2_elastic3d(t_end=1.0)
    prob, grid, N = build_problem(geo, dict(src, numberParticles=1001), mat, obs, dict(opts, exact_count=True))
    P, keep = prob.to_ctypes()
    ref, ref_stats = get_context(0).forward(P, prob.tables)
    out = torch.empty(prob.hist_len, dtype=torch.int64, device="cuda:0")
    torch.cuda.synchronize()
    st = _lib.RtmcStats()
    _lib.check(_lib.load().rtmc_forward_noalloc(C.byref(P), prob.tables.handle, C.c_void_p(out.data_ptr()), None,
                                                C.byref(st)))
    assert st.device_status == 0 and st.observations == ref_stats["observations"]
    assert np.array_equal(out.cpu().numpy(), ref)
