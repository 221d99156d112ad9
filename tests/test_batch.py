"""Batched runs (rtmc_batch_*): one persistent, graph-captured launch over many instances
sharing an observation grid.  Each instance must give exactly the histogram of its own
single run (same seed and particle ids: the same trajectories, integer counts)."""
import numpy as np
import pytest

from radiativetransfermontecarlo_gb300 import build_problem, get_context
from radiativetransfermontecarlo_gb300 import workloads as W
from radiativetransfermontecarlo_gb300.batch import Batch, autotune

pytestmark = pytest.mark.gpu


def _instances(k, n_cap):
    out = []
    for i in range(k):
        geo, src, mat, obs, opts = W.c4_instance(i)
        src = dict(src, numberParticles=min(src["numberParticles"], n_cap))
        out.append((geo, src, mat, obs, dict(opts, exact_count=True, seed=100 + i)))
    return out


def test_c4_parameter_ranges():
    lcs, cvs, fs, qs, ns = [], [], [], [], []
    for i in range(256):
        geo, src, mat, obs, opts = W.c4_instance(i)
        lcs.append(mat.CorrelationLength); cvs.append(mat.coefficients_of_variation[0])
        fs.append(mat.Frequency); qs.append(mat.Q); ns.append(src["numberParticles"])
    assert 0.02 <= min(lcs) and max(lcs) <= 1 and 0.01 <= min(cvs) and max(cvs) <= 0.2
    assert 1 <= min(fs) and max(fs) <= 20 and set(qs) <= {float("inf"), 100.0, 500.0}
    assert 1e4 <= min(ns) and max(ns) <= 1e7 and len(set(qs)) == 3


def test_batch_equals_single_runs():
    """Every instance equals its own single run on the same kernel design (lockstep warp
    batches, or one particle per thread for the event-heavy instances), bin for bin."""
    inst = _instances(12, 6000)
    b = Batch(inst)
    st = b.run()
    assert st["device_status"] == 0
    H = b.histograms()
    sched = b.schedule()
    ctx = get_context(0)
    total = 0
    try:
        for i, (geo, src, mat, obs, opts) in enumerate(inst):
            prob, grid, N = build_problem(geo, src, mat, obs, dict(opts, precision="fp32"))
            P, keep = prob.to_ctypes()
            ctx.set_schedule(int(sched[i]))
            ref, s = ctx.forward(P, prob.tables)
            assert np.array_equal(H[i], ref), i
            total += s["scatter_events"]
    finally:
        ctx.set_schedule(-1)
    assert st["scatter_events"] == total
    # a second replay of the graph gives the same result
    b.run()
    assert np.array_equal(b.histograms(), H)
    b.close()


def test_batch_autotune_keeps_results():
    inst = _instances(6, 4000)
    b = Batch(inst)
    b.run()
    H = b.histograms()
    shape, times = autotune(b, blocks=(256, 512), rings=(4, 8), chunks=(2048, 16384), repeats=1)
    assert shape in times and len(times) >= 4
    b.run()
    assert np.array_equal(b.histograms(), H)
    b.close()


def test_batch_instances_match_oracle_fp64():
    """C4 instances in one FP64 batched launch against the oracle's event scheme on the same
    Philox stream: lockstep instances (1, 8, 9) and event-heavy ones (0, 13, 36: 120-350
    scatterings per particle, Q = 500, 100 and Inf) that the event-major kernel runs.
    Counts, scatterings and kills are equal; bins equal up to edge ties."""
    from oracle import oracle as O
    picks = [0, 1, 8, 9, 13, 36]
    inst = []
    for i in picks:
        geo, src, mat, obs, opts = W.c4_instance(i)
        src = dict(src, numberParticles=1500)
        inst.append((geo, src, mat, obs, dict(opts, exact_count=True, seed=200 + i, precision="fp64")))
    b = Batch(inst)
    sched = b.schedule()
    assert list(sched) == [1, 0, 0, 0, 1, 1], sched  # event-heavy instances on rt_transport_batch_em
    st = b.run()
    assert st["device_status"] == 0 and st["launches"] == 2  # both kernels of the graph ran
    H = b.histograms()
    tot = {"scatter_events": 0, "kills": 0}
    for k, prob in enumerate(b.problems):
        ref, rs, _ = O.run(prob, O.table_knots(prob.tables), scheme="event")
        diff = int(np.abs(H[k] - ref).sum() >> prob.hist_shift)
        assert diff <= max(4, 1e-6 * rs["observations"]), (picks[k], diff)
        for key in tot:
            tot[key] += rs[key]
    assert st["scatter_events"] == tot["scatter_events"] and st["kills"] == tot["kills"]
    b.close()


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_batch_split_kernel_equals_ring_kernel(precision):
    """The lockstep instances on the split kernel (rt_transport_batch_split) and on the ring
    kernel (rt_transport_batch) give the same histograms, with segment lists long enough
    and with two segments per particle (most particles then run whole in the events
    phase), for several work-item sizes."""
    inst = [(g, s, m, o, dict(op, precision=precision)) for g, s, m, o, op in _instances(8, 5000)]
    ctx = get_context(0)
    out = []
    try:
        for segs in (0, 2):
            ctx.set_launch(0, segs, 0)
            b = Batch(inst)
            for shape in ((512, 8, 0), (0, -1, 0), (0, -1, 1000), (256, 4, 3000)):
                b.set_launch(*shape)
                st = b.run()
                assert st["device_status"] == 0
                out.append((segs, shape, b.histograms(), st["scatter_events"], st["observations"]))
            b.close()
    finally:
        ctx.set_launch(0, 0, 0)
    h0, ev0, ob0 = out[0][2:]
    assert h0.any()
    for segs, shape, h, ev, ob in out[1:]:
        assert np.array_equal(h, h0), (segs, shape)
        assert ev == ev0 and ob == ob0, (segs, shape)


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_batch_em_shared_histogram_equals_device_histogram(precision):
    """The event-major instances binned in the block's shared-memory histogram and with
    64-bit atomics into device memory give the same histograms (instances 0, 13 and 36 are
    event-heavy; 1 and 8 run on the lockstep kernel beside them)."""
    picks = [0, 1, 8, 13, 36]
    inst = []
    for i in picks:
        geo, src, mat, obs, opts = W.c4_instance(i)
        inst.append((geo, dict(src, numberParticles=3000), mat, obs,
                     dict(opts, exact_count=True, seed=300 + i, precision=precision)))
    b = Batch(inst)
    assert list(b.schedule()) == [1, 0, 0, 1, 1]
    out = []
    for shared in (0, 1, -1):
        b.set_em_histogram(shared)
        st = b.run()
        assert st["device_status"] == 0 and st["launches"] == 2
        out.append((b.histograms(), st["scatter_events"], st["observations"]))
    b.close()
    h0, ev0, ob0 = out[0]
    assert h0[[0, 3, 4]].any()
    for h, ev, ob in out[1:]:
        assert np.array_equal(h, h0) and ev == ev0 and ob == ob0


def test_batch_set_schedule_moves_instances_between_kernels():
    """Every instance gives the same histogram on either kernel: all lockstep, all
    event-major, and the automatic split restored; tune_schedule keeps the results."""
    from radiativetransfermontecarlo_gb300.batch import tune_schedule
    picks = [0, 1, 8, 13, 36]
    inst = []
    for i in picks:
        geo, src, mat, obs, opts = W.c4_instance(i)
        inst.append((geo, dict(src, numberParticles=2500), mat, obs, dict(opts, exact_count=True, seed=400 + i)))
    b = Batch(inst)
    auto = b.schedule()
    assert list(auto) == [1, 0, 0, 1, 1]
    b.run()
    H = b.histograms()
    for em in ([0] * 5, [1] * 5, None):
        b.set_schedule(em)
        assert list(b.schedule()) == (list(auto) if em is None else em)
        st = b.run()
        assert st["device_status"] == 0
        assert np.array_equal(b.histograms(), H), em
    ev = b.expected_events()
    n_obs = np.array([b._arr[i].n_obs for i in range(len(picks))])
    assert list((4 * ev >= n_obs).astype(int)) == list(auto)
    best, times = tune_schedule(b, factors=(1, 4, 1000), repeats=1)
    assert best in times and len(times) == 3
    b.run()
    assert np.array_equal(b.histograms(), H)
    b.close()
