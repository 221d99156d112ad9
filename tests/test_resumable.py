"""Checkpoint and resume (resumable.py): a run cut into particle chunks, stopped and
resumed from its snapshot, gives the histogram of one uninterrupted run bit for bit.

CPU: the chunking, the snapshot files and their refusals, with a stand-in for the
context whose forward is a fixed function of the particle ids it is given (as the
device's is: Philox keyed by particle id).  GPU: the real transport against a single
radiativeTransfer call."""
import json

import numpy as np
import pytest

from radiativetransfermontecarlo_gb300 import build_problem, radiativeTransfer
from radiativetransfermontecarlo_gb300 import resumable as R
from radiativetransfermontecarlo_gb300 import workloads as W


class _IdContext:
    """forward(P, tables): each particle id p adds 1 << hist_shift to bins (p * 7919) and
    (p * 104729 + 3) mod hist_len; the counters count particles."""

    def __init__(self):
        self.calls = []

    def forward(self, P, tables):
        ids = np.arange(P.pid0, P.pid0 + P.n_particles, dtype=np.int64)
        h = np.zeros(P.hist_len, dtype=np.int64)
        np.add.at(h, (ids * 7919) % P.hist_len, np.int64(1) << P.hist_shift)
        np.add.at(h, (ids * 104729 + 3) % P.hist_len, np.int64(1) << P.hist_shift)
        self.calls.append((P.pid0, P.n_particles))
        st = dict.fromkeys(R.COUNTERS, 0)
        st["scatter_events"] = int(P.n_particles) * 3
        st["observations"] = 2 * int(P.n_particles)
        return h, st


def _c1(n=25_000):
    geo, src, mat, obs, opts = W.c1_acoustic3d(n=n)
    return geo, src, mat, obs, dict(opts, exact_count=True)


def test_resume_after_stop_equals_one_run(tmp_path, monkeypatch):
    ctx = _IdContext()
    monkeypatch.setattr(R, "get_context", lambda device=0: ctx)
    geo, src, mat, obs, opts = _c1()
    one = R.radiative_transfer_resumable(geo, src, mat, obs, opts, checkpoint=str(tmp_path / "a"), chunk=10 ** 9)
    assert ctx.calls == [(0, 25_000)]
    ck = str(tmp_path / "b")
    ctx.calls.clear()
    assert R.radiative_transfer_resumable(geo, src, mat, obs, opts, checkpoint=ck, chunk=4_000, max_chunks=2) is None
    assert R.radiative_transfer_resumable(geo, src, mat, obs, opts, checkpoint=ck, chunk=4_000, max_chunks=3) is None
    meta = json.load(open(ck))
    assert meta["next"] == 20_000 and meta["counters"]["observations"] == 40_000
    res = R.radiative_transfer_resumable(geo, src, mat, obs, opts, checkpoint=ck, chunk=4_000)
    assert ctx.calls == [(0, 4000), (4000, 4000), (8000, 4000), (12000, 4000), (16000, 4000), (20000, 4000),
                         (24000, 1000)]
    assert np.array_equal(res["energyDensity"], one["energyDensity"]) and np.array_equal(res["energy"], one["energy"])
    assert res["stats"]["scatter_events"] == one["stats"]["scatter_events"] == 75_000
    assert res["stats"]["chunks_this_call"] == 2 and res["stats"]["particles"] == 25_000
    # a finished snapshot returns its result without running anything
    ctx.calls.clear()
    again = R.radiative_transfer_resumable(geo, src, mat, obs, dict(opts, return_counts=True), checkpoint=str(tmp_path / "a"))
    prob, _, _ = build_problem(geo, src, mat, obs, opts)
    assert ctx.calls == [] and int(again["E"].sum()) == (2 * 25_000) << prob.hist_shift


def test_snapshot_of_another_problem_or_damaged_is_refused(tmp_path, monkeypatch):
    ctx = _IdContext()
    monkeypatch.setattr(R, "get_context", lambda device=0: ctx)
    geo, src, mat, obs, opts = _c1()
    ck = str(tmp_path / "c")
    assert R.radiative_transfer_resumable(geo, src, mat, obs, opts, checkpoint=ck, chunk=5_000, max_chunks=1) is None
    with pytest.raises(ValueError, match="another problem"):
        R.radiative_transfer_resumable(geo, src, mat, obs, dict(opts, seed=1), checkpoint=ck, chunk=5_000)
    with pytest.raises(ValueError, match="another problem"):
        R.radiative_transfer_resumable(geo, dict(src, numberParticles=30_000), mat, obs, opts, checkpoint=ck)
    with pytest.raises(ValueError, match="another problem"):  # another observation grid (its edges)
        R.radiative_transfer_resumable(geo, src, mat, dict(obs, x=obs["x"] * 1.5), opts, checkpoint=ck)
    h = np.fromfile(ck + ".hist", dtype=np.uint64)
    h[7] += np.uint64(1)
    h.tofile(ck + ".hist")
    with pytest.raises(ValueError, match="damaged"):
        R.radiative_transfer_resumable(geo, src, mat, obs, opts, checkpoint=ck, chunk=5_000)
    with pytest.raises(ValueError, match="chunk"):
        R.radiative_transfer_resumable(geo, src, mat, obs, opts, checkpoint=str(tmp_path / "d"), chunk=0)


def test_uint32_counts_saturate_like_the_device_narrowing():
    """The finished run's uint32 E is (int64 sum >> hist_shift) saturated at 2^32 - 1, as
    rt_narrow_u32 narrows the device's sum."""
    h = np.array([0, 5 << 40, (3 << 31) << 30, 1 << 62, (1 << 40) - 1], dtype=np.uint64)
    u = R.narrow_u32(h, 40)
    assert u.dtype == np.uint32
    assert list(u) == [0, 5, 3 << 21, 1 << 22, 0]
    assert list(R.narrow_u32(h, 0)) == [0, 0xFFFFFFFF, 0xFFFFFFFF, 0xFFFFFFFF, 0xFFFFFFFF]


@pytest.mark.gpu
def test_resumed_transport_equals_one_radiative_transfer_call(tmp_path):
    """The real transport in 3 chunks, stopped after the first and resumed, against one
    radiativeTransfer call: energyDensity, energy and the counters are the same."""
    geo, src, mat, obs, opts = W.c1_acoustic3d(n=30_000)
    opts = dict(opts, exact_count=True)
    one = radiativeTransfer(geo, src, mat, obs, opts)
    ck = str(tmp_path / "g")
    assert R.radiative_transfer_resumable(geo, src, mat, obs, opts, checkpoint=ck, chunk=10_000, max_chunks=1) is None
    res = R.radiative_transfer_resumable(geo, src, mat, obs, opts, checkpoint=ck, chunk=10_000)
    assert res["stats"]["chunks_this_call"] == 2
    assert np.array_equal(res["energyDensity"], one["energyDensity"]) and np.array_equal(res["energy"], one["energy"])
    for k in ("scatter_events", "observations", "kills"):
        assert res["stats"][k] == one["stats"][k], k
