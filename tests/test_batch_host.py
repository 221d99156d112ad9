"""Host logic of the batched launch (batch.py) on CPU, with stand-ins for the batch: the
launch-shape and kernel-split tuners time each candidate once, keep the fastest and leave
it set."""
from types import SimpleNamespace

import numpy as np

from radiativetransfermontecarlo_gb300 import batch as B


class _FakeBatch:
    """expected events 1, 10, 40, 100 per particle over 250 instants; a launch takes
    100 ms + 10 ms per event-major instance with under 50 expected events + 30 ms per
    lockstep instance with 50 or more (so the best split puts 40 and 100 event-major)."""

    def __init__(self):
        self.problems = [object()] * 4
        self._arr = [SimpleNamespace(n_obs=250) for _ in range(4)]
        self.ev = np.array([1.0, 10.0, 40.0, 100.0])
        self.em = (8 * self.ev >= 250).astype(np.int32)
        self.schedules, self.shapes = [], []

    def expected_events(self):
        return self.ev.copy()

    def set_schedule(self, em=None):
        self.em = np.array(em, dtype=np.int32)
        self.schedules.append(tuple(self.em))

    def set_launch(self, block=0, ring=0, chunk=0):
        if block == 256 and ring == 4:
            raise B._lib.RtmcError("shape refused")
        self.shapes.append((block, ring, chunk))

    def run(self):
        heavy = self.ev >= 50
        ms = 100.0 + 10.0 * np.sum((self.em == 1) & ~heavy) + 30.0 * np.sum((self.em == 0) & heavy)
        if self.shapes:
            b, r, c = self.shapes[-1]
            ms += {4096: 0.0, 16384: 5.0}.get(c, 9.0) + (0.0 if b in (0, 512) else 3.0)
        return {"kernel_ms": float(ms)}


def test_tune_schedule_keeps_the_fastest_split():
    b = _FakeBatch()
    best, times = B.tune_schedule(b, factors=(1, 2, 4, 8, 16, 32), repeats=1)
    # factor f puts an instance event-major when f x events >= 250: f = 1, 2 none (the
    # heavy instance on the lockstep kernel: 130 ms), 4 the 100 (100 ms), 8 and 16 also the
    # 40 (110 ms), 32 also the 10 (120 ms)
    assert times == {1: 130.0, 2: 130.0, 4: 100.0, 8: 110.0, 16: 110.0, 32: 120.0}
    assert best == 4
    assert tuple(b.em) == tuple((best * b.ev >= 250).astype(np.int32))
    # splits that an earlier factor already produced are not timed again
    distinct = {tuple((f * b.ev >= 250).astype(np.int32)) for f in (1, 2, 4, 8, 16, 32)}
    assert len(b.schedules) == len(distinct) + 1


def test_autotune_skips_refused_shapes_and_keeps_the_fastest():
    b = _FakeBatch()
    shape, times = B.autotune(b, blocks=(256, 512), rings=(4, 8), chunks=(4096, 16384), split_chunks=(4096,), repeats=1)
    assert (256, 4, 4096) not in times and (0, -1, 4096) in times
    assert shape == min(times, key=times.get) and b.shapes[-1] == shape
    assert times[shape] == min(times.values())
