"""The batch runner's host loop on the CPU, with a stand-in for the device stack: running one chunk
ahead (asynchronous series takes) gives the same series, ring-down steps and Z(f) for every scene
as processing each chunk before the next, across compactions and decision steps, and the same
ring-down step as the reference's residual rule applied to the scene's whole series."""
import math

import numpy as np
import pytest

from em_lab_gb300 import batch, configs


def series_of(scene_id, t0, n):
    """A damped tone per scene, a function of the scene and the absolute step only (so a compaction
    cannot change it): (n, 2) float32 V, I."""
    t = np.arange(t0, t0 + n, dtype=np.float64)
    tau = 120.0 + 37.0 * (scene_id % 7)
    w = 0.11 + 0.013 * (scene_id % 5)
    env = np.exp(-t / tau) * (1.0 - np.exp(-t / 8.0))
    v = env * np.sin(w * t)
    i = 0.02 * env * np.cos(w * t + 0.3)
    return np.stack([v, i], axis=1).astype(np.float32)


class FakeStack:
    def __init__(self, ids):
        self.ids = list(ids)
        self.t = 0
        self.rec = []
        self.slots = {}
        self.next_slot = 0
        self.steps_log = []

    def step(self, n):
        self.rec.append(np.stack([series_of(s, self.t, n) for s in self.ids], axis=1))
        self.t += n
        self.steps_log.append(n)

    def _take(self):
        out = np.concatenate(self.rec) if self.rec else np.zeros((0, len(self.ids), 2), np.float32)
        self.rec = []
        return out

    def ports_take_series(self, n):
        return self._take()

    def ports_take_series_async(self):
        assert len(self.slots) < 2, "at most two takes may wait"
        k = self.next_slot
        self.next_slot ^= 1
        self.slots[k] = self._take()
        return k, self.slots[k].shape[0]

    def ports_collect_series(self, slot, rows):
        out = self.slots.pop(slot)
        assert out.shape[0] == rows
        return out

    def compact(self, keep):
        assert not self.rec and not self.slots, "compaction with a chunk still in flight"
        self.ids = [s for s, k in zip(self.ids, keep) if k]

    def close(self):
        pass


class FakeGroup:
    def __init__(self, scenes, indices, chunk, tune=True, far=None, ragged=False):
        self.indices = list(indices)
        self.scenes = [scenes[i] for i in indices]
        self.stack = FakeStack(indices)
        self.chunk = chunk
        self.far = None

    def compact(self, keep):
        self.stack.compact(keep)
        self.indices = [i for i, k in zip(self.indices, keep) if k]
        self.scenes = [s for s, k in zip(self.scenes, keep) if k]


@pytest.fixture
def scenes():
    return [configs.batched_scene(13, i, edges=(48,)) for i in range(9)]


def run(scenes, monkeypatch, pipelined, **kw):
    monkeypatch.setattr(batch, "_Group", FakeGroup)
    r = batch.BatchRunner(scenes, chunk=64, max_steps=4000, **kw)
    if not pipelined:
        r.far = "off"  # with far-field monitors the loop processes every chunk before the next
    res = r.run()
    return r, res


def test_one_chunk_ahead_equals_chunk_by_chunk(scenes, monkeypatch):
    _, a = run(scenes, monkeypatch, True)
    _, b = run(scenes, monkeypatch, False)
    assert all(x.done for x in a)
    for x, y in zip(a, b):
        assert x.steps == y.steps and x.rung_down == y.rung_down
        np.testing.assert_array_equal(np.concatenate(x.series), np.concatenate(y.series))
        np.testing.assert_array_equal(x.sweep["z"], y.sweep["z"])


def test_ring_down_step_follows_the_reference_residual(scenes, monkeypatch):
    """Each scene stops at the first whole chunk after its minimum steps at which the residual of
    the series so far (largest |V| of the last 5 % over the peak) is at most 1e-3."""
    _, res = run(scenes, monkeypatch, True)
    for i, (sc, r) in enumerate(zip(scenes, res)):
        period = sc.wavelength / float(sc.grid.courant)
        lo = int(math.ceil(4.0 * period))
        full = series_of(i, 0, 4000)
        want = None
        for n in range(64, 4001, 64):
            if n >= lo and batch.residual(full[:n, 0]) <= 1e-3:
                want = n
                break
        assert want is not None and r.steps == want, (i, r.steps, want)
        np.testing.assert_array_equal(np.concatenate(r.series), full[:want])


def test_decisions_with_one_chunk_in_flight(scenes, monkeypatch):
    """decide() sees each scene's series up to its decision step; accepted scenes stop there and
    rejected ones run on to ring-down exactly as without a decision."""
    _, ref = run(scenes, monkeypatch, True)
    at = [130 + 17 * i for i in range(len(scenes))]
    seen = {}

    def decide(idx, series):
        for i, s in zip(idx, series):
            seen[i] = s.shape[0]
        return [i % 2 == 0 for i in idx]

    _, res = run(scenes, monkeypatch, True, decide_at=at, decide=decide)
    for i, (r, q) in enumerate(zip(res, ref)):
        if q.steps > at[i]:
            assert seen[i] == at[i]
        if i in seen and i % 2 == 0:
            assert r.accepted and r.steps == at[i]
        else:
            assert r.steps == q.steps
            np.testing.assert_array_equal(r.sweep["z"], q.sweep["z"])
