"""Host logic of the served form's request loop (scone_gb300/serve.py) against a fake batch: admission
waits while the arena is full and resumes when completions free memory; latency is arrival to
completion; the Poisson driver offers the requested rate.  No GPU is used."""
import numpy as np

from scone_gb300 import serve


class FakeBatch:
    """Stands in for BatchGPU: `capacity` instances fit the arena; every pump completes the oldest
    submitted request with a fixed device latency."""

    def __init__(self, capacity):
        self.capacity = capacity
        self.live = set()
        self.queue = []
        self.t = 0.0
        self.next_slot = 100

    def clock(self):
        return self.t

    def serve_start(self, wave, item=0):
        self.wave = wave

    def instance(self, parent, pop, cycles, master):
        if len(self.live) >= self.capacity:
            return None
        s = self.next_slot
        self.next_slot += 1
        self.live.add(s)
        return s

    def submit(self, slot):
        self.queue.append(slot)

    def pump(self, wait=False):
        if not self.queue:
            return []
        s = self.queue.pop(0)
        return [(s, 0.5)]

    def bins(self, slot):
        return np.zeros((1, 3))

    def remove(self, slot):
        self.live.remove(slot)

    def serve_stop(self):
        pass


def test_admission_waits_for_memory():
    B = FakeBatch(capacity=2)
    S = serve.SolveServer(B, catalogue=[7, 8, 9])
    reqs = [serve.Request(i, "fixed", i % 3, 10, 2, 1234 + i, arrival=0.0) for i in range(5)]
    for r in reqs:
        S.submit(r)
    assert len(S.running) == 2 and len(S.waiting) == 3      # the arena holds two instances
    done = []
    B.t = 1.0
    while S.outstanding():
        done += S.pump()
        assert len(B.live) <= 2
    assert sorted(r.rid for r in done) == list(range(5))
    for r in done:
        # latency = device latency since submission + time spent waiting for admission
        assert abs(r.latency - (0.5 + (r.submitted - r.arrival))) < 1e-12
    assert all(r.bins is not None for r in done)


def test_poisson_driver_offers_the_rate():
    class Clocked(FakeBatch):
        def clock(self):
            self.t += 1e-4                                   # 0.1 ms per call
            return self.t

    B = Clocked(capacity=10 ** 6)
    S = serve.SolveServer(B, catalogue=list(range(4)))
    done, wall, n = serve.poisson_run(S, [(100, 2)] * 4, rate=500.0, duration=2.0, seed=3)
    assert 800 <= n <= 1200                                  # ~1000 arrivals in 2 s at 500/s
    assert len(done) == n
    s = serve.latency_summary(done, wall, 500.0 * 200)
    assert s["completed"] == n and s["p99_ms"] >= s["p50_ms"] > 0
    assert s["by_kind"]["fixed"]["completed"] == n


def test_latency_summary_by_kind():
    reqs = []
    for i in range(10):
        r = serve.Request(i, "fixed" if i < 8 else "eigen", 0, 10, 1, i, arrival=0.0)
        r.latency = 0.01 if i < 8 else 2.0
        reqs.append(r)
    s = serve.latency_summary(reqs, 1.0, 0.0)
    assert s["by_kind"]["fixed"] == {"completed": 8, "p50_ms": 10.0, "p99_ms": 10.0}
    assert s["by_kind"]["eigen"]["completed"] == 2 and abs(s["by_kind"]["eigen"]["p50_ms"] - 2000.0) < 1e-9
    assert s["p99_ms"] > 1000.0                       # the overall tail is the eigenvalue requests
