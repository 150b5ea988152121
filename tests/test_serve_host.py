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


class FakeEigenHandle:
    """Stands in for a TransportOperatorGPU of the eigen pool: counts the cycles it runs."""

    def __init__(self):
        self.cycles = 0

    def eigen_init(self, pop, master):
        self.cycles = 0

    def eigen_cycle(self, admin, atch):
        self.cycles += 1

        class St:
            k_new = 1.0
        return St()

    def keff(self, admin):
        return 1.0, 0.001


class FakePool:
    def __init__(self, size):
        self.free = [(FakeEigenHandle(), (0, 1, 2, 3)) for _ in range(size)]

    def take(self):
        return self.free.pop() if self.free else None

    def give(self, h):
        self.free.append(h)


class BacklogBatch(FakeBatch):
    """FakeBatch that reports a device backlog (histories queued) the test sets."""
    backlog = 0

    def serve_status(self):
        return self.backlog, len(self.queue), 0


def test_eigen_requests_shed_when_their_queue_is_full():
    B = BacklogBatch(capacity=100)
    S = serve.SolveServer(B, catalogue=[0], eigen=FakePool(1), eigen_cycles=(1, 2), eigen_queue_max=2)
    reqs = [serve.Request(i, "eigen", -1, 10, 3, i, arrival=0.0) for i in range(5)]
    for r in reqs:
        S.submit(r)
    # one runs (the pool has one handle), two wait, the last two are shed at arrival
    assert len(S.eigen_running) == 1 and len(S.eigen_waiting) == 2 and S.shed == 2
    done = []
    while S.outstanding():
        done += S.pump()
    done += S.pump()
    shed = [r for r in done if r.status == "shed"]
    assert sorted(r.rid for r in shed) == [3, 4]
    assert all(r.status == "done" and r.k is not None for r in done if r.rid < 3)
    s = serve.latency_summary(done, 1.0, 0.0)
    assert s["shed"] == 2 and s["completed"] == 3 and s["shed_histories"] == 60


def test_eigen_cycles_wait_while_the_fixed_source_backlog_is_high():
    B = BacklogBatch(capacity=100)
    S = serve.SolveServer(B, catalogue=[0], eigen=FakePool(1), eigen_cycles=(1, 2), defer_backlog=1000)
    S.submit(serve.Request(0, "eigen", -1, 10, 3, 5, arrival=0.0))
    h = S.eigen_running[0].handle[0]
    B.backlog = 5000
    for _ in range(4):
        S.pump()
    assert h.cycles == 0 and S.deferred_turns == 4           # deferred while the backlog is high
    B.backlog = 0
    done = []
    while S.outstanding():
        done += S.pump()
    assert h.cycles == 3 and done[0].status == "done"


def test_queue_growth_summary():
    log = [(0.5 * i, 0, 1000 * i, 3, i // 2, 1) for i in range(20)]
    g = serve.queue_growth(log)
    assert g["samples"] == 20
    assert abs(g["device_backlog_histories"]["growth_per_s_second_half"] - 2000.0) < 1e-6
    assert g["eigen_waiting"]["max"] == 9
