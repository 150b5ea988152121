"""Request loop of the served form: independent fixed-source solves arriving over time, run by
continuous batching on one GPU.

The problem catalogue (geometry, MG data, sources, clerks) stays resident in a BatchGPU arena.  A
request names a catalogue entry, a history count and an RNG seed; it is admitted as an instance
(its own score memory, taken from the arena, so the arena's size is the HBM budget that admission
obeys) as soon as memory allows, and joins the next wave of the batched kernel: every wave gives
each active request an equal share of its histories, so requests that arrive while others run start
at once and overlap with them on the device.  Completed requests return their scoreMemory bins and
their latency (arrival to device completion of their last wave).

Eigenvalue requests (the lattice k-eigenvalue problem) run on a small pool of resident
TransportOperatorGPU handles, one cycle per loop turn, on their own CUDA streams beside the waves.
Their admission policy protects the fixed-source requests under overload: at most the pool's size
run at once; an arrival that finds `eigen_queue_max` requests already waiting is shed (completed at
once with status "shed"); and while the fixed-source backlog (histories queued on the device) exceeds
`defer_backlog`, no eigenvalue cycle is launched that turn (the running ones are deferred).
"""
import collections
import math

import numpy as np

from . import abi, gpu


class Request:
    __slots__ = ("rid", "kind", "template", "pop", "cycles", "master", "arrival", "slot", "submitted",
                 "latency", "bins", "k", "handle", "cycle", "histories", "status")

    def __init__(self, rid, kind, template, pop, cycles, master, arrival):
        self.rid, self.kind, self.template = rid, kind, template
        self.pop, self.cycles, self.master, self.arrival = pop, cycles, master, arrival
        self.slot = self.submitted = self.latency = self.bins = self.k = self.handle = None
        self.cycle = 0
        self.histories = pop * cycles
        self.status = "queued"


class EigenPool:
    """Resident lattice eigenvalue handles; a request takes one, runs inactive + active cycles."""

    def __init__(self, problem, size, precision, transport, pop, form=abi.FORM_HISTORY):
        self.problem = problem
        self.free = []
        for _ in range(size):
            t = gpu.TransportOperatorGPU(problem, precision=precision, transport=transport,
                                         max_bank=int(2.5 * pop) + 4096, form=form)
            inact = t.upload_tally([])
            ia = t.upload_tally([abi.clerk(abi.CLERK_KEFF_ANALOG)])
            act = t.upload_tally([])
            aa = t.upload_tally([abi.clerk(abi.CLERK_KEFF_IMPLICIT)])
            t.attach_tally(inact, ia)
            t.attach_tally(act, aa)
            self.free.append((t, (inact, ia, act, aa)))

    def take(self):
        return self.free.pop() if self.free else None

    def give(self, h):
        self.free.append(h)


class SolveServer:
    """Continuous-batching request loop over a BatchGPU (fixed-source requests) and an optional
    EigenPool (eigenvalue requests)."""

    def __init__(self, batch, catalogue, wave_histories=1 << 23, item_histories=256, eigen=None,
                 eigen_cycles=(20, 40), eigen_share=2, eigen_queue_max=None, defer_backlog=None):
        self.B = batch
        self.catalogue = catalogue            # resident slots that requests instantiate
        self.waiting = collections.deque()    # fixed-source requests not yet admitted (arena full)
        self.running = {}                     # slot -> request
        self.eigen = eigen
        self.eigen_cycles = eigen_cycles
        self.eigen_waiting = collections.deque()
        self.eigen_running = []
        self.done = []
        self.eigen_share = eigen_share        # blocks per SM the waves leave free while eigen requests run
        self.eigen_queue_max = eigen_queue_max  # eigen arrivals beyond this many waiting are shed (None: never)
        self.defer_backlog = defer_backlog    # fixed-source histories queued above which eigen cycles wait
        self.shed = 0
        self.deferred_turns = 0
        self.B.serve_start(wave_histories, item_histories)

    # ---- requests
    def submit(self, req):
        if req.kind == "eigen":
            if self.eigen_queue_max is not None and len(self.eigen_waiting) >= self.eigen_queue_max:
                req.status = "shed"                    # rejected at arrival: the eigen queue is full
                req.latency = 0.0
                self.shed += 1
                self.done.append(req)
                return
            self.eigen_waiting.append(req)
        else:
            self.waiting.append(req)
        self._admit()

    def _admit(self):
        while self.waiting:
            r = self.waiting[0]
            slot = self.B.instance(self.catalogue[r.template], r.pop, r.cycles, r.master)
            if slot is None:
                break                          # HBM budget exhausted: wait for completions
            self.waiting.popleft()
            r.slot = slot
            r.submitted = self.B.clock()
            r.status = "running"
            self.B.submit(slot)
            self.running[slot] = r
        while self.eigen_waiting and self.eigen is not None:
            h = self.eigen.take()
            if h is None:
                break
            r = self.eigen_waiting.popleft()
            t, (inact, ia, act, aa) = h
            t.eigen_init(r.pop, r.master)
            r.handle = h
            r.submitted = self.B.clock()
            r.status = "running"
            self.eigen_running.append(r)

    def _eigen_step(self):
        """One cycle of every running eigenvalue request."""
        still = []
        for r in self.eigen_running:
            t, (inact, ia, act, aa) = r.handle
            if r.cycle < self.eigen_cycles[0]:
                t.eigen_cycle(inact, ia)
            else:
                st = t.eigen_cycle(act, aa)
                r.k = st.k_new
            r.cycle += 1
            if r.cycle >= sum(self.eigen_cycles):
                r.latency = self.B.clock() - r.arrival
                r.k = t.keff(aa)
                r.status = "done"
                self.eigen.give(r.handle)
                r.handle = None
                self.done.append(r)
            else:
                still.append(r)
        self.eigen_running = still

    def pump(self, wait=False):
        """Launch and retire waves; returns the requests completed since the last call."""
        for slot, lat in self.B.pump(wait=wait and bool(self.running) and not self.eigen_running):
            r = self.running.pop(slot)
            r.latency = lat + (r.submitted - r.arrival)
            r.bins = self.B.bins(slot)
            r.status = "done"
            self.B.remove(slot)
            self.done.append(r)
        if self.eigen_running:
            if self.defer_backlog is not None and (self.waiting or self.B.serve_status()[0] > self.defer_backlog):
                self.deferred_turns += 1               # fixed-source backlog: eigen cycles wait a turn
            else:
                self._eigen_step()
        self._admit()
        if self.eigen is not None and hasattr(self.B, "serve_share"):
            self.B.serve_share(self.eigen_share, bool(self.eigen_running))
        out, self.done = self.done, []
        return out

    def outstanding(self):
        return len(self.waiting) + len(self.running) + len(self.eigen_waiting) + len(self.eigen_running)

    def queue_state(self):
        """(fixed-source requests waiting for memory, histories queued on the device, fixed-source
        requests running, eigenvalue requests waiting, eigenvalue requests running)."""
        return (len(self.waiting), int(self.B.serve_status()[0]), len(self.running), len(self.eigen_waiting),
                len(self.eigen_running))

    def stop(self):
        self.B.serve_stop()


def poisson_run(server, templates, rate, duration, seed=1, eigen_fraction=0.0, eigen_pop=100000,
                drain=True, max_drain_s=120.0, queue_log=None, log_every=0.5):
    """Drives `server` with a Poisson arrival stream of `rate` requests/s for `duration` seconds.
    templates: [(pop, cycles)] of the catalogue entries (fixed-source requests copy their entry's
    size); a fraction `eigen_fraction` of requests are eigenvalue requests.  Returns the completed
    requests and the wall time.  With a list `queue_log`, (seconds since start, *server.queue_state())
    is appended every `log_every` seconds."""
    rng = np.random.default_rng(seed)
    clock = server.B.clock
    t0 = clock()
    next_at = t0 + rng.exponential(1.0 / rate)
    rid = 0
    finished = []
    end = t0 + duration
    next_log = t0
    while True:
        now = clock()
        if queue_log is not None and now >= next_log:
            queue_log.append((now - t0,) + server.queue_state())
            next_log += log_every
        while next_at <= now and next_at < end:
            if eigen_fraction > 0 and rng.uniform() < eigen_fraction:
                cyc = sum(server.eigen_cycles)
                r = Request(rid, "eigen", -1, eigen_pop, cyc, int(rng.integers(1, 2 ** 62)), next_at)
            else:
                k = int(rng.integers(len(templates)))
                pop, cycles = templates[k]
                r = Request(rid, "fixed", k, pop, cycles, int(rng.integers(1, 2 ** 62)), next_at)
            server.submit(r)
            rid += 1
            next_at += rng.exponential(1.0 / rate)
        if now >= end and (not drain or server.outstanding() == 0 or now > end + max_drain_s):
            break
        idle = next_at - now
        finished += server.pump(wait=idle > 0.002 or now >= end)
    wall = clock() - t0
    return finished, wall, rid


def latency_summary(reqs, wall, offered_histories):
    """Completed requests, latency percentiles over all of them and per request kind (fixed-source
    requests take milliseconds, eigenvalue requests seconds), and the achieved history rate."""
    shed = [r for r in reqs if r.status == "shed"]
    reqs = [r for r in reqs if r.status != "shed"]
    lat = np.array([r.latency for r in reqs]) if reqs else np.zeros(1)
    hist = float(sum(r.histories for r in reqs))
    by_kind = {}
    for kind in sorted({r.kind for r in reqs}):
        lk = np.array([r.latency for r in reqs if r.kind == kind])
        by_kind[kind] = {"completed": int(lk.size), "p50_ms": float(np.percentile(lk, 50) * 1e3),
                         "p99_ms": float(np.percentile(lk, 99) * 1e3)}
    return {
        "completed": len(reqs),
        "p50_ms": float(np.percentile(lat, 50) * 1e3),
        "p99_ms": float(np.percentile(lat, 99) * 1e3),
        "mean_ms": float(lat.mean() * 1e3),
        "by_kind": by_kind,
        "histories_per_s": hist / wall if wall > 0 else 0.0,
        "offered_histories_per_s": offered_histories,
        "wall_s": wall,
        "shed": len(shed),
        "shed_histories": float(sum(r.histories for r in shed)),
    }


def queue_growth(log):
    """Summary of a queue log of poisson_run: the largest and last value of each queue and the
    growth rate (per second, least squares) of the fixed-source device backlog and of the waiting
    requests over the second half of the run."""
    if len(log) < 4:
        return {}
    a = np.array(log, dtype=np.float64)
    names = ["fixed_waiting_for_memory", "device_backlog_histories", "fixed_running", "eigen_waiting", "eigen_running"]
    out = {"samples": int(a.shape[0])}
    half = a[a[:, 0] >= a[-1, 0] / 2]
    for i, n in enumerate(names):
        col = a[:, i + 1]
        out[n] = {"max": float(col.max()), "last": float(col[-1])}
        if half.shape[0] >= 2 and n in ("fixed_waiting_for_memory", "device_backlog_histories", "eigen_waiting"):
            out[n]["growth_per_s_second_half"] = float(np.polyfit(half[:, 0], half[:, i + 1], 1)[0])
    return out
