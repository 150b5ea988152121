"""Python face of libsconegpu (ctypes over the C ABI in include/scone_gpu.h).

`TransportOperatorGPU` plays the role of SCONE's transportOperator + collisionOperator for a whole
particle bank: it owns the resident geometry (geometryStd), MG nuclear data (baseMgNeutronDatabase)
and tally admins (tallyAdmin / tallyClerk / scoreMemory) on the GPU.  There is no CPU fallback:
constructing it without the compiled library or without a CUDA device raises.
"""
import ctypes as C
import os

import numpy as np

from . import abi

_LIB = None


def library_path():
    return os.path.join(os.path.dirname(os.path.abspath(__file__)), "_build", "libsconegpu.so")


def load(build=True):
    """Load (building first if needed) libsconegpu.so; raises if it cannot be loaded."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = library_path()
    if build:
        from . import build as _b
        _b.build()
    if not os.path.exists(path):
        raise RuntimeError(f"libsconegpu.so is missing at {path}; run scone_gb300.build.build()")
    L = C.CDLL(path)
    vp, i32, i64, u64, f64, P = C.c_void_p, C.c_int32, C.c_int64, C.c_uint64, C.c_double, C.POINTER
    sig = {
        "sg_create": (i32, [P(abi.Config), P(vp)]), "sg_destroy": (i32, [vp]),
        "sg_last_error": (i32, [vp, C.c_char_p, C.c_size_t]),
        "sg_upload_geometry": (i32, [vp, P(abi.GeometryDesc)]),
        "sg_upload_mg": (i32, [vp, P(abi.MGDesc)]),
        "sg_upload_ce": (i32, [vp, P(abi.CEDesc)]),
        "sg_upload_tally": (i32, [vp, P(abi.TallyDesc), P(i32)]),
        "sg_set_collision": (i32, [vp, P(abi.CollisionDesc)]),
        "sg_attach_tally": (i32, [vp, i32, i32]),
        "sg_set_point_source": (i32, [vp, P(abi.PointSourceDesc)]),
        "sg_generate_source": (i32, [vp, u64, i32, P(abi.Bank)]),
        "sg_transport_bank": (i32, [vp, i32, P(abi.Bank), i32, u64, f64, P(abi.Bank), i32, P(abi.CycleStats)]),
        "sg_tally_cycle_start": (i32, [vp, i32, f64]), "sg_tally_cycle_end": (i32, [vp, i32, f64, f64]),
        "sg_tally_size": (i32, [vp, i32, P(i64)]), "sg_get_bins": (i32, [vp, i32, P(f64), i64]),
        "sg_get_keff": (i32, [vp, i32, P(f64), P(f64)]),
        "sg_eigen_init": (i32, [vp, i32, u64, f64]), "sg_eigen_cycle": (i32, [vp, i32, i32, P(abi.CycleStats)]),
        "sg_eigen_state": (i32, [vp, P(u64), P(f64)]), "sg_eigen_get_bank": (i32, [vp, P(abi.Bank), i32, P(i32)]),
        "sg_eigen_cycle_bank": (i32, [vp, i32, i32, P(abi.Bank), i32, P(u64), P(f64), f64, P(abi.Bank),
                                      P(abi.CycleStats)]),
        "sg_fixed_source_cycle": (i32, [vp, i32, i32, P(u64), P(abi.CycleStats)]),
        "sg_fixed_source_cycle_shard": (i32, [vp, i32, i32, i32, P(u64), P(abi.CycleStats)]),
        "sg_normalise_shard": (i32, [vp, P(abi.Bank), i32, i64, i64, i32, u64, P(abi.Bank), i32, P(i32)]),
        "sg_tally_get_scores": (i32, [vp, i32, P(f64), i64]), "sg_tally_set_scores": (i32, [vp, i32, P(f64), i64]),
        "sg_set_file_source": (i32, [vp, P(abi.Bank), i32]),
        "sg_bank_write_file": (i32, [C.c_char_p, P(abi.Bank), i32, i32]),
        "sg_bank_count_file": (i32, [C.c_char_p, i32, P(i64)]),
        "sg_bank_read_file": (i32, [C.c_char_p, i32, P(abi.Bank), i32, P(i32)]),
        "sg_get_history_records": (i32, [vp, P(i32), P(u64), i32]),
        "sg_rng_draws": (i32, [P(u64), P(f64), i32]), "sg_rng_skip": (u64, [u64, i64]),
        "sg_transport_bank_noalloc": (i32, [vp, i32, P(abi.Bank), i32, u64, f64, P(abi.Bank), i32, P(i32)]),
        "sg_batch_create": (i32, [P(abi.BatchConfig), P(vp)]), "sg_batch_destroy": (i32, [vp]),
        "sg_batch_last_error": (i32, [vp, C.c_char_p, C.c_size_t]),
        "sg_batch_add": (i32, [vp, P(abi.ProblemDesc), P(i32)]), "sg_batch_remove": (i32, [vp, i32]),
        "sg_batch_instance": (i32, [vp, i32, i32, i32, u64, P(i32)]),
        "sg_batch_memory": (i32, [vp, P(i64), P(i64)]),
        "sg_batch_set_tuning": (i32, [vp, P(abi.BatchTuning)]), "sg_batch_get_tuning": (i32, [vp, P(abi.BatchTuning)]),
        "sg_batch_run": (i32, [vp, P(i32), i32, P(abi.BatchStats)]),
        "sg_batch_run_plain": (i32, [vp, P(i32), i32, i32, P(abi.BatchStats)]),
        "sg_batch_autotune": (i32, [vp, P(i32), i32, P(abi.BatchTuning)]),
        "sg_batch_autotune_plain": (i32, [vp, P(i32), i32, P(abi.EventTuning)]),
        "sg_set_event_tuning": (i32, [vp, P(abi.EventTuning)]), "sg_get_event_tuning": (i32, [vp, P(abi.EventTuning)]),
        "sg_batch_tally_size": (i32, [vp, i32, P(i64)]), "sg_batch_get_bins": (i32, [vp, i32, P(f64), i64]),
        "sg_batch_clear_tally": (i32, [vp, i32]),
        "sg_serve_start": (i32, [vp, i64, i32]), "sg_serve_submit": (i32, [vp, i32]),
        "sg_serve_pump": (i32, [vp, i32, P(i32), P(f64), i32, P(i32)]), "sg_serve_stop": (i32, [vp]),
        "sg_serve_status": (i32, [vp, P(i64), P(i32), P(i64)]), "sg_serve_clock": (f64, []),
        "sg_serve_counts": (i32, [vp, P(i64), P(i64)]), "sg_serve_share": (i32, [vp, i32, i32]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype, fn.argtypes = res, args
    _LIB = L
    return L


class SconeGpuError(RuntimeError):
    pass


class TransportOperatorGPU:
    """A GPU transport operator for whole banks (the `gen:` loop of SCONE's physics packages)."""

    def __init__(self, problem=None, precision=abi.PREC_FP64, transport=abi.TRANSPORT_ST, max_bank=1 << 20,
                 device=0, record_histories=False, form=abi.FORM_EVENT, ht_cutoff=0.0):
        self.L = load()
        self.h = C.c_void_p()
        self._keep = []
        cfg = abi.Config(precision, transport, device, max_bank, 1 if record_histories else 0, form, ht_cutoff)
        rc = self.L.sg_create(C.byref(cfg), C.byref(self.h))
        if rc != 0:
            raise SconeGpuError(f"sg_create failed with {rc} (is a CUDA device present?)")
        self.max_bank = max_bank
        if problem is not None:
            self.upload_geometry(problem.geometry)
            if problem.mg is not None:
                self.upload_mg(problem.mg)
            if getattr(problem, "ce", None) is not None:
                self.upload_ce(problem.ce)
            if problem.source:
                self.set_point_source(**problem.source)

    def _check(self, rc):
        if rc != 0:
            buf = C.create_string_buffer(512)
            self.L.sg_last_error(self.h, buf, 512)
            raise SconeGpuError(f"libsconegpu error {rc}: {buf.value.decode()}")
        return rc

    def close(self):
        if self.h:
            self.L.sg_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload_geometry(self, g):
        s, keep = abi.geometry_struct(g)
        self._keep.append(keep)
        self._check(self.L.sg_upload_geometry(self.h, C.byref(s)))

    def upload_mg(self, m):
        s, keep = abi.mg_struct(m)
        self._keep.append(keep)
        self._check(self.L.sg_upload_mg(self.h, C.byref(s)))

    def upload_ce(self, d):
        s, keep = abi.ce_struct(d)
        self._keep.append(keep)
        self._check(self.L.sg_upload_ce(self.h, C.byref(s)))

    def upload_tally(self, clerks, batch_size=1, norm_clerk=-1, norm_val=1.0):
        t, arr = abi.tally_struct(clerks, batch_size, norm_clerk, norm_val)
        self._keep.append(arr)
        a = C.c_int32()
        self._check(self.L.sg_upload_tally(self.h, C.byref(t), C.byref(a)))
        return a.value

    def attach_tally(self, admin, atch):
        self._check(self.L.sg_attach_tally(self.h, admin, atch))

    def set_point_source(self, r, G=1, dir=(1.0, 0.0, 0.0), isotropic=True, prob_g=None, E=0.0):
        s, keep = abi.point_source_struct(r, G, dir, isotropic, prob_g, E)
        self._keep.append((s, keep))
        self._check(self.L.sg_set_point_source(self.h, C.byref(s)))

    def generate_source(self, master, n):
        b = abi.HostBank(n)
        self._check(self.L.sg_generate_source(self.h, C.c_uint64(master), n, C.byref(b.struct)))
        return b

    def transport_bank(self, admin, bank, master, k_eff=1.0, next_cap=None):
        n = bank.n
        cap = next_cap if next_cap is not None else max(4 * n, 16)
        nxt = abi.HostBank(cap)
        st = abi.CycleStats()
        self._check(self.L.sg_transport_bank(self.h, admin, C.byref(bank.struct), n, C.c_uint64(master), k_eff,
                                             C.byref(nxt.struct), cap, C.byref(st)))
        return nxt, st

    def tally_cycle_start(self, admin, w):
        self._check(self.L.sg_tally_cycle_start(self.h, admin, w))

    def tally_cycle_end(self, admin, w, k=1.0):
        self._check(self.L.sg_tally_cycle_end(self.h, admin, w, k))

    def bins(self, admin):
        n = C.c_int64()
        self._check(self.L.sg_tally_size(self.h, admin, C.byref(n)))
        out = np.zeros(3 * max(n.value, 1))
        self._check(self.L.sg_get_bins(self.h, admin, out.ctypes.data_as(C.POINTER(C.c_double)), n.value))
        return out[:3 * n.value].reshape(3, n.value).T.copy()

    def normalise_shard(self, sites, n, before, tot_sites, tot_pop, master, cap):
        """This process's part of normSize_Repr over a population split over processes
        (sg_normalise_shard): returns (bank, n_out)."""
        out = abi.HostBank(max(cap, 1))
        m = C.c_int32()
        self._check(self.L.sg_normalise_shard(self.h, C.byref(sites.struct), n, before, tot_sites, tot_pop,
                                                C.c_uint64(master), C.byref(out.struct), cap, C.byref(m)))
        return out, m.value

    def _tally_n(self, admin):
        n = C.c_int64()
        self._check(self.L.sg_tally_size(self.h, admin, C.byref(n)))
        return n.value

    def get_scores(self, admin):
        """The running-batch scores of an admin (summed over processes for a synchronised tally)."""
        out = np.zeros(max(self._tally_n(admin), 1))
        self._check(self.L.sg_tally_get_scores(self.h, admin, out.ctypes.data_as(C.POINTER(C.c_double)), out.size))
        return out[:self._tally_n(admin)].copy()

    def set_scores(self, admin, scores):
        s = np.ascontiguousarray(scores, dtype=np.float64)
        if s.size < self._tally_n(admin):
            raise ValueError("set_scores: fewer values than the tally has bins")
        self._check(self.L.sg_tally_set_scores(self.h, admin, s.ctypes.data_as(C.POINTER(C.c_double)), s.size))

    def keff(self, admin):
        k, s = C.c_double(), C.c_double()
        self._check(self.L.sg_get_keff(self.h, admin, C.byref(k), C.byref(s)))
        return k.value, s.value

    def history_records(self, n):
        c = np.zeros(n, np.int32)
        r = np.zeros(n, np.uint64)
        self._check(self.L.sg_get_history_records(self.h, c.ctypes.data_as(C.POINTER(C.c_int32)),
                                                  r.ctypes.data_as(C.POINTER(C.c_uint64)), n))
        return c, r

    def eigen_init(self, pop, master, k0=1.0):
        self._check(self.L.sg_eigen_init(self.h, pop, C.c_uint64(master), k0))

    def eigen_cycle(self, admin, atch):
        st = abi.CycleStats()
        self._check(self.L.sg_eigen_cycle(self.h, admin, atch, C.byref(st)))
        return st

    def eigen_cycle_bank(self, admin, atch, bank, pop, master, k_eff, k_end, out):
        """One whole eigenvalue cycle on host banks (thisCycle `bank`, normalised next bank into
        `out`); returns (master, k_new, stats)."""
        m, k = C.c_uint64(master), C.c_double(k_eff)
        st = abi.CycleStats()
        self._check(self.L.sg_eigen_cycle_bank(self.h, admin, atch, C.byref(bank.struct), pop, C.byref(m), C.byref(k),
                                               k_end, C.byref(out.struct), C.byref(st)))
        return m.value, k.value, st

    def eigen_state(self):
        m, k = C.c_uint64(), C.c_double()
        self._check(self.L.sg_eigen_state(self.h, C.byref(m), C.byref(k)))
        return m.value, k.value

    def eigen_bank(self, cap):
        b = abi.HostBank(cap)
        pop = C.c_int32()
        self._check(self.L.sg_eigen_get_bank(self.h, C.byref(b.struct), cap, C.byref(pop)))
        return b, pop.value

    def set_collision(self, desc):
        """neutronMGimp / neutronCEimp options (an abi.collision() description)."""
        self._keep.append(desc)
        self._check(self.L.sg_set_collision(self.h, C.byref(desc)))

    def set_file_source(self, bank):
        """fileSource: fixed-source cycles sample their particles from this host bank."""
        self._keep.append(bank)
        self._check(self.L.sg_set_file_source(self.h, C.byref(bank.struct), bank.n))

    def fixed_source_cycle(self, admin, n, master, total=None):
        """One fixed-source cycle of n histories; with `total`, n is this process's share of a
        population of `total` split over processes (master already strided by the offset)."""
        m = C.c_uint64(master)
        st = abi.CycleStats()
        if total is None:
            self._check(self.L.sg_fixed_source_cycle(self.h, admin, n, C.byref(m), C.byref(st)))
        else:
            self._check(self.L.sg_fixed_source_cycle_shard(self.h, admin, n, total, C.byref(m), C.byref(st)))
        return m.value, st


class BatchGPU:
    """Many independent fixed-source problems resident on one GPU (sg_batch_* / sg_serve_*).

    ``add(problem, pop, cycles, master)`` uploads a problem into the batch arena and returns its slot;
    ``run(slots)`` transports every cycle of the listed problems in one persistent launch (the batched
    form); ``run_plain(slots, form)`` runs them one problem per launch sequence (the plain form);
    ``bins(slot)`` returns scoreMemory bins(N, {BIN, CSUM, CSUM2}) as an (N, 3) array.  Serving:
    ``serve_start(wave_histories)``, ``submit(slot)``, ``pump(wait)`` -> [(slot, latency_s)]."""

    def __init__(self, precision=abi.PREC_MIXED, transport=abi.TRANSPORT_DT, device=0, max_problems=4096,
                 arena_bytes=1 << 30, max_work_items=1 << 20, ht_cutoff=0.0):
        self.L = load()
        self.b = C.c_void_p()
        cfg = abi.BatchConfig(precision, transport, device, max_problems, arena_bytes, max_work_items, 0, ht_cutoff)
        rc = self.L.sg_batch_create(C.byref(cfg), C.byref(self.b))
        if rc != 0:
            raise SconeGpuError(f"sg_batch_create failed with {rc} (is a CUDA device present?)")
        self.meta = {}

    def _check(self, rc, ok=(0,)):
        if rc not in ok:
            buf = C.create_string_buffer(512)
            self.L.sg_batch_last_error(self.b, buf, 512)
            raise SconeGpuError(f"libsconegpu error {rc}: {buf.value.decode()}")
        return rc

    def close(self):
        if self.b:
            self.L.sg_batch_destroy(self.b)
            self.b = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add(self, problem, pop, cycles, master, clerks=None):
        """Upload a fixed-source MG problem; returns its slot (SconeGpuError with code -2 when the
        arena or the slots are full)."""
        g, kg = abi.geometry_struct(problem.geometry)
        m, km = abi.mg_struct(problem.mg)
        src = dict(problem.source)
        s, ks = abi.point_source_struct(src.pop("r"), **src)
        t, kt = abi.tally_struct(clerks if clerks is not None else problem.tallies["flux"])
        d = abi.ProblemDesc(C.pointer(g), C.pointer(m), C.pointer(s), C.pointer(t), int(pop), int(cycles),
                            C.c_uint64(master))
        slot = C.c_int32()
        self._check(self.L.sg_batch_add(self.b, C.byref(d), C.byref(slot)))
        self.meta[slot.value] = dict(pop=int(pop), cycles=int(cycles))
        del kg, km, ks, kt
        return slot.value

    def try_add(self, problem, pop, cycles, master, clerks=None):
        """As add, but returns None when the arena or the slots are full (admission by HBM budget)."""
        try:
            return self.add(problem, pop, cycles, master, clerks)
        except SconeGpuError as e:
            if "error -2:" in str(e):
                return None
            raise

    def instance(self, parent, pop, cycles, master):
        """A request on resident problem `parent`'s data with its own size, seed and score memory;
        None when the arena or the slots are full (admission by HBM budget)."""
        slot = C.c_int32()
        rc = self._check(self.L.sg_batch_instance(self.b, parent, int(pop), int(cycles), C.c_uint64(master),
                                                  C.byref(slot)), ok=(0, -2))
        if rc == -2:
            return None
        self.meta[slot.value] = dict(pop=int(pop), cycles=int(cycles), parent=parent)
        return slot.value

    def remove(self, slot):
        self._check(self.L.sg_batch_remove(self.b, slot))
        self.meta.pop(slot, None)

    def memory(self):
        u, c = C.c_int64(), C.c_int64()
        self._check(self.L.sg_batch_memory(self.b, C.byref(u), C.byref(c)))
        return u.value, c.value

    @staticmethod
    def _slots(slots):
        a = np.ascontiguousarray(slots, dtype=np.int32)
        return a, a.ctypes.data_as(C.POINTER(C.c_int32))

    def tuning(self):
        t = abi.BatchTuning()
        self._check(self.L.sg_batch_get_tuning(self.b, C.byref(t)))
        return t.as_dict()

    def set_tuning(self, **kw):
        t = abi.BatchTuning()
        self._check(self.L.sg_batch_get_tuning(self.b, C.byref(t)))
        for k, v in kw.items():
            setattr(t, k, int(v))
        self._check(self.L.sg_batch_set_tuning(self.b, C.byref(t)))

    def run(self, slots):
        a, p = self._slots(slots)
        st = abi.BatchStats()
        self._check(self.L.sg_batch_run(self.b, p, len(a), C.byref(st)))
        return st

    def run_plain(self, slots, form=abi.FORM_EVENT):
        a, p = self._slots(slots)
        st = abi.BatchStats()
        self._check(self.L.sg_batch_run_plain(self.b, p, len(a), form, C.byref(st)))
        return st

    def autotune(self, slots):
        a, p = self._slots(slots)
        t = abi.BatchTuning()
        self._check(self.L.sg_batch_autotune(self.b, p, len(a), C.byref(t)))
        return t.as_dict()

    def autotune_plain(self, slots):
        """Queue thresholds of the plain event form, picked by timing on the listed problems."""
        a, p = self._slots(slots)
        t = abi.EventTuning()
        self._check(self.L.sg_batch_autotune_plain(self.b, p, len(a), C.byref(t)))
        return t.as_dict()

    def bins(self, slot):
        n = C.c_int64()
        self._check(self.L.sg_batch_tally_size(self.b, slot, C.byref(n)))
        out = np.zeros(3 * max(n.value, 1))
        self._check(self.L.sg_batch_get_bins(self.b, slot, out.ctypes.data_as(C.POINTER(C.c_double)), n.value))
        return out[:3 * n.value].reshape(3, n.value).T.copy()

    def clear_tally(self, slot):
        self._check(self.L.sg_batch_clear_tally(self.b, slot))

    # ---- serving
    def serve_start(self, wave_histories, item_histories=0):
        self._check(self.L.sg_serve_start(self.b, int(wave_histories), int(item_histories)))

    def submit(self, slot):
        self._check(self.L.sg_serve_submit(self.b, slot))

    def pump(self, wait=False, cap=4096):
        s = np.zeros(cap, np.int32)
        lat = np.zeros(cap)
        n = C.c_int32()
        self._check(self.L.sg_serve_pump(self.b, 1 if wait else 0, s.ctypes.data_as(C.POINTER(C.c_int32)),
                                         lat.ctypes.data_as(C.POINTER(C.c_double)), cap, C.byref(n)))
        return list(zip(s[:n.value].tolist(), lat[:n.value].tolist()))

    def serve_status(self):
        q, a, w = C.c_int64(), C.c_int32(), C.c_int64()
        self._check(self.L.sg_serve_status(self.b, C.byref(q), C.byref(a), C.byref(w)))
        return q.value, a.value, w.value

    def serve_share(self, blocks_per_sm, on):
        """Leave `blocks_per_sm` resident blocks per SM to other streams while `on`."""
        self._check(self.L.sg_serve_share(self.b, int(blocks_per_sm), 1 if on else 0))

    def serve_counts(self):
        """(histories, flight events) of the waves retired since serve_start."""
        h, e = C.c_int64(), C.c_int64()
        self._check(self.L.sg_serve_counts(self.b, C.byref(h), C.byref(e)))
        return h.value, e.value

    def serve_stop(self):
        self._check(self.L.sg_serve_stop(self.b))

    def clock(self):
        return self.L.sg_serve_clock()


def write_bank_file(path, bank, n=None, binary=True):
    """particleDungeon%printToFile: `path` + .bin / .txt."""
    rc = load().sg_bank_write_file(path.encode(), C.byref(bank.struct), bank.n if n is None else n, int(binary))
    if rc != 0:
        raise SconeGpuError(f"sg_bank_write_file failed with {rc}")


def read_bank_file(path, binary=True):
    """The particles of a printToFile file (fileSource's reader), as an abi.HostBank."""
    L = load()
    cnt = C.c_int64()
    if L.sg_bank_count_file(path.encode(), int(binary), C.byref(cnt)) != 0:
        raise SconeGpuError(f"cannot read {path}")
    b = abi.HostBank(cnt.value)
    got = C.c_int32()
    if L.sg_bank_read_file(path.encode(), int(binary), C.byref(b.struct), cnt.value, C.byref(got)) != 0:
        raise SconeGpuError(f"cannot read {path}")
    return b


def rng_draws(state, n):
    L = load()
    s = C.c_uint64(state)
    out = np.zeros(n)
    L.sg_rng_draws(C.byref(s), out.ctypes.data_as(C.POINTER(C.c_double)), n)
    return out, s.value


def rng_skip(state, k):
    return load().sg_rng_skip(C.c_uint64(state), C.c_int64(k))
