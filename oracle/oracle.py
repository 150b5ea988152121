"""TEST INFRASTRUCTURE: ctypes loader of the CPU oracle (liboracle built from scone_oracle.cpp).

Only tests/, __graft_entry__.smoke() and bench.py's CPU legs import this module.  The oracle is a
scalar restatement of SCONE's algorithm and is never a product code path.
"""
import ctypes as C
import os
import subprocess

import numpy as np

from scone_gb300 import abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libsconeoracle.so")


def build(force=False):
    src = os.path.join(HERE, "scone_oracle.cpp")
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        vp = C.c_void_p
        i32, i64, u64, f64 = C.c_int32, C.c_int64, C.c_uint64, C.c_double
        P = C.POINTER
        sig = {
            "or_create": (i32, [i32, P(vp)]), "or_destroy": (i32, [vp]),
            "or_set_ht_cutoff": (i32, [vp, C.c_double]),
            "or_set_file_source": (i32, [vp, P(abi.Bank), i32]),
            "or_fixed_source_cycle_shard": (i32, [vp, i32, i32, i32, P(C.c_uint64), P(abi.CycleStats)]),
            "or_normalise_shard": (i32, [vp, P(abi.Bank), i32, C.c_int64, C.c_int64, i32, u64, P(abi.Bank), i32,
                                         P(i32)]),
            "or_normalise": (i32, [vp, P(abi.Bank), i32, i32, u64, P(abi.Bank), i32, P(i32)]),
            "or_tally_get_scores": (i32, [vp, i32, P(f64), C.c_int64]),
            "or_tally_set_scores": (i32, [vp, i32, P(f64), C.c_int64]),
            "or_sample_legendre_p1": (i32, [C.c_double, P(C.c_uint64), P(C.c_double), i32]),
            "or_last_error": (i32, [vp, C.c_char_p, C.c_size_t]),
            "or_upload_geometry": (i32, [vp, P(abi.GeometryDesc)]),
            "or_upload_mg": (i32, [vp, P(abi.MGDesc)]),
            "or_upload_tally": (i32, [vp, P(abi.TallyDesc), P(i32)]),
            "or_attach_tally": (i32, [vp, i32, i32]),
            "or_set_point_source": (i32, [vp, P(abi.PointSourceDesc)]),
            "or_generate_source": (i32, [vp, u64, i32, P(abi.Bank)]),
            "or_transport_bank": (i32, [vp, i32, P(abi.Bank), i32, u64, f64, P(abi.Bank), i32, P(abi.CycleStats)]),
            "or_tally_cycle_start": (i32, [vp, i32, f64]), "or_tally_cycle_end": (i32, [vp, i32, f64, f64]),
            "or_tally_size": (i32, [vp, i32, P(i64)]), "or_get_bins": (i32, [vp, i32, P(f64), i64]),
            "or_get_keff": (i32, [vp, i32, P(f64), P(f64)]),
            "or_get_history_records": (i32, [vp, P(i32), P(u64), i32]),
            "or_eigen_init": (i32, [vp, i32, u64, f64]), "or_eigen_cycle": (i32, [vp, i32, i32, P(abi.CycleStats)]),
            "or_eigen_cycle_omp": (i32, [vp, i32, i32, i32, P(abi.CycleStats)]),
            "or_eigen_state": (i32, [vp, P(u64), P(f64)]), "or_eigen_get_bank": (i32, [vp, P(abi.Bank), i32, P(i32)]),
            "or_fixed_source_cycle": (i32, [vp, i32, i32, P(u64), P(abi.CycleStats)]),
            "or_rng_draws": (i32, [P(u64), P(f64), i32]), "or_rng_skip": (u64, [u64, i64]),
            "or_surf_eval": (i32, [i32, P(f64), P(i32), P(f64), P(f64), P(f64)]),
            "or_surf_bc": (i32, [i32, P(f64), P(i32), i32, P(f64), P(f64)]),
            "or_coords_init": (i32, [vp, P(f64), P(f64)]), "or_coords_place": (i32, [vp]),
            "or_coords_move": (i32, [vp, i32, P(f64), P(i32)]),
            "or_coords_get": (i32, [vp, i32, P(f64), P(f64), P(i32)]),
            "or_what_is_at": (i32, [vp, P(f64), P(f64), P(i32), P(i32)]),
            "or_bounds": (i32, [vp, P(f64)]), "or_mg_info": (i32, [vp, i32, i32, P(f64)]),
            "or_rotate_vector": (i32, [P(f64), f64, f64, P(f64)]),
            "or_scoremem_new": (i32, [i64, i32, P(vp)]), "or_scoremem_free": (i32, [vp]),
            "or_scoremem_score": (i32, [vp, f64, i64]), "or_scoremem_accumulate": (i32, [vp, f64, i64]),
            "or_scoremem_close": (i32, [vp, f64]), "or_scoremem_reduce": (i32, [vp]),
            "or_scoremem_closebin": (i32, [vp, f64, i64]), "or_scoremem_closecycle": (i32, [vp, f64]), "or_scoremem_result": (i32, [vp, i64, i32, P(f64), P(f64)]),
            "or_timed_gen_loop": (i64, [vp, i32, P(abi.Bank), i32, u64, f64, i32, P(i64)]),
            "or_upload_ce": (i32, [vp, P(abi.CEDesc)]),
            "or_ce_micro": (i32, [vp, i32, f64, P(f64)]), "or_ce_mat_total": (i32, [vp, i32, f64, P(f64)]),
            "or_ce_majorant": (i32, [vp, f64, P(f64)]), "or_ce_union_size": (i32, [vp, P(i64)]),
            "or_asymptotic_scatter": (i32, [f64, f64, f64, P(f64)]),
            "or_target_velocity": (i32, [f64, P(f64), f64, f64, P(u64), P(f64)]),
            "or_grid_search": (i32, [P(f64), i32, f64]),
            "or_set_collision": (i32, [vp, P(abi.CollisionDesc)]),
            "or_map_point": (i32, [vp, P(abi.AxisDesc), i32, P(f64), i32, i32, i32, f64, i32, P(i32)]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype, fn.argtypes = res, args
        _lib = L
    return _lib


def _d(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a, a.ctypes.data_as(C.POINTER(C.c_double))


class Oracle:
    """Python face of the oracle with the same methods as scone_gb300.TransportOperatorGPU."""

    def __init__(self, problem=None, transport=abi.TRANSPORT_ST, ht_cutoff=0.0):
        self.L = lib()
        self.h = C.c_void_p()
        self._keep = []
        self._check(self.L.or_create(transport, C.byref(self.h)))
        if ht_cutoff > 0.0:
            self._check(self.L.or_set_ht_cutoff(self.h, ht_cutoff))
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
            self.L.or_last_error(self.h, buf, 512)
            raise RuntimeError(f"oracle error {rc}: {buf.value.decode()}")
        return rc

    def close(self):
        if self.h:
            self.L.or_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload_geometry(self, g):
        s, keep = abi.geometry_struct(g)
        self._keep.append(keep)
        self._check(self.L.or_upload_geometry(self.h, C.byref(s)))

    def upload_mg(self, m):
        s, keep = abi.mg_struct(m)
        self._keep.append(keep)
        self._check(self.L.or_upload_mg(self.h, C.byref(s)))

    def upload_ce(self, d):
        s, keep = abi.ce_struct(d)
        self._keep.append(keep)
        self._check(self.L.or_upload_ce(self.h, C.byref(s)))

    def ce_micro(self, nuc, E):
        out = np.zeros(4)
        self._check(self.L.or_ce_micro(self.h, nuc, E, out.ctypes.data_as(C.POINTER(C.c_double))))
        return out

    def ce_mat_total(self, mat, E):
        v = C.c_double()
        self._check(self.L.or_ce_mat_total(self.h, mat, E, C.byref(v)))
        return v.value

    def ce_majorant(self, E):
        v = C.c_double()
        self._check(self.L.or_ce_majorant(self.h, E, C.byref(v)))
        return v.value

    def ce_union_size(self):
        n = C.c_int64()
        self._check(self.L.or_ce_union_size(self.h, C.byref(n)))
        return n.value

    def set_collision(self, desc):
        """neutronMGimp / neutronCEimp options (an abi.collision() description)."""
        self._keep.append(desc)
        self._check(self.L.or_set_collision(self.h, C.byref(desc)))

    def map_point(self, axes, r=(0.0, 0.0, 0.0), G=1, mat=1, cell=0, E=0.0, mg=True):
        """Bin (1-based, 0 outside) of one particle state in the multiMap of `axes` (as for abi.clerk)."""
        c = abi.clerk(abi.CLERK_COLLISION, axes=axes)
        _, pr = _d(r)
        b = C.c_int32()
        self._check(self.L.or_map_point(self.h, c.axes, c.n_axes, pr, G, mat, cell, float(E), 1 if mg else 0,
                                        C.byref(b)))
        return b.value

    def grid_search(self, bounds, v):
        """grid%search of an unstructured grid: 1-based bin of `v`, 0 outside."""
        b, pb = _d(bounds)
        return self.L.or_grid_search(pb, len(b), float(v))

    def upload_tally(self, clerks, batch_size=1, norm_clerk=-1, norm_val=1.0):
        t, arr = abi.tally_struct(clerks, batch_size, norm_clerk, norm_val)
        self._keep.append(arr)
        a = C.c_int32()
        self._check(self.L.or_upload_tally(self.h, C.byref(t), C.byref(a)))
        return a.value

    def attach_tally(self, admin, atch):
        self._check(self.L.or_attach_tally(self.h, admin, atch))

    def set_point_source(self, r, G=1, dir=(1.0, 0.0, 0.0), isotropic=True, prob_g=None, E=0.0):
        s, keep = abi.point_source_struct(r, G, dir, isotropic, prob_g, E)
        self._keep.append((s, keep))
        self._check(self.L.or_set_point_source(self.h, C.byref(s)))

    def generate_source(self, master, n):
        b = abi.HostBank(n)
        self._check(self.L.or_generate_source(self.h, C.c_uint64(master), n, C.byref(b.struct)))
        return b

    def transport_bank(self, admin, bank, master, k_eff=1.0, next_cap=None):
        n = bank.n
        cap = next_cap if next_cap is not None else max(4 * n, 16)
        nxt = abi.HostBank(cap)
        st = abi.CycleStats()
        self._check(self.L.or_transport_bank(self.h, admin, C.byref(bank.struct), n, C.c_uint64(master),
                                             k_eff, C.byref(nxt.struct), cap, C.byref(st)))
        return nxt, st

    def tally_cycle_start(self, admin, w):
        self._check(self.L.or_tally_cycle_start(self.h, admin, w))

    def tally_cycle_end(self, admin, w, k=1.0):
        self._check(self.L.or_tally_cycle_end(self.h, admin, w, k))

    def bins(self, admin):
        n = C.c_int64()
        self._check(self.L.or_tally_size(self.h, admin, C.byref(n)))
        out = np.zeros(3 * n.value)
        self._check(self.L.or_get_bins(self.h, admin, out.ctypes.data_as(C.POINTER(C.c_double)), n.value))
        return out.reshape(3, n.value).T.copy()

    def normalise_shard(self, sites, n, before, tot_sites, tot_pop, master, cap):
        """This process's part of normSize_Repr over a population split over processes
        (or_normalise_shard): returns (bank, n_out)."""
        out = abi.HostBank(max(cap, 1))
        m = C.c_int32()
        self._check(self.L.or_normalise_shard(self.h, C.byref(sites.struct), n, before, tot_sites, tot_pop,
                                                C.c_uint64(master), C.byref(out.struct), cap, C.byref(m)))
        return out, m.value

    def normalise(self, sites, n, tot_pop, master, cap):
        """normSize_Repr of a single-process run (the sites sorted by brood): (bank, n_out)."""
        out = abi.HostBank(max(cap, 1))
        m = C.c_int32()
        self._check(self.L.or_normalise(self.h, C.byref(sites.struct), n, tot_pop, C.c_uint64(master),
                                        C.byref(out.struct), cap, C.byref(m)))
        return out, m.value

    def _tally_n(self, admin):
        n = C.c_int64()
        self._check(self.L.or_tally_size(self.h, admin, C.byref(n)))
        return n.value

    def get_scores(self, admin):
        """The running-batch scores of an admin (summed over processes for a synchronised tally)."""
        out = np.zeros(max(self._tally_n(admin), 1))
        self._check(self.L.or_tally_get_scores(self.h, admin, out.ctypes.data_as(C.POINTER(C.c_double)), out.size))
        return out[:self._tally_n(admin)].copy()

    def set_scores(self, admin, scores):
        s = np.ascontiguousarray(scores, dtype=np.float64)
        if s.size < self._tally_n(admin):
            raise ValueError("set_scores: fewer values than the tally has bins")
        self._check(self.L.or_tally_set_scores(self.h, admin, s.ctypes.data_as(C.POINTER(C.c_double)), s.size))

    def keff(self, admin):
        k, s = C.c_double(), C.c_double()
        self._check(self.L.or_get_keff(self.h, admin, C.byref(k), C.byref(s)))
        return k.value, s.value

    def history_records(self, n):
        c = np.zeros(n, np.int32)
        r = np.zeros(n, np.uint64)
        self._check(self.L.or_get_history_records(self.h, c.ctypes.data_as(C.POINTER(C.c_int32)),
                                                  r.ctypes.data_as(C.POINTER(C.c_uint64)), n))
        return c, r

    def eigen_init(self, pop, master, k0=1.0):
        self._check(self.L.or_eigen_init(self.h, pop, C.c_uint64(master), k0))

    def eigen_cycle(self, admin, atch):
        st = abi.CycleStats()
        self._check(self.L.or_eigen_cycle(self.h, admin, atch, C.byref(st)))
        return st

    def eigen_cycle_omp(self, admin, atch, threads=0):
        """The same cycle with OpenMP over histories (SCONE's OpenMP build): the CPU baseline."""
        st = abi.CycleStats()
        self._check(self.L.or_eigen_cycle_omp(self.h, admin, atch, threads, C.byref(st)))
        return st

    def eigen_state(self):
        m, k = C.c_uint64(), C.c_double()
        self._check(self.L.or_eigen_state(self.h, C.byref(m), C.byref(k)))
        return m.value, k.value

    def eigen_bank(self, cap):
        b = abi.HostBank(cap)
        pop = C.c_int32()
        self._check(self.L.or_eigen_get_bank(self.h, C.byref(b.struct), cap, C.byref(pop)))
        return b, pop.value

    def set_file_source(self, bank):
        self._keep.append(bank)
        self._check(self.L.or_set_file_source(self.h, C.byref(bank.struct), bank.n))

    def fixed_source_cycle(self, admin, n, master, total=None):
        """One fixed-source cycle of n histories; with `total`, n is this process's share of a
        population of `total` split over processes (master already strided by the offset)."""
        m = C.c_uint64(master)
        st = abi.CycleStats()
        if total is None:
            self._check(self.L.or_fixed_source_cycle(self.h, admin, n, C.byref(m), C.byref(st)))
        else:
            self._check(self.L.or_fixed_source_cycle_shard(self.h, admin, n, total, C.byref(m), C.byref(st)))
        return m.value, st

    # geometry probes
    def coords_init(self, r, u):
        _, pr = _d(r)
        _, pu = _d(u)
        self.L.or_coords_init(self.h, pr, pu)

    def coords_place(self):
        self.L.or_coords_place(self.h)

    def coords_move(self, mode, max_dist):
        d = C.c_double(max_dist)
        ev = C.c_int32()
        self.L.or_coords_move(self.h, mode, C.byref(d), C.byref(ev))
        return d.value, ev.value

    def coords_get(self, level=0):
        r = np.zeros(3)
        u = np.zeros(3)
        info = np.zeros(5, np.int32)
        self.L.or_coords_get(self.h, level, r.ctypes.data_as(C.POINTER(C.c_double)),
                             u.ctypes.data_as(C.POINTER(C.c_double)), info.ctypes.data_as(C.POINTER(C.c_int32)))
        return r, u, dict(nesting=int(info[0]), mat=int(info[1]), uid=int(info[2]), local=int(info[3]), uni=int(info[4]))

    def what_is_at(self, r, u=(1.0, 0.0, 0.0)):
        _, pr = _d(r)
        _, pu = _d(u)
        m, i = C.c_int32(), C.c_int32()
        self.L.or_what_is_at(self.h, pr, pu, C.byref(m), C.byref(i))
        return m.value, i.value

    def bounds(self):
        b = np.zeros(6)
        self.L.or_bounds(self.h, b.ctypes.data_as(C.POINTER(C.c_double)))
        return b

    def mg_info(self, mat, G):
        o = np.zeros(6)
        self.L.or_mg_info(self.h, mat, G, o.ctypes.data_as(C.POINTER(C.c_double)))
        return dict(total=o[0], scatter=o[1], capture=o[2], fission=o[3], nu_fission=o[4], majorant=o[5])

    def timed_gen_loop(self, admin, bank, master, k_eff=1.0, threads=0):
        ev = C.c_int64()
        n = self.L.or_timed_gen_loop(self.h, admin, C.byref(bank.struct), bank.n, C.c_uint64(master), k_eff,
                                     threads, C.byref(ev))
        return n, ev.value


def sample_legendre_p1(a, state, n):
    """n samples of SCONE's sampleLegendre_P1 for a = 3 P1/P0 from RNG `state`."""
    s = C.c_uint64(state)
    out = np.zeros(n)
    rc = lib().or_sample_legendre_p1(a, C.byref(s), out.ctypes.data_as(C.POINTER(C.c_double)), n)
    if rc != 0:
        raise RuntimeError(f"oracle error {rc}")
    return out, s.value


def rng_draws(state, n):
    s = C.c_uint64(state)
    out = np.zeros(n)
    lib().or_rng_draws(C.byref(s), out.ctypes.data_as(C.POINTER(C.c_double)), n)
    return out, s.value


def rng_skip(state, k):
    return lib().or_rng_skip(C.c_uint64(state), C.c_int64(k))


def surf_eval(type_, par, r, u, bc=None):
    p = np.zeros(abi.SG_SURF_NPAR)
    p[:len(par)] = par
    _, pp = _d(p)
    _, pr = _d(r)
    _, pu = _d(u)
    out = np.zeros(5)
    bcp = None
    if bc is not None:
        b = np.ascontiguousarray(bc, np.int32)
        bcp = b.ctypes.data_as(C.POINTER(C.c_int32))
    lib().or_surf_eval(type_, pp, bcp, pr, pu, out.ctypes.data_as(C.POINTER(C.c_double)))
    return dict(evaluate=out[0], distance=out[1], halfspace=bool(out[2]), going=bool(out[3]), tol=out[4])


def surf_bc(type_, par, bc, r, u, transform=False):
    p = np.zeros(abi.SG_SURF_NPAR)
    p[:len(par)] = par
    _, pp = _d(p)
    r = np.array(r, dtype=np.float64)
    u = np.array(u, dtype=np.float64)
    b = np.ascontiguousarray(bc, np.int32)
    lib().or_surf_bc(type_, pp, b.ctypes.data_as(C.POINTER(C.c_int32)), 1 if transform else 0,
                     r.ctypes.data_as(C.POINTER(C.c_double)), u.ctypes.data_as(C.POINTER(C.c_double)))
    return r, u


def rotate_vector(d, mu, phi):
    _, pd = _d(d)
    out = np.zeros(3)
    lib().or_rotate_vector(pd, mu, phi, out.ctypes.data_as(C.POINTER(C.c_double)))
    return out


class ScoreMemory:
    def __init__(self, n, batch=1):
        self.L = lib()
        self.h = C.c_void_p()
        self.L.or_scoremem_new(n, batch, C.byref(self.h))

    def score(self, s, idx):
        self.L.or_scoremem_score(self.h, s, idx)

    def accumulate(self, s, idx):
        self.L.or_scoremem_accumulate(self.h, s, idx)

    def close_cycle(self, f=1.0):
        self.L.or_scoremem_close(self.h, f)

    def reduce_bins(self):
        self.L.or_scoremem_reduce(self.h)

    def close_bin(self, f, idx):
        self.L.or_scoremem_closebin(self.h, f, idx)

    def close_cycle_only(self, f):
        self.L.or_scoremem_closecycle(self.h, f)

    def result(self, idx, samples=-1):
        m, s = C.c_double(), C.c_double()
        self.L.or_scoremem_result(self.h, idx, samples, C.byref(m), C.byref(s))
        return m.value, s.value

    def __del__(self):
        try:
            self.L.or_scoremem_free(self.h)
        except Exception:
            pass


def asymptotic_scatter(E, mu, A):
    out = np.zeros(2)
    lib().or_asymptotic_scatter(E, mu, A, out.ctypes.data_as(C.POINTER(C.c_double)))
    return out[0], out[1]


def target_velocity(E, d, A, kT, state):
    d, dp = _d(d)
    s = C.c_uint64(state)
    v = np.zeros(3)
    lib().or_target_velocity(E, dp, A, kT, C.byref(s), v.ctypes.data_as(C.POINTER(C.c_double)))
    return v, s.value
