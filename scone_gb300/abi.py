"""ctypes mirrors of the C ABI structs declared in include/scone_gpu.h.

The same structs describe a problem to the CUDA library (libsconegpu) and, in the tests, to the
CPU oracle.  Helper builders keep the numpy arrays they point to alive for as long as the struct.
"""
import ctypes as C
import numpy as np

SG_OK = 0
SG_SURF_NPAR = 6
SG_VOID_MAT = 2147483647

# surface types
XPLANE, YPLANE, ZPLANE, PLANE = 1, 2, 3, 4
XCYL, YCYL, ZCYL, SPHERE, BOX = 5, 6, 7, 8, 9
XSQCYL, YSQCYL, ZSQCYL = 10, 11, 12
# universe types
UNI_ROOT, UNI_CELL, UNI_PIN, UNI_LAT = 1, 2, 3, 4
# boundary conditions
BC_VACUUM, BC_REFLECTIVE, BC_PERIODIC = 0, 1, 2
# unionCell operators in a cell's surface list: '<', '>', ':' (union), '#' (complement)
CELL_OPEN, CELL_CLOSE, CELL_UNION, CELL_COMPLEMENT = -2147483647, -2147483646, -2147483645, -2147483644
# precision forms
PREC_FP64, PREC_MIXED = 0, 1
# execution forms
FORM_EVENT, FORM_HISTORY = 0, 1
# transport operators
TRANSPORT_ST, TRANSPORT_DT, TRANSPORT_ST_NOCACHE, TRANSPORT_HT, TRANSPORT_HT_NOCACHE = 1, 2, 3, 4, 5
# clerks
CLERK_COLLISION, CLERK_TRACK, CLERK_KEFF_ANALOG, CLERK_KEFF_IMPLICIT = 1, 2, 3, 4
CLERK_SURFACE_CURRENT = 5
# map axes
AXIS_X, AXIS_Y, AXIS_Z, AXIS_GROUP, AXIS_MATERIAL, AXIS_ENERGY, AXIS_CELL = 1, 2, 3, 4, 5, 6, 7
# grids of space and energy axes (grid_class.f90): default = lin for space, log for energy
GRID_DEFAULT, GRID_LIN, GRID_LOG, GRID_UNSTRUCT = 0, 1, 2, 3
# responses (macro MTs from SharedModules/endfConstants.f90:116-130)
RESP_FLUX = 0
MACRO_TOTAL, MACRO_CAPTURE, MACRO_FISSION, MACRO_NUFISSION, MACRO_ABSORPTION = -1, -2, -6, -7, -21

i32p = C.POINTER(C.c_int32)
f64p = C.POINTER(C.c_double)


class GeometryDesc(C.Structure):
    _fields_ = [
        ("n_surf", C.c_int32), ("surf_type", i32p), ("surf_par", f64p),
        ("border_surf", C.c_int32), ("bc", C.c_int32 * 6),
        ("n_cell", C.c_int32), ("cell_ptr", i32p), ("cell_surf", i32p),
        ("n_uni", C.c_int32), ("uni_type", i32p), ("uni_origin", f64p),
        ("uni_iptr", i32p), ("uni_ipar", i32p), ("uni_dptr", i32p), ("uni_dpar", f64p),
        ("uni_fptr", i32p), ("uni_fill", i32p), ("root_uni", C.c_int32), ("uni_rot", f64p),
    ]


class MGDesc(C.Structure):
    _fields_ = [
        ("n_mat", C.c_int32), ("n_g", C.c_int32),
        ("capture", f64p), ("fission", f64p), ("nu", f64p), ("chi", f64p),
        ("p0", f64p), ("prod", f64p), ("fissile", i32p), ("avg_dist", C.c_double), ("p1", f64p),
    ]


class AxisDesc(C.Structure):
    _fields_ = [("kind", C.c_int32), ("n", C.c_int32), ("min", C.c_double), ("max", C.c_double),
                ("grid", C.c_int32), ("cell_rest", C.c_int32), ("bounds", f64p), ("cells", i32p)]


class ClerkDesc(C.Structure):
    _fields_ = [
        ("type", C.c_int32), ("handle_virtual", C.c_int32), ("n_resp", C.c_int32),
        ("resp", C.c_int32 * 4), ("n_axes", C.c_int32), ("axes", AxisDesc * 3),
        ("filter_g_top", C.c_int32), ("filter_g_low", C.c_int32),
        ("current_axis", C.c_int32), ("n_planes", C.c_int32), ("planes", C.c_double * 8),
    ]


class TallyDesc(C.Structure):
    _fields_ = [
        ("n_clerks", C.c_int32), ("clerks", C.POINTER(ClerkDesc)), ("batch_size", C.c_int32),
        ("norm_clerk", C.c_int32), ("norm_val", C.c_double),
    ]


class PointSourceDesc(C.Structure):
    _fields_ = [
        ("r", C.c_double * 3), ("dir", C.c_double * 3), ("isotropic", C.c_int32),
        ("G", C.c_int32), ("n_prob_g", C.c_int32), ("prob_g", f64p), ("E", C.c_double),
    ]


class Config(C.Structure):
    _fields_ = [
        ("precision", C.c_int32), ("transport", C.c_int32), ("device", C.c_int32),
        ("max_bank", C.c_int32), ("record_histories", C.c_int32), ("form", C.c_int32),
        ("ht_cutoff", C.c_double),
    ]


class Bank(C.Structure):
    _fields_ = [
        ("wgt", f64p), ("r", f64p), ("dir", f64p), ("G", i32p), ("time", f64p), ("brood_id", i32p),
        ("E", f64p),
    ]


class CEDesc(C.Structure):
    _fields_ = [
        ("n_nuc", C.c_int32), ("nuc_ptr", C.POINTER(C.c_int64)), ("e", f64p), ("xs", f64p),
        ("A", f64p), ("kT", f64p), ("n_mat", C.c_int32), ("mat_ptr", i32p), ("mat_nuc", i32p),
        ("mat_dens", f64p), ("majorant", C.c_int32), ("min_e", C.c_double), ("max_e", C.c_double),
        ("thresh_e", C.c_double), ("thresh_a", C.c_double), ("avg_dist", C.c_double),
    ]


class CycleStats(C.Structure):
    _fields_ = [
        ("n_histories", C.c_int64), ("n_events", C.c_int64), ("n_collisions", C.c_int64),
        ("n_next", C.c_int64), ("start_weight", C.c_double), ("end_weight", C.c_double),
        ("k_eff", C.c_double), ("k_new", C.c_double), ("transport_ms", C.c_double),
        ("cycle_ms", C.c_double), ("n_kernels", C.c_int64),
    ]


class BatchConfig(C.Structure):
    _fields_ = [
        ("precision", C.c_int32), ("transport", C.c_int32), ("device", C.c_int32),
        ("max_problems", C.c_int32), ("arena_bytes", C.c_int64), ("max_work_items", C.c_int32),
        ("reserved", C.c_int32), ("ht_cutoff", C.c_double),
    ]


class ProblemDesc(C.Structure):
    _fields_ = [
        ("geometry", C.POINTER(GeometryDesc)), ("mg", C.POINTER(MGDesc)),
        ("source", C.POINTER(PointSourceDesc)), ("tally", C.POINTER(TallyDesc)),
        ("pop", C.c_int32), ("cycles", C.c_int32), ("master_state", C.c_uint64),
    ]


class BatchTuning(C.Structure):
    _fields_ = [
        ("item_histories", C.c_int32), ("blocks_per_sm", C.c_int32), ("block_threads", C.c_int32),
        ("order", C.c_int32),
    ]

    def as_dict(self):
        return {k: int(getattr(self, k)) for k, _ in self._fields_}


class EventTuning(C.Structure):
    _fields_ = [("rounds_per_check", C.c_int32), ("tail_min", C.c_int32), ("tail_divisor", C.c_int32)]

    def as_dict(self):
        return {k: int(getattr(self, k)) for k, _ in self._fields_}


class BatchStats(C.Structure):
    _fields_ = [
        ("n_histories", C.c_int64), ("n_events", C.c_int64), ("n_collisions", C.c_int64),
        ("n_problems", C.c_int32), ("n_items", C.c_int32), ("kernel_ms", C.c_double),
        ("run_ms", C.c_double), ("n_kernels", C.c_int64),
    ]


def _p(a, ct):
    return a.ctypes.data_as(C.POINTER(ct))


class HostBank:
    """SoA particle bank in (optionally pinned) host numpy arrays, viewable as an sg_bank."""

    def __init__(self, n, arrays=None):
        self.n = int(n)
        if arrays is None:
            arrays = dict(
                wgt=np.ones(n, np.float64), r=np.zeros((n, 3), np.float64),
                dir=np.zeros((n, 3), np.float64), G=np.ones(n, np.int32),
                time=np.zeros(n, np.float64), brood_id=np.zeros(n, np.int32),
                E=np.zeros(n, np.float64))
        self.a = arrays
        if "E" not in self.a:
            self.a["E"] = np.zeros(self.n, np.float64)
        for k in ("wgt", "r", "dir", "time", "E"):
            self.a[k] = np.ascontiguousarray(self.a[k], dtype=np.float64)
        for k in ("G", "brood_id"):
            self.a[k] = np.ascontiguousarray(self.a[k], dtype=np.int32)
        self.struct = Bank(_p(self.a["wgt"], C.c_double), _p(self.a["r"], C.c_double),
                           _p(self.a["dir"], C.c_double), _p(self.a["G"], C.c_int32),
                           _p(self.a["time"], C.c_double), _p(self.a["brood_id"], C.c_int32),
                           _p(self.a["E"], C.c_double))

    def __getitem__(self, k):
        return self.a[k]

    def head(self, m):
        return {k: v[:m].copy() for k, v in self.a.items()}


def geometry_struct(g):
    """Build a GeometryDesc from a dict of numpy arrays (see problems.Geometry)."""
    keep = {}

    def arr(name, dt):
        a = np.ascontiguousarray(g[name], dtype=dt)
        if a.size == 0:
            a = np.zeros(1, dtype=dt)
        keep[name] = a
        return _p(a, C.c_int32 if dt == np.int32 else C.c_double)

    s = GeometryDesc()
    s.n_surf = len(g["surf_type"])
    s.surf_type = arr("surf_type", np.int32)
    s.surf_par = arr("surf_par", np.float64)
    s.border_surf = int(g["border_surf"])
    for i in range(6):
        s.bc[i] = int(g["bc"][i])
    s.n_cell = len(g["cell_ptr"]) - 1
    s.cell_ptr = arr("cell_ptr", np.int32)
    s.cell_surf = arr("cell_surf", np.int32)
    s.n_uni = len(g["uni_type"])
    s.uni_type = arr("uni_type", np.int32)
    s.uni_origin = arr("uni_origin", np.float64)
    s.uni_iptr = arr("uni_iptr", np.int32)
    s.uni_ipar = arr("uni_ipar", np.int32)
    s.uni_dptr = arr("uni_dptr", np.int32)
    s.uni_dpar = arr("uni_dpar", np.float64)
    s.uni_fptr = arr("uni_fptr", np.int32)
    s.uni_fill = arr("uni_fill", np.int32)
    s.root_uni = int(g["root_uni"])
    if g.get("uni_rot") is not None:
        s.uni_rot = arr("uni_rot", np.float64)
    return s, keep


def mg_struct(m):
    keep = {}

    def arr(name, dt):
        a = np.ascontiguousarray(m[name], dtype=dt)
        keep[name] = a
        return _p(a, C.c_int32 if dt == np.int32 else C.c_double)

    s = MGDesc()
    s.n_mat, s.n_g = int(m["n_mat"]), int(m["n_g"])
    s.capture = arr("capture", np.float64)
    s.fission = arr("fission", np.float64)
    s.nu = arr("nu", np.float64)
    s.chi = arr("chi", np.float64)
    s.p0 = arr("p0", np.float64)
    s.prod = arr("prod", np.float64)
    s.fissile = arr("fissile", np.int32)
    s.avg_dist = float(m.get("avg_dist", 0.0))
    s.p1 = arr("p1", np.float64) if m.get("p1") is not None else C.cast(None, f64p)
    return s, keep


COLL_STD, COLL_IMP = 0, 1


class CollisionDesc(C.Structure):
    _fields_ = [
        ("kind", C.c_int32), ("imp_abs", C.c_int32), ("roulette", C.c_int32), ("split", C.c_int32),
        ("weight_windows", C.c_int32), ("max_split", C.c_int32),
        ("min_wgt", C.c_double), ("max_wgt", C.c_double), ("av_wgt", C.c_double),
        ("ww_n_axes", C.c_int32), ("ww_axes", AxisDesc * 3), ("ww_lower", f64p), ("ww_upper", f64p),
        ("ww_const_survival", C.c_double), ("buffer_depth", C.c_int32),
    ]


def collision(kind=COLL_IMP, imp_abs=False, roulette=False, split=False, max_split=1000, min_wgt=0.25,
              max_wgt=1.25, av_wgt=0.5, ww_axes=None, ww_lower=None, ww_upper=None, ww_const_survival=0.0,
              buffer_depth=0):
    """Describe a collision processor: neutronMGstd/CEstd (COLL_STD) or neutronMGimp/CEimp (COLL_IMP)
    with its options and defaults; weight windows when ww_axes is given (a map as for clerk())."""
    d = CollisionDesc()
    d.kind, d.imp_abs, d.roulette, d.split = kind, int(imp_abs), int(roulette), int(split)
    d.max_split, d.min_wgt, d.max_wgt, d.av_wgt = max_split, min_wgt, max_wgt, av_wgt
    d.buffer_depth = buffer_depth
    keep = []
    if ww_axes is not None:
        m = clerk(CLERK_COLLISION, axes=ww_axes)
        keep.append(m)
        d.weight_windows = 1
        d.ww_n_axes = m.n_axes
        for i in range(m.n_axes):
            d.ww_axes[i] = m.axes[i]
        lo = np.ascontiguousarray(ww_lower, dtype=np.float64)
        up = np.ascontiguousarray(ww_upper, dtype=np.float64)
        keep += [lo, up]
        d.ww_lower = lo.ctypes.data_as(f64p)
        d.ww_upper = up.ctypes.data_as(f64p)
        d.ww_const_survival = ww_const_survival
    d._keep = keep
    return d


def unstruct_axis(kind, bounds):
    """A spaceMap / energyMap axis on an unstructured grid of ascending bounds (grid 'unstruct')."""
    b = np.ascontiguousarray(bounds, dtype=np.float64)
    return {"kind": kind, "n": len(b) - 1, "grid": GRID_UNSTRUCT, "bounds": b}


def cell_axis(cells, undef_bin=False):
    """A cellMap axis over 0-based cell indices of the geometry; `undef_bin` adds the rest bin."""
    c = np.ascontiguousarray(cells, dtype=np.int32)
    return {"kind": AXIS_CELL, "n": len(c), "cells": c, "cell_rest": 1 if undef_bin else 0}


def axis_bins(ax):
    """Bins of one axis given to clerk()."""
    if isinstance(ax, dict):
        return ax["n"] + (1 if ax.get("cell_rest") else 0)
    return ax[1]


def clerk(type_, resp=(RESP_FLUX,), axes=(), handle_virtual=1, g_filter=None, current_axis=0, planes=()):
    """Describe one tally clerk; axes in multiMap order, each (kind, n, min, max[, grid]) or a dict
    from unstruct_axis() / cell_axis().

    Surface-current clerks take the normal axis (AXIS_X/Y/Z) and up to 8 plane positions."""
    c = ClerkDesc()
    c.type = type_
    c.handle_virtual = handle_virtual
    c.n_resp = len(resp)
    for i, r in enumerate(resp):
        c.resp[i] = r
    c.n_axes = len(axes)
    keep = []
    for i, ax in enumerate(axes):
        d = c.axes[i]
        if isinstance(ax, dict):
            d.kind, d.n = ax["kind"], ax["n"]
            d.min, d.max = ax.get("min", 0.0), ax.get("max", 0.0)
            d.grid, d.cell_rest = ax.get("grid", GRID_DEFAULT), ax.get("cell_rest", 0)
            if ax.get("bounds") is not None:
                keep.append(ax["bounds"])
                d.bounds = ax["bounds"].ctypes.data_as(f64p)
            if ax.get("cells") is not None:
                keep.append(ax["cells"])
                d.cells = ax["cells"].ctypes.data_as(i32p)
        else:
            d.kind, d.n, d.min, d.max = ax[:4]
            d.grid = ax[4] if len(ax) > 4 else GRID_DEFAULT
    c._keep = keep
    if g_filter is not None:
        c.filter_g_top, c.filter_g_low = g_filter
    c.current_axis = current_axis
    c.n_planes = len(planes)
    for i, x in enumerate(planes):
        c.planes[i] = x
    return c


def tally_struct(clerks, batch_size=1, norm_clerk=-1, norm_val=1.0):
    arr = (ClerkDesc * max(1, len(clerks)))(*clerks)
    t = TallyDesc(len(clerks), C.cast(arr, C.POINTER(ClerkDesc)), batch_size, norm_clerk, norm_val)
    return t, arr


def point_source_struct(r, G=1, dir=(1.0, 0.0, 0.0), isotropic=True, prob_g=None, E=0.0):
    s = PointSourceDesc()
    s.E = E
    for i in range(3):
        s.r[i] = r[i]
        s.dir[i] = dir[i]
    s.isotropic = 1 if isotropic else 0
    s.G = G
    keep = None
    if prob_g is not None:
        keep = np.ascontiguousarray(prob_g, dtype=np.float64)
        s.n_prob_g = len(keep)
        s.prob_g = _p(keep, C.c_double)
    else:
        s.n_prob_g = 0
        s.prob_g = C.cast(None, f64p)
    return s, keep


def ce_struct(d):
    """Build a CEDesc from a dict (see problems.ce_data)."""
    keep = {}

    def arr(name, dt, ct):
        a = np.ascontiguousarray(d[name], dtype=dt)
        keep[name] = a
        return _p(a, ct)

    s = CEDesc()
    s.n_nuc = len(d["A"])
    s.nuc_ptr = arr("nuc_ptr", np.int64, C.c_int64)
    s.e = arr("e", np.float64, C.c_double)
    s.xs = arr("xs", np.float64, C.c_double)
    s.A = arr("A", np.float64, C.c_double)
    s.kT = arr("kT", np.float64, C.c_double)
    s.n_mat = len(d["mat_ptr"]) - 1
    s.mat_ptr = arr("mat_ptr", np.int32, C.c_int32)
    s.mat_nuc = arr("mat_nuc", np.int32, C.c_int32)
    s.mat_dens = arr("mat_dens", np.float64, C.c_double)
    s.majorant = int(d.get("majorant", 1))
    s.min_e = float(d.get("min_e", 1.0e-11))
    s.max_e = float(d.get("max_e", 20.0))
    s.thresh_e = float(d.get("thresh_e", 400.0))
    s.thresh_a = float(d.get("thresh_a", 1.0))
    s.avg_dist = float(d.get("avg_dist", 0.0))
    return s, keep
