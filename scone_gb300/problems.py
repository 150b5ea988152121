"""Problem descriptions for libsconegpu: a CSG geometry builder, MG data, tallies and the seeded
synthetic generators for the benchmark workloads.

The generators stand in for SCONE input decks (SCONE's own dictionary parser is not part of the
transport hot path); they produce the same geometry tables that SCONE's `geometryStd%init`
(Geometry/csg_class.f90:50-207) and MG `baseMgNeutronDatabase%init`
(NuclearData/mgNeutronData/baseMgNeutron/baseMgNeutronDatabase_class.f90:340-410) build.

Workloads (all synthetic, seeded with numpy default_rng):
  * ``infinite_medium_2g``  -- 2-group infinite homogeneous medium, point source (fixed source).
  * ``lattice_17x17_7g``    -- 17x17 pin lattice, 7 groups, k-eigenvalue.
"""
import numpy as np

from . import abi

VOID = abi.SG_VOID_MAT


def uni_fill(u):
    """Fill code of a nested universe (0-based index u): -uniIdx with uniIdx 1-based."""
    return -(u + 1)


class GeometryBuilder:
    def __init__(self):
        self.surf_type, self.surf_par = [], []
        self.cells = []
        self.unis = []          # (type, origin, ipar, dpar, fills)
        self.root = None
        self.border = None
        self.bc = [0] * 6

    def surface(self, type_, *par):
        p = list(par) + [0.0] * (abi.SG_SURF_NPAR - len(par))
        self.surf_type.append(type_)
        self.surf_par.append(p)
        return len(self.surf_type) - 1

    def cell(self, signed_surfs):
        """signed 1-based surface indices: -(s+1) for the -ve halfspace of surface s (0-based)."""
        self.cells.append(list(signed_surfs))
        return len(self.cells) - 1

    def universe(self, type_, fills, ipar=(), dpar=(), origin=(0.0, 0.0, 0.0)):
        self.unis.append((type_, list(origin), list(ipar), list(dpar), list(fills)))
        return len(self.unis) - 1

    def root_universe(self, border_surf, fill, bc=(0, 0, 0, 0, 0, 0)):
        self.border = border_surf
        self.bc = list(bc)
        self.root = self.universe(abi.UNI_ROOT, [fill], ipar=[border_surf])
        return self.root

    def pin_universe(self, radii, fills, origin=(0.0, 0.0, 0.0)):
        return self.universe(abi.UNI_PIN, fills, dpar=sorted(radii), origin=origin)

    def lattice_universe(self, shape, pitch, fills_local_order, pad_fill, offset=True):
        return self.universe(abi.UNI_LAT, list(fills_local_order) + [pad_fill],
                             ipar=list(shape) + [1 if offset else 0], dpar=list(pitch))

    def cell_universe(self, cell_idx, fills):
        return self.universe(abi.UNI_CELL, fills, ipar=cell_idx)

    def arrays(self):
        def ptr(lists):
            p = np.zeros(len(lists) + 1, np.int32)
            for i, l in enumerate(lists):
                p[i + 1] = p[i] + len(l)
            return p

        def cat(lists, dt):
            flat = [x for l in lists for x in l]
            return np.array(flat, dtype=dt)

        return dict(
            surf_type=np.array(self.surf_type, np.int32),
            surf_par=np.array(self.surf_par, np.float64).reshape(-1, abi.SG_SURF_NPAR),
            border_surf=self.border, bc=list(self.bc),
            cell_ptr=ptr(self.cells), cell_surf=cat(self.cells, np.int32),
            uni_type=np.array([u[0] for u in self.unis], np.int32),
            uni_origin=np.array([u[1] for u in self.unis], np.float64).reshape(-1, 3),
            uni_iptr=ptr([u[2] for u in self.unis]), uni_ipar=cat([u[2] for u in self.unis], np.int32),
            uni_dptr=ptr([u[3] for u in self.unis]), uni_dpar=cat([u[3] for u in self.unis], np.float64),
            uni_fptr=ptr([u[4] for u in self.unis]), uni_fill=cat([u[4] for u in self.unis], np.int32),
            root_uni=self.root,
        )


def lattice_fills_from_map(map_values, shape):
    """latUniverse input `map` (WYSIWYG: top row first) -> fills in local-ID order.

    Restates the flip of latUniverse%init (Geometry/Universes/latUniverse_class.f90:199-226).
    """
    nx, ny, nz = shape
    nz = max(nz, 1)
    m = np.asarray(map_values).reshape(ny * nz, nx)     # rows of the input, top first
    m = m[::-1]                                          # flip Y (and Z) rows
    return list(m.reshape(-1))


# ----------------------------------------------------------------------------- MG data
def mg_data(n_g, total, scatter_matrix, capture=None, fission=None, nu=None, chi=None,
            prod=None, avg_dist=0.0):
    """Assemble an MG desc dict; scatter_matrix[m][g_in][g_out] (xsFile `P0` layout)."""
    total = np.asarray(total, np.float64)
    n_mat = total.shape[0]
    P0 = np.asarray(scatter_matrix, np.float64).reshape(n_mat, n_g, n_g)
    if capture is None:
        capture = total - P0.sum(axis=2)
    fissile = np.zeros(n_mat, np.int32)
    fis = np.zeros((n_mat, n_g)) if fission is None else np.asarray(fission, np.float64)
    if fission is not None:
        fissile = (fis.sum(axis=1) > 0).astype(np.int32)
    return dict(
        n_mat=n_mat, n_g=n_g, capture=np.asarray(capture, np.float64), fission=fis,
        nu=np.zeros((n_mat, n_g)) if nu is None else np.asarray(nu, np.float64),
        chi=np.zeros((n_mat, n_g)) if chi is None else np.asarray(chi, np.float64),
        p0=P0, prod=np.ones_like(P0) if prod is None else np.asarray(prod, np.float64),
        fissile=fissile, avg_dist=avg_dist)


class Problem:
    """Geometry + data + tallies + source of one transport problem."""

    def __init__(self, geometry, mg, name="", source=None, tallies=None, eigen=False, meta=None):
        self.geometry = geometry
        self.mg = mg
        self.name = name
        self.source = source or {}
        self.tallies = tallies or {}
        self.eigen = eigen
        self.meta = meta or {}


# ----------------------------------------------------------------------------- workloads
def infinite_medium_2g(seed=7, half_width=10.0):
    """Fixed-source transport in an infinite homogeneous medium, 2 groups.

    Sigma_t ~ U[0.5, 2.0] /cm per group, scattering ratio 0.9 with a lower-triangular (downscatter)
    2x2 P0, capture = 0.1 Sigma_t, no fission; an all-reflective box makes the medium infinite
    (as SCONE's InputFiles/SCONE_Inf deck does).  Isotropic point source at the origin, group 1.
    """
    rng = np.random.default_rng(seed)
    sig_t = rng.uniform(0.5, 2.0, size=2)
    split = rng.uniform(0.3, 0.9)               # in-group fraction of group-1 scattering
    P0 = np.zeros((1, 2, 2))
    P0[0, 0, 0] = 0.9 * sig_t[0] * split
    P0[0, 0, 1] = 0.9 * sig_t[0] * (1.0 - split)
    P0[0, 1, 1] = 0.9 * sig_t[1]
    capture = 0.1 * sig_t
    mg = mg_data(2, sig_t[None, :], P0, capture=capture[None, :])
    gb = GeometryBuilder()
    box = gb.surface(abi.BOX, 0.0, 0.0, 0.0, half_width, half_width, half_width)
    gb.root_universe(box, 1, bc=[abi.BC_REFLECTIVE] * 6)
    tallies = dict(flux=[abi.clerk(abi.CLERK_COLLISION, resp=(abi.RESP_FLUX,),
                                   axes=[(abi.AXIS_GROUP, 2, 0.0, 0.0)])])
    return Problem(gb.arrays(), mg, name="infinite_medium_2g", eigen=False,
                   source=dict(r=(0.0, 0.0, 0.0), G=1), tallies=tallies,
                   meta=dict(seed=seed, sigma_t=sig_t.tolist()))


def _lattice_xs(rng, n_g, fissile):
    """One region's 7-group data: Sigma_t ~ U[0.2, 2.0], downscatter-dominant P0 with upscatter in
    the last two groups, nu*Sigma_f only where fissile."""
    sig_t = rng.uniform(0.2, 2.0, size=n_g)
    c = rng.uniform(0.55, 0.85, size=n_g) if fissile else rng.uniform(0.92, 0.99, size=n_g)
    P0 = np.zeros((n_g, n_g))
    for g in range(n_g):
        s = c[g] * sig_t[g]
        w = np.zeros(n_g)
        w[g] = rng.uniform(0.5, 0.8)                       # in-group
        for d in range(1, n_g - g):                         # downscatter, decaying
            w[g + d] = rng.uniform(0.05, 0.3) * 0.5 ** (d - 1)
        if g >= n_g - 2:                                    # upscatter in the last 2 groups
            w[g - 1] = rng.uniform(0.02, 0.1)
        P0[g] = s * w / w.sum()
    absorb = sig_t - P0.sum(axis=1)
    if fissile:
        frac = rng.uniform(0.25, 0.6, size=n_g)
        fis = absorb * frac
        cap = absorb - fis
        nu = rng.uniform(2.4, 2.9, size=n_g)
    else:
        fis = np.zeros(n_g)
        cap = absorb
        nu = np.zeros(n_g)
    return sig_t, P0, cap, fis, nu


def lattice_17x17_7g(seed=11, n_fuel=4, pitch=1.26, radius=0.54, n=17):
    """2D 17x17 square lattice of cylindrical pins (r 0.54 cm, pitch 1.26 cm) in a reflective box,
    7 groups with seeded synthetic XS per region (moderator + n_fuel fuel types), k-eigenvalue.

    The geometry has the shape of SCONE's C5G7 deck (root box -> latUniverse -> pinUniverse), the
    cross sections are synthetic.  Tally: 17x17x7 mesh flux (collision estimator).
    """
    rng = np.random.default_rng(seed)
    n_g = 7
    mats = [_lattice_xs(rng, n_g, False)] + [_lattice_xs(rng, n_g, True) for _ in range(n_fuel)]
    chi = np.zeros((len(mats), n_g))
    for m in range(1, len(mats)):
        x = np.array([0.58, 0.41, 0.01, 0, 0, 0, 0]) * rng.uniform(0.9, 1.1, size=n_g)
        chi[m] = x / x.sum()
    mg = mg_data(n_g, np.array([m[0] for m in mats]), np.array([m[1] for m in mats]),
                 capture=np.array([m[2] for m in mats]), fission=np.array([m[3] for m in mats]),
                 nu=np.array([m[4] for m in mats]), chi=chi)
    gb = GeometryBuilder()
    hw = n * pitch / 2.0
    box = gb.surface(abi.BOX, 0.0, 0.0, 0.0, hw, hw, hw)
    pins = [gb.pin_universe([radius], [2 + f, 1]) for f in range(n_fuel)]
    layout = rng.integers(0, n_fuel, size=n * n)
    lat = gb.lattice_universe((n, n, 0), (pitch, pitch, 0.0), [uni_fill(pins[k]) for k in layout], 1)
    gb.root_universe(box, uni_fill(lat), bc=[abi.BC_REFLECTIVE] * 6)
    tallies = dict(mesh=[abi.clerk(abi.CLERK_COLLISION, resp=(abi.RESP_FLUX,),
                                   axes=[(abi.AXIS_X, n, -hw, hw), (abi.AXIS_Y, n, -hw, hw),
                                         (abi.AXIS_GROUP, n_g, 0.0, 0.0)])])
    return Problem(gb.arrays(), mg, name="lattice_17x17_7g", eigen=True, tallies=tallies,
                   meta=dict(seed=seed, n_fuel=n_fuel, pitch=pitch, radius=radius, n=n))


def scone_test_lat():
    """SCONE's IntegrationTestFiles/Geometry/test_lat rebuilt with this builder.

    Materials (dictionary key order): water = 1, mox43 = 2, uox = 3.  Boundary (1 1 2 2 0 0).
    """
    water, mox43, uox = 1, 2, 3
    gb = GeometryBuilder()
    sq_bound = gb.surface(abi.ZSQCYL, 0.0, 0.0, 0.0, 1.26, 1.26, 0.0)
    sq_pin = gb.surface(abi.ZSQCYL, 0.0, 0.0, 0.0, 0.5, 0.5, 0.0)
    c_in = gb.cell([-(sq_pin + 1)])
    c_out = gb.cell([sq_pin + 1])
    pin31 = gb.pin_universe([0.54], [mox43, water])
    sqpin = gb.cell_universe([c_in, c_out], [uox, water])
    ids = {31: pin31, 32: sqpin}
    fills = [uni_fill(ids[v]) for v in lattice_fills_from_map([31, 32, 32, 31], (2, 2, 0))]
    lat = gb.lattice_universe((2, 2, 0), (1.26, 1.26, 0.0), fills, water)
    gb.root_universe(sq_bound, uni_fill(lat), bc=[1, 1, 2, 2, 0, 0])
    return gb.arrays(), dict(water=water, mox43=mox43, uox=uox)
