"""Problem descriptions for libsconegpu: a CSG geometry builder, MG data, tallies and the seeded
synthetic generators for the benchmark workloads.

The generators stand in for SCONE input decks (SCONE's own dictionary parser is not part of the
transport hot path); they produce the same geometry tables that SCONE's `geometryStd%init`
(Geometry/csg_class.f90:50-207) and MG `baseMgNeutronDatabase%init`
(NuclearData/mgNeutronData/baseMgNeutron/baseMgNeutronDatabase_class.f90:340-410) build.

Workloads (all synthetic, seeded with numpy default_rng):
  * ``infinite_medium_2g``  -- 2-group infinite homogeneous medium, point source (fixed source).
  * ``lattice_17x17_7g``    -- 17x17 pin lattice, 7 groups, k-eigenvalue.
  * ``ce_slab_3layer``      -- continuous-energy 3-layer slab (5/20/5 cm), 10 synthetic nuclides,
                               fixed source, log-energy surface-current tally.
  * ``batched_uneven``      -- many independent fixed-source problems of uneven size (group counts
                               {1,2,4,7,16}, a sphere or a 1-D multi-slab, log-uniform history counts).
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
        self.rot = {}           # universe -> (phi, theta, psi) Euler angles in degrees
        self.root = None
        self.border = None
        self.bc = [0] * 6

    def surface(self, type_, *par):
        p = list(par) + [0.0] * (abi.SG_SURF_NPAR - len(par))
        self.surf_type.append(type_)
        self.surf_par.append(p)
        return len(self.surf_type) - 1

    def cell(self, signed_surfs):
        """signed 1-based surface indices: -(s+1) for the -ve halfspace of surface s (0-based); a list
        with abi.CELL_* operator tokens ('<', '>', ':', '#') is a unionCell."""
        self.cells.append(list(signed_surfs))
        return len(self.cells) - 1

    def universe(self, type_, fills, ipar=(), dpar=(), origin=(0.0, 0.0, 0.0)):
        self.unis.append((type_, list(origin), list(ipar), list(dpar), list(fills)))
        return len(self.unis) - 1

    def rotate(self, uni, angles):
        """Give universe `uni` the `rotation` (phi, theta, psi) in degrees, ZXZ Euler angles."""
        self.rot[uni] = tuple(float(a) for a in angles)
        return uni

    def root_universe(self, border_surf, fill, bc=(0, 0, 0, 0, 0, 0)):
        self.border = border_surf
        self.bc = list(bc)
        self.root = self.universe(abi.UNI_ROOT, [fill], ipar=[border_surf])
        return self.root

    def pin_universe(self, radii, fills, origin=(0.0, 0.0, 0.0)):
        return self.universe(abi.UNI_PIN, fills, dpar=sorted(radii), origin=origin)

    def lattice_universe(self, shape, pitch, fills_local_order, pad_fill, offset=True, origin=(0.0, 0.0, 0.0)):
        return self.universe(abi.UNI_LAT, list(fills_local_order) + [pad_fill],
                             ipar=list(shape) + [1 if offset else 0], dpar=list(pitch), origin=origin)

    def cell_universe(self, cell_idx, fills, origin=(0.0, 0.0, 0.0)):
        return self.universe(abi.UNI_CELL, fills, ipar=cell_idx, origin=origin)

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
            uni_rot=(np.array([self.rot.get(i, (0.0, 0.0, 0.0)) for i in range(len(self.unis))], np.float64)
                     if self.rot else None),
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
            prod=None, avg_dist=0.0, p1=None):
    """Assemble an MG desc dict; scatter_matrix[m][g_in][g_out] (xsFile `P0` layout); p1 in the same
    layout makes the scattering linearly anisotropic (xsFile `P1`, `PN P1`)."""
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
        fissile=fissile, avg_dist=avg_dist,
        p1=None if p1 is None else np.asarray(p1, np.float64).reshape(n_mat, n_g, n_g))


class Problem:
    """Geometry + data + tallies + source of one transport problem."""

    def __init__(self, geometry, mg, name="", source=None, tallies=None, eigen=False, meta=None, ce=None):
        self.geometry = geometry
        self.mg = mg
        self.ce = ce
        self.name = name
        self.source = source or {}
        self.tallies = tallies or {}
        self.eigen = eigen
        self.meta = meta or {}


# ----------------------------------------------------------------------------- workloads
def infinite_medium_2g(seed=7, half_width=10.0, p1_ratio=None):
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
    # optional linearly anisotropic scattering: P1 = p1_ratio * P0 (mean scattering cosine p1_ratio)
    p1 = None if p1_ratio is None else np.asarray(p1_ratio, np.float64) * P0
    mg = mg_data(2, sig_t[None, :], P0, capture=capture[None, :], p1=p1)
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


def scone_test_lat_problem(seed=13, n_g=4):
    """A transport problem on SCONE's test_lat geometry: the squareCylinder root with reflective x and
    periodic y boundaries (BC 1 1 2 2 0 0, z unbounded), a 2x2 lattice of a cylindrical pin and a
    square pin in a cellUniverse.  n_g groups of seeded synthetic data (water non-fissile, mox43 and
    uox fissile, as the lattice workload's regions); an isotropic point source in group 1 at
    (0.3, -0.2, 0); collision mesh flux (4x4 over the root) per group, track flux per material."""
    g, mats = scone_test_lat()
    rng = np.random.default_rng(seed)
    regions = [_lattice_xs(rng, n_g, False), _lattice_xs(rng, n_g, True), _lattice_xs(rng, n_g, True)]
    chi = np.zeros((3, n_g))
    for m in (1, 2):
        x = rng.uniform(0.1, 1.0, size=n_g) * np.exp(-np.arange(n_g))
        chi[m] = x / x.sum()
    mg = mg_data(n_g, np.array([r[0] for r in regions]), np.array([r[1] for r in regions]),
                 capture=np.array([r[2] for r in regions]), fission=np.array([r[3] for r in regions]),
                 nu=np.array([r[4] for r in regions]), chi=chi)
    tallies = dict(flux=[abi.clerk(abi.CLERK_COLLISION, axes=[(abi.AXIS_X, 4, -1.26, 1.26), (abi.AXIS_Y, 4, -1.26, 1.26),
                                                              (abi.AXIS_GROUP, n_g, 0.0, 0.0)]),
                         abi.clerk(abi.CLERK_TRACK, axes=[(abi.AXIS_MATERIAL, 3, 0.0, 0.0)])])
    return Problem(g, mg, name="scone_test_lat", source=dict(r=(0.3, -0.2, 0.0), G=1), tallies=tallies,
                   meta=dict(mats=mats, seed=seed))


def plane_cells(seed=47):
    """General planes (plane_class.f90) and the box's periodic boundary: a box (half-width 4 cm) with
    periodic x, reflective y and vacuum z faces holds a cellUniverse of four cells cut by two tilted
    planes (normals (1, 2, 0.5) and (-0.3, 1, 1.5), offsets 0.7 and -0.4) and a sphere (r 1.5 cm at
    (1, 0, 0)), two materials alternating; 2 groups (synthetic XS as in the infinite-medium workload),
    a point source at the origin, collision flux per material and group and a track-length x mesh
    over [-4.5, 4.5] (its bin edges stay off the periodic faces, where a track that starts right after
    a periodic translation would be binned by the last bit of its position)."""
    rng = np.random.default_rng(seed)
    gb = GeometryBuilder()
    box = gb.surface(abi.BOX, 0.0, 0.0, 0.0, 4.0, 4.0, 4.0)
    p1 = gb.surface(abi.PLANE, 1.0, 2.0, 0.5, 0.7)
    p2 = gb.surface(abi.PLANE, -0.3, 1.0, 1.5, -0.4)
    sph = gb.surface(abi.SPHERE, 1.0, 0.0, 0.0, 1.5)
    cells = [gb.cell([-(sph + 1), -(p1 + 1)]), gb.cell([-(sph + 1), p1 + 1]),
             gb.cell([sph + 1, -(p2 + 1)]), gb.cell([sph + 1, p2 + 1])]
    uni = gb.cell_universe(cells, [1, 2, 2, 1])
    gb.root_universe(box, uni_fill(uni), bc=[abi.BC_PERIODIC, abi.BC_PERIODIC, abi.BC_REFLECTIVE,
                                             abi.BC_REFLECTIVE, abi.BC_VACUUM, abi.BC_VACUUM])
    mats = [_fixed_source_xs(rng, 2), _fixed_source_xs(rng, 2)]
    mg = mg_data(2, np.array([m[0] for m in mats]), np.array([m[1] for m in mats]),
                 capture=np.array([m[2] for m in mats]))
    tallies = dict(flux=[abi.clerk(abi.CLERK_COLLISION, axes=[(abi.AXIS_MATERIAL, 2, 0.0, 0.0),
                                                              (abi.AXIS_GROUP, 2, 0.0, 0.0)]),
                         abi.clerk(abi.CLERK_TRACK, axes=[(abi.AXIS_X, 8, -4.5, 4.5)])])
    return Problem(gb.arrays(), mg, name="plane_cells", source=dict(r=(0.0, 0.0, 0.0), G=1), tallies=tallies)


# ----------------------------------------------------------------------------- CE data
KT_293K = 2.53e-8          # kT at 293.6 K [MeV]


def synthetic_nuclide(rng, n_points, A, kT=KT_293K, e_min=1.0e-11, e_max=20.0):
    """One synthetic non-fissile nuclide on a log-spaced grid of n_points over [e_min, e_max] MeV.

    elastic = potential scattering + a_el E^-1/2 + Lorentzian (single-level Breit-Wigner shaped)
    peaks; capture = a_c E^-1/2 + the capture part of the same peaks (with the sqrt(E0/E) factor);
    total = elastic + capture; no inelastic channel.  20-200 peaks at log-uniform energies in
    [10 eV, 100 keV] with relative widths in [5e-4, 5e-3], heights 3-1000 b and elastic
    fractions in [0.6, 0.99]."""
    e = np.geomspace(e_min, e_max, n_points)
    e[0], e[-1] = e_min, e_max
    s_pot = rng.uniform(2.0, 20.0)
    a_el = rng.uniform(0.0, 1.0e-3)
    a_c = rng.uniform(1.0e-5, 2.0e-3)
    n_peaks = int(rng.integers(20, 201))
    e0 = 10.0 ** rng.uniform(-5.0, -1.0, n_peaks)
    width = e0 * 10.0 ** rng.uniform(-3.3, -2.3, n_peaks)
    height = 10.0 ** rng.uniform(0.5, 3.0, n_peaks)
    gn = rng.uniform(0.6, 0.99, n_peaks)
    inv_sqrt = 1.0 / np.sqrt(e)
    el = s_pot + a_el * inv_sqrt
    cap = a_c * inv_sqrt
    for k in range(n_peaks):
        lor = 1.0 / (1.0 + (2.0 * (e - e0[k]) / width[k]) ** 2)
        el = el + height[k] * gn[k] * lor
        cap = cap + height[k] * (1.0 - gn[k]) * np.sqrt(e0[k]) * inv_sqrt * lor
    xs = np.zeros((n_points, 4))
    xs[:, 0] = el + cap
    xs[:, 1] = el
    xs[:, 3] = cap
    return dict(e=e, xs=xs, A=float(A), kT=float(kT))


def ce_data(nuclides, materials, **settings):
    """Assemble an sg_ce_desc dict: nuclides = [dict(e, xs, A, kT)], materials = [[(nuc, dens)]]."""
    nuc_ptr = np.zeros(len(nuclides) + 1, np.int64)
    for i, n in enumerate(nuclides):
        nuc_ptr[i + 1] = nuc_ptr[i] + len(n["e"])
    mat_ptr = np.zeros(len(materials) + 1, np.int32)
    for i, m in enumerate(materials):
        mat_ptr[i + 1] = mat_ptr[i] + len(m)
    d = dict(
        nuc_ptr=nuc_ptr,
        e=np.concatenate([n["e"] for n in nuclides]).astype(np.float64),
        xs=np.concatenate([n["xs"] for n in nuclides]).astype(np.float64).reshape(-1, 4),
        A=np.array([n["A"] for n in nuclides], np.float64),
        kT=np.array([n["kT"] for n in nuclides], np.float64),
        mat_ptr=mat_ptr,
        mat_nuc=np.array([k for m in materials for k, _ in m], np.int32),
        mat_dens=np.array([x for m in materials for _, x in m], np.float64))
    d.update(settings)
    return d


def ce_slab_3layer(seed=23, n_nuc=10, points=(20000, 100000), scale=1.0, source_E=2.0):
    """Continuous-energy fixed-source 3-layer slab: x in [0,5], [5,25], [25,30] cm (xPlane cells of a
    cellUniverse), vacuum in x, reflective in y and z; 10 synthetic nuclides with log grids of
    U{2e4..1e5} points over [1e-11, 20] MeV and masses A ~ U[1, 60] (nuclide 4 has A = 1, which
    always scatters from a moving target), kT = 2.53e-8 MeV; isotropic 2 MeV point source at the
    slab centre.  Tallies: 200-bin log-energy current through the planes x = 0, 5, 25, 30, and a
    collision-estimator flux per material and 200 log-energy bins.

    ``scale`` < 1 shrinks the grids (a cheaper case with the same structure for the tests)."""
    rng = np.random.default_rng(seed)
    sizes = rng.integers(points[0], points[1] + 1, n_nuc)
    sizes = np.maximum(64, (sizes * scale).astype(int))
    A = rng.uniform(1.0, 60.0, n_nuc)
    A[4] = 1.0
    nucs = [synthetic_nuclide(rng, int(sizes[i]), A[i]) for i in range(n_nuc)]
    dens = lambda: float(rng.uniform(0.004, 0.03))
    materials = [
        [(0, dens()), (1, dens()), (2, dens()), (3, dens())],
        [(2, dens()), (3, dens()), (4, dens()), (5, dens()), (6, dens()), (7, dens())],
        [(6, dens()), (7, dens()), (8, dens()), (9, dens())],
    ]
    ce = ce_data(nucs, materials)
    gb = GeometryBuilder()
    box = gb.surface(abi.BOX, 15.0, 0.0, 0.0, 15.0, 50.0, 50.0)
    p5 = gb.surface(abi.XPLANE, 5.0)
    p25 = gb.surface(abi.XPLANE, 25.0)
    c1 = gb.cell([-(p5 + 1)])
    c2 = gb.cell([p5 + 1, -(p25 + 1)])
    c3 = gb.cell([p25 + 1])
    slab = gb.cell_universe([c1, c2, c3], [1, 2, 3])
    bc = [abi.BC_VACUUM, abi.BC_VACUUM] + [abi.BC_REFLECTIVE] * 4
    gb.root_universe(box, uni_fill(slab), bc=bc)
    e_axis = (abi.AXIS_ENERGY, 200, 1.0e-11, 20.0)
    tallies = dict(
        current=[abi.clerk(abi.CLERK_SURFACE_CURRENT, axes=[e_axis], current_axis=abi.AXIS_X,
                           planes=(0.0, 5.0, 25.0, 30.0))],
        flux=[abi.clerk(abi.CLERK_COLLISION, axes=[e_axis, (abi.AXIS_MATERIAL, 3, 0.0, 0.0)])])
    return Problem(gb.arrays(), None, name="ce_slab_3layer", eigen=False, ce=ce,
                   source=dict(r=(15.0, 0.0, 0.0), E=source_E), tallies=tallies,
                   meta=dict(seed=seed, grid_points=[int(x) for x in sizes], A=A.tolist()))


def ce_infinite_medium(A=1.0, sigma_s=20.0, sigma_c=0.1, dens=0.05, kT=KT_293K, n_points=4000,
                       source_E=None):
    """One nuclide with constant elastic and capture cross sections in an all-reflective box: the
    collision-density spectrum approaches the Maxwellian flux E exp(-E/kT) when the source starts
    near thermal energies (free-gas scattering for A = 1)."""
    e = np.geomspace(1.0e-11, 20.0, n_points)
    e[0], e[-1] = 1.0e-11, 20.0
    xs = np.zeros((n_points, 4))
    xs[:, 1] = sigma_s
    xs[:, 3] = sigma_c
    xs[:, 0] = sigma_s + sigma_c
    ce = ce_data([dict(e=e, xs=xs, A=A, kT=kT)], [[(0, dens)]])
    gb = GeometryBuilder()
    box = gb.surface(abi.BOX, 0.0, 0.0, 0.0, 100.0, 100.0, 100.0)
    gb.root_universe(box, 1, bc=[abi.BC_REFLECTIVE] * 6)
    return Problem(gb.arrays(), None, name="ce_infinite_medium", ce=ce,
                   source=dict(r=(0.0, 0.0, 0.0), E=kT if source_E is None else source_E))


# ----------------------------------------------------------------------------- batched workload
GROUP_CHOICES = (1, 2, 4, 7, 16)


def _fixed_source_xs(rng, n_g):
    """One material's data as in the infinite-medium workload, for n_g groups: Sigma_t ~ U[0.5, 2.0],
    scattering ratio 0.9 with downscatter only (an in-group fraction, the rest spread over the lower
    energy groups, decaying), capture 0.1 Sigma_t, no fission."""
    sig_t = rng.uniform(0.5, 2.0, size=n_g)
    P0 = np.zeros((n_g, n_g))
    for g in range(n_g):
        s = 0.9 * sig_t[g]
        if g == n_g - 1:
            P0[g, g] = s
            continue
        w = np.zeros(n_g)
        w[g] = rng.uniform(0.3, 0.9)
        for d in range(1, n_g - g):
            w[g + d] = (1.0 - w[g]) * 0.5 ** d
        P0[g] = s * w / w.sum()
    return sig_t, P0, 0.1 * sig_t


def fixed_source_problem(rng, n_g, kind, radius=None, layers=None):
    """One problem of the batched workload: a homogeneous sphere (vacuum boundary) or a 1-D multi-slab
    (xPlane layers in a cellUniverse, vacuum in x, reflective in y and z), n_g groups, an isotropic
    point source in group 1 at the origin, and a collision-estimator flux tally per group."""
    gb = GeometryBuilder()
    if kind == "sphere":
        R = float(radius if radius is not None else rng.uniform(1.0, 50.0))
        sph = gb.surface(abi.SPHERE, 0.0, 0.0, 0.0, R)
        gb.root_universe(sph, 1, bc=[abi.BC_VACUUM] * 6)
        mats = [_fixed_source_xs(rng, n_g)]
        meta = dict(kind="sphere", radius=R)
    else:
        L = int(layers if layers is not None else rng.integers(2, 11))
        widths = rng.uniform(1.0, 10.0, size=L)
        edges = np.concatenate([[0.0], np.cumsum(widths)])
        edges = edges - edges[-1] / 2.0                      # slab centred on the source
        half = edges[-1]
        box = gb.surface(abi.BOX, 0.0, 0.0, 0.0, half, 10.0, 10.0)
        planes = [gb.surface(abi.XPLANE, float(x)) for x in edges[1:-1]]
        cells = []
        for i in range(L):
            sides = []
            if i > 0:
                sides.append(planes[i - 1] + 1)
            if i < L - 1:
                sides.append(-(planes[i] + 1))
            cells.append(gb.cell(sides))
        slab = gb.cell_universe(cells, list(range(1, L + 1)))
        gb.root_universe(box, uni_fill(slab), bc=[abi.BC_VACUUM, abi.BC_VACUUM] + [abi.BC_REFLECTIVE] * 4)
        mats = [_fixed_source_xs(rng, n_g) for _ in range(L)]
        meta = dict(kind="slab", layers=L, edges=edges.tolist())
    mg = mg_data(n_g, np.array([m[0] for m in mats]), np.array([m[1] for m in mats]),
                 capture=np.array([m[2] for m in mats]))
    tallies = dict(flux=[abi.clerk(abi.CLERK_COLLISION, resp=(abi.RESP_FLUX,),
                                   axes=[(abi.AXIS_GROUP, n_g, 0.0, 0.0)])])
    meta["groups"] = n_g
    return Problem(gb.arrays(), mg, name=f"{meta['kind']}_{n_g}g", eigen=False,
                   source=dict(r=(0.0, 0.0, 0.0), G=1), tallies=tallies, meta=meta)


def batched_uneven(n_problems=4096, seed=31, hist_min=1.0e3, hist_max=1.0e6, cycles=10):
    """The uneven batch: n_problems independent fixed-source problems, each with a seeded group count
    in {1, 2, 4, 7, 16}, a sphere (radius U[1, 50] cm) or a 1-D multi-slab (2-10 layers), synthetic XS
    as in the infinite-medium workload and a log-uniform history count in [hist_min, hist_max], run as
    `cycles` cycles of pop = histories / cycles.  Returns [(problem, pop, cycles, master)]."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n_problems):
        n_g = int(rng.choice(GROUP_CHOICES))
        kind = "sphere" if rng.uniform() < 0.5 else "slab"
        p = fixed_source_problem(rng, n_g, kind)
        hist = float(np.exp(rng.uniform(np.log(hist_min), np.log(hist_max))))
        pop = max(1, int(round(hist / cycles)))
        master = int(rng.integers(1, 2 ** 63 - 1))
        p.meta["index"] = i
        out.append((p, pop, cycles, master))
    return out


def union_cell_slab(seed=41):
    """Two overlapping spheres (r 2 cm at x = 0 and x = 3) inside a reflective box (half-width 6 cm)
    as unionCells: material 1 fills the union `< -1 : -2 >`, material 2 its complement
    `# < -1 : -2 >`; an isotropic point source at the origin, 2 groups (synthetic XS as in the
    infinite-medium workload) and a collision flux per material and group."""
    rng = np.random.default_rng(seed)
    gb = GeometryBuilder()
    box = gb.surface(abi.BOX, 0.0, 0.0, 0.0, 6.0, 6.0, 6.0)
    s1 = gb.surface(abi.SPHERE, 0.0, 0.0, 0.0, 2.0)
    s2 = gb.surface(abi.SPHERE, 3.0, 0.0, 0.0, 2.0)
    O, C, U, N = abi.CELL_OPEN, abi.CELL_CLOSE, abi.CELL_UNION, abi.CELL_COMPLEMENT
    inside = gb.cell([O, -(s1 + 1), U, -(s2 + 1), C])
    outside = gb.cell([N, O, -(s1 + 1), U, -(s2 + 1), C])
    uni = gb.cell_universe([inside, outside], [1, 2])
    gb.root_universe(box, uni_fill(uni), bc=[abi.BC_REFLECTIVE] * 6)
    mats = [_fixed_source_xs(rng, 2), _fixed_source_xs(rng, 2)]
    mg = mg_data(2, np.array([m[0] for m in mats]), np.array([m[1] for m in mats]),
                 capture=np.array([m[2] for m in mats]))
    tallies = dict(flux=[abi.clerk(abi.CLERK_COLLISION, axes=[(abi.AXIS_MATERIAL, 2, 0.0, 0.0),
                                                              (abi.AXIS_GROUP, 2, 0.0, 0.0)])])
    return Problem(gb.arrays(), mg, name="union_cell_spheres", source=dict(r=(0.0, 0.0, 0.0), G=1),
                   tallies=tallies)


def rotated_pins(seed=43):
    """Rotated universes (universe `rotation`, ZXZ Euler angles): a vacuum box (half-width 5 cm)
    holds a cellUniverse turned 30 degrees about z and offset to x = 0.5; its half x < 0 holds a pin
    universe turned 90 degrees about x (the pin's axis along y of the cell universe), its other half
    a second material; a point source and collision/track flux per material and group."""
    rng = np.random.default_rng(seed)
    gb = GeometryBuilder()
    box = gb.surface(abi.BOX, 0.0, 0.0, 0.0, 5.0, 5.0, 5.0)
    xp = gb.surface(abi.XPLANE, 0.0)
    pin = gb.pin_universe([1.2], [1, 2])
    gb.rotate(pin, (0.0, 90.0, 0.0))
    left = gb.cell([-(xp + 1)])
    right = gb.cell([xp + 1])
    cu = gb.cell_universe([left, right], [uni_fill(pin), 3], origin=(0.5, 0.0, 0.0))
    gb.rotate(cu, (30.0, 0.0, 0.0))
    gb.root_universe(box, uni_fill(cu), bc=[abi.BC_VACUUM] * 6)
    mats = [_fixed_source_xs(rng, 2) for _ in range(3)]
    mg = mg_data(2, np.array([m[0] for m in mats]), np.array([m[1] for m in mats]),
                 capture=np.array([m[2] for m in mats]))
    axes = [(abi.AXIS_MATERIAL, 3, 0.0, 0.0), (abi.AXIS_GROUP, 2, 0.0, 0.0)]
    tallies = dict(flux=[abi.clerk(abi.CLERK_COLLISION, axes=axes), abi.clerk(abi.CLERK_TRACK, axes=axes),
                         abi.clerk(abi.CLERK_COLLISION, axes=[(abi.AXIS_X, 10, -5.0, 5.0), (abi.AXIS_Y, 10, -5.0, 5.0)])])
    return Problem(gb.arrays(), mg, name="rotated_pins", source=dict(r=(-1.0, 0.3, 0.2), G=1), tallies=tallies)
