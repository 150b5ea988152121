"""Pins the CPU oracle to SCONE: the known answers of SCONE's own unit and integration tests
(cited per test) and a Python big-integer evaluation of its RNG (tests/golden/make_golden.py)."""
import json
import math
import os

import numpy as np
import pytest

from scone_gb300 import abi, problems

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "scone_golden.json")))
SURF_TOL = 1.0e-12
INF = 2.0 ** 63
SQRT2 = math.sqrt(2.0)


# ---------------------------------------------------------------- RNG (RandomNumbers/RNG_class.f90)
def test_rng_draws_match_bigint_recurrence(oracle_mod):
    g = GOLD["rng"]
    xs, s = oracle_mod.rng_draws(g["seed"], 1000)
    assert np.array_equal(xs[:64], np.array(g["draws"]))
    assert str(s) == g["state_1000"]


def test_rng_skip_matches_bigint(oracle_mod):
    g = GOLD["rng"]
    for k, v in g["skip"].items():
        assert str(oracle_mod.rng_skip(g["seed"], int(k))) == v, k
    for k, v in g["skip_negative"].items():
        assert str(oracle_mod.rng_skip(g["seed"], int(k))) == v, k


def test_rng_skip_forward_backward_scone(oracle_mod):
    # RandomNumbers/Tests/RNG_test.f90:36-70
    seed = 0x5C3A84C9
    first, _ = oracle_mod.rng_draws(seed, 1)
    N = 13456757
    seq, s_end = oracle_mod.rng_draws(seed, N + 1)
    s2 = oracle_mod.rng_skip(seed, N)
    r2_end, s2 = oracle_mod.rng_draws(s2, 1)
    assert r2_end[0] == seq[N]          # the (N+1)-th draw: r_end after N draws following the first
    back = oracle_mod.rng_skip(s2, -(N + 1))
    r2_start, _ = oracle_mod.rng_draws(back, 1)
    assert r2_start[0] == first[0]


def test_rng_pow_of_gsq_table_is_successive_squares():
    # RNG_class.f90:53-59 documents the table as g^(2^j) mod 2^63
    G, M = 2806196910506780709, (1 << 63) - 1
    g = G
    for j, v in enumerate(GOLD["pow_of_gsq"][:60]):
        g = (g * g) & M
        assert g == int(v), j


# ---------------------------------------------------------------- scoreMemory (Tallies/Tests/scoreMemory_test.f90:92-200)
def test_score_memory_golden(oracle_mod):
    A, M = 2469, 65521
    seed = 9294
    rnd = []
    for _ in range(200):
        seed = (A * seed) % M
        rnd.append(seed / float(M))
    rnd = np.array(rnd)
    scores = 2.0 + np.sin(math.pi * rnd - math.pi / 2)
    ints = (rnd * 100).astype(np.int32)
    mem = oracle_mod.ScoreMemory(7, 1)
    for i in range(10):
        for j in range(20 * i, 20 * i + 20):
            mem.score(float(scores[j]), 1)
            mem.score(float(ints[j]), 2)
            mem.score(float(ints[j]), 3)
            mem.accumulate(float(scores[j]), 4)
            mem.accumulate(float(ints[j]), 5)
            mem.accumulate(float(ints[j]), 6)
        mem.reduce_bins()
        mem.close_bin(1.2, 3)
        mem.close_cycle_only(0.7)
    tol = 1e-9
    m, s = mem.result(1)
    assert abs(m - 26.401471259728442) < tol and abs(s - 0.645969443981583) < tol
    m, s = mem.result(2)
    assert abs(m - 623.0) < tol and abs(s - 27.982494527829360) < tol
    m, s = mem.result(3)
    assert abs(m - 1068.0) < tol and abs(s - 47.969990619136050) < tol
    m, s = mem.result(4, 200)
    assert abs(m - 1.885819375694888) < tol and abs(s - 0.049102082638055) < tol
    m, s = mem.result(5, 200)
    assert abs(m - 44.5) < tol and abs(s - 2.015580019267494) < tol
    m, s = mem.result(7)
    assert m == 0.0 and s == 0.0
    m, s = mem.result(-7)
    assert m == 0.0 and s == 0.0


# ---------------------------------------------------------------- surfaces (Geometry/Surfaces/Tests)
def _unit(v):
    v = np.array(v, float)
    return v / np.linalg.norm(v)


@pytest.mark.parametrize("axis", [0, 1, 2])
def test_cylinder_distance_and_halfspace(oracle_mod, axis):
    # cylinder_test.f90:200-340 -- origin (2,2,2), radius 2, x/y/z cylinders
    typ = [abi.XCYL, abi.YCYL, abi.ZCYL][axis]
    par = [2.0, 2.0, 2.0, 2.0]
    a = axis
    p1, p2 = [(1, 2), (0, 2), (0, 1)][axis]
    ev = lambda r, u: oracle_mod.surf_eval(typ, par, r, u)
    tol = 1e-7
    # halfspace
    r = np.full(3, 2.0); r[p1] = 0.0
    u = np.zeros(3); u[p1] = 1.0; u[a] = 1.0; u = _unit(u)
    assert not ev(r, u)["halfspace"]
    assert not ev(r - SURF_TOL * u, u)["halfspace"]
    assert ev(r - SQRT2 * 1.00001 * SURF_TOL * u, u)["halfspace"]
    assert ev(r - 2.0 * u, u)["halfspace"]
    assert not ev(r + 2.0 * u, u)["halfspace"]
    ut = np.zeros(3); ut[p2] = 1.0; ut[a] = 1.0
    assert ev(r, _unit(ut))["halfspace"]
    # distance outside
    r = np.full(3, 2.0); r[p1] = -1.0
    u = np.zeros(3); u[a] = 1.0; u[p1] = 1.0; u = _unit(u)
    assert abs(ev(r, u)["distance"] - SQRT2) < tol * SQRT2
    u = np.zeros(3); u[a] = 1.0; u[p1] = math.sqrt(3.0) / 2; u[p2] = 0.5; u = _unit(u)
    ref = 1.275200556 * SQRT2
    assert abs(ev(r, u)["distance"] - ref) < tol * ref
    u = np.zeros(3); u[a] = 1.0e20; u[p1] = 1.0; u = _unit(u)
    assert ev(r, u)["distance"] == INF
    # at the surface
    r = np.full(3, 2.0); r[p1] = 0.0
    u = np.zeros(3); u[a] = 1.0; u[p1] = 1.0; u = _unit(u)
    assert abs(ev(r, u)["distance"] - 4 * SQRT2) < tol * 4 * SQRT2
    assert ev(r, -u)["distance"] == INF
    # outside within tolerance
    r = np.full(3, 2.0); r[p1] = -0.5 * SURF_TOL
    ref = (4.0 + 0.5 * SURF_TOL) * SQRT2
    assert abs(ev(r, u)["distance"] - ref) < tol * ref
    # inside
    r = np.full(3, 2.0); r[p1] = 1.0
    assert abs(ev(r, u)["distance"] - 3 * SQRT2) < tol * 3 * SQRT2
    assert abs(ev(r, -u)["distance"] - SQRT2) < tol * SQRT2


BOX = [1.0, 2.0, 1.0, 1.0, 2.0, 3.0]   # box_test.f90:12 origin (1 2 1) halfwidth (1 2 3)


def test_box_distance(oracle_mod):
    # box_test.f90:testDistance
    ev = lambda r, u: oracle_mod.surf_eval(abi.BOX, BOX, r, u)["distance"]
    tol = 1e-7
    r = [-2.0, 0.001, 1.0]
    assert abs(ev(r, [1, 0, 0]) - 2.0) < tol * 2
    assert ev(r, [-1, 0, 0]) == INF
    assert ev(r, _unit([1, -0.002, 1])) == INF
    assert abs(ev(r, _unit([1, 0, 1])) - 2 * SQRT2) < tol * 2 * SQRT2
    assert ev([-2.7, -0.3, 1.0 / 3.0], _unit([2.7, 0.3, 3.0 + 2.0 / 3.0])) == INF
    assert ev([-2.0, 0.0, 1.0], [1, 0, 0]) == INF
    r = [1.0, 2.0, -2.0]
    assert abs(ev(r, [0, 0, 1]) - 6.0) < tol * 6
    assert ev(r, [0, 0, -1]) == INF
    assert abs(ev([1.0, 2.0, -2.0 - 0.5 * SURF_TOL], [0, 0, 1]) - (6.0 + 0.5 * SURF_TOL)) < tol * 6
    u = _unit([0, 1, 1])
    assert abs(ev([1.0, 2.0, -1.0], u) - 2 * SQRT2) < tol * 2 * SQRT2
    assert abs(ev([1.0, 2.0, -1.0], -u) - SQRT2) < tol * SQRT2


def test_box_boundary_conditions(oracle_mod):
    # box_test.f90:testBC -- BC (vacuum, reflective, periodic, periodic, reflective, reflective)
    bc = [0, 1, 2, 2, 1, 1]
    f = lambda r, u, t=False: oracle_mod.surf_bc(abi.BOX, BOX, bc, r, u, transform=t)
    r, u = f([0.0, 1.0, -1.0], [1, 0, 0])
    assert np.allclose(r, [0, 1, -1]) and np.allclose(u, [1, 0, 0])
    r, u = f([1.0, 1.0, -2.0], [0, 0, -1])
    assert np.allclose(r, [1, 1, -2]) and np.allclose(u, [0, 0, 1])
    r, u = f([1.0, 0.0, -1.0], [0, -1, 0])
    assert np.allclose(r, [1, 4, -1]) and np.allclose(u, [0, -1, 0])
    r, u = f([2.0, 0.0, 4.0], _unit([1, -1, 1]))
    assert np.allclose(r, [2, 4, 4], atol=1e-6) and np.allclose(u, _unit([-1, -1, -1]), atol=1e-6)
    r, u = f([4.5, -10.0, 4.0], _unit([1, 1, 1]), True)
    assert np.allclose(r, [-0.5, 2.0, 4.0], atol=1e-6) and np.allclose(u, _unit([-1, 1, -1]), atol=1e-6)
    r, u = f([2.0, 0.0, 4.0], _unit([1, -1, 1]), True)
    assert np.allclose(r, [2, 4, 4], atol=1e-6) and np.allclose(u, _unit([-1, -1, -1]), atol=1e-6)


def test_aplane_and_sphere(oracle_mod):
    # aPlane_test / sphere_test behaviour: distance along the axis, tolerance band, parallel miss
    ev = lambda t, p, r, u: oracle_mod.surf_eval(t, p, r, u)
    assert abs(ev(abi.XPLANE, [3.0], [1.0, 0, 0], [1, 0, 0])["distance"] - 2.0) < 1e-12
    assert ev(abi.XPLANE, [3.0], [1.0, 0, 0], [-1, 0, 0])["distance"] == INF
    assert ev(abi.XPLANE, [3.0], [3.0 - 0.5 * SURF_TOL, 0, 0], [1, 0, 0])["distance"] == INF
    assert ev(abi.XPLANE, [3.0], [1.0, 0, 0], [0, 1, 0])["distance"] == INF
    s = ev(abi.SPHERE, [0, 0, 0, 2.0], [0.0, 0, 0], [1, 0, 0])
    assert abs(s["distance"] - 2.0) < 1e-12 and not s["halfspace"]
    s = ev(abi.SPHERE, [0, 0, 0, 2.0], [-4.0, 0, 0], [1, 0, 0])
    assert abs(s["distance"] - 2.0) < 1e-12 and s["halfspace"]
    assert ev(abi.SPHERE, [0, 0, 0, 2.0], [-4.0, 3.0, 0], [1, 0, 0])["distance"] == INF


def test_rotate_vector_properties(oracle_mod):
    # rotateVector (genericProcedures.f90:1047-1084): result is unit and at cosine mu to the input
    rng = np.random.default_rng(3)
    for _ in range(200):
        d = _unit(rng.normal(size=3))
        mu = rng.uniform(-1, 1)
        phi = rng.uniform(0, 2 * math.pi)
        out = oracle_mod.rotate_vector(d, mu, phi)
        assert abs(np.linalg.norm(out) - 1.0) < 1e-14
        assert abs(out @ d - mu) < 1e-12
    out = oracle_mod.rotate_vector([0.0, 0.0, 1.0], 0.3, 1.1)       # the |w| ~ 1 branch
    assert abs(out[2] - 0.3) < 1e-12


# ---------------------------------------------------------------- geometryStd (Geometry/Tests/geometryStd_iTest.f90:44-250)
def test_geometry_std_lattice_itest(oracle_mod):
    g, mats = problems.scone_test_lat()
    o = oracle_mod.Oracle()
    o.upload_geometry(g)
    tol = 1e-7
    assert o.what_is_at([0, 0, 0])[0] == mats["water"]
    assert o.what_is_at([0.63, -0.09, 0.0], [0, -1, 0])[0] == mats["mox43"]
    o.coords_init([0.1, 0.1, 0.0], [0, 0, 1])
    o.coords_place()
    for lvl, ref in ((0, [0.1, 0.1, 0.0]), (1, [0.1, 0.1, 0.0]), (2, [0.1 - 0.63, 0.1 - 0.63, 0.0])):
        r, u, _ = o.coords_get(lvl)
        assert np.allclose(r, ref, atol=tol) and np.allclose(u, [0, 0, 1])
    # unique IDs of the shrunk graph (slicePlot 'uniqueID' pixels 5,5 and 1,1)
    assert o.what_is_at([-0.63, -0.63, 0.0])[1] == 2
    assert o.what_is_at([-0.63 - 0.6, -0.63 - 0.6, 0.0])[1] == 3
    assert np.allclose(o.bounds(), [-1.26, -1.26, 0, 1.26, 1.26, 0], atol=tol)
    u = _unit([-1, -2, 0])
    o.coords_init([0, 0, 0], u)
    o.coords_move(3, 3.0)                                  # teleport
    r, uu, info = o.coords_get(0)
    assert np.allclose(r, [-1.1783592, -0.1632816, 0], atol=tol)
    assert np.allclose(uu, _unit([1, -2, 0]), atol=tol) and info["mat"] == mats["water"]
    o.coords_init([0, 0, 0], [0, -1, 0])                   # geometry moveGlobal
    d, ev = o.coords_move(2, 1.0)
    r, _, info = o.coords_get(0)
    assert ev == 1 and np.allclose(r, [0, -1, 0], atol=tol) and abs(d - 1.0) < tol
    d, ev = o.coords_move(2, 1.0)
    r, _, info = o.coords_get(0)
    assert ev == 2 and np.allclose(r, [0, 1.26, 0], atol=tol) and abs(d - 0.26) < tol
    o.coords_init([-0.63, -0.63, 0.0], [0, -1, 0])         # move (no cache)
    o.coords_place()
    for maxd, ev_ref, r_ref, d_ref in ((1.0, 3, [-0.63, -1.13, 0], 0.5), (1.0, 2, [-0.63, 1.26, 0], 0.13),
                                       (0.08, 1, [-0.63, 1.18, 0], 0.08)):
        d, ev = o.coords_move(0, maxd)
        r, _, info = o.coords_get(0)
        assert ev == ev_ref and np.allclose(r, r_ref, atol=tol) and abs(d - d_ref) < tol
        assert info["mat"] == mats["water"]


def _lattice_uni1_geometry():
    # latUniverse_test.f90:18-29 uni1: pitch (1 2 3), shape (3 2 2) (fills replaced by materials)
    gb = problems.GeometryBuilder()
    box = gb.surface(abi.BOX, 0, 0, 0, 50.0, 50.0, 50.0)
    lat = gb.lattice_universe((3, 2, 2), (1.0, 2.0, 3.0), list(range(1, 13)), 13)
    gb.root_universe(box, problems.uni_fill(lat), bc=[0] * 6)
    return gb.arrays()


def test_lattice_universe_enter_and_distance(oracle_mod):
    # latUniverse_test.f90:112-260
    o = oracle_mod.Oracle()
    o.upload_geometry(_lattice_uni1_geometry())
    for r, u, loc in (([1.0, 1.0, 0.5], [0, 0, 1], 12), ([1.6, 0.5, 0.5], [0, 0, 1], 13),
                      ([-0.5, 0.0, 0.0], _unit([-1, 1, -1]), 4)):
        o.coords_init(r, u)
        o.coords_place()
        assert o.coords_get(1)[2]["local"] == loc
    o.coords_init([0.0, 0.1, 0.5], [0.0, -0.0, 1.0])
    o.coords_place()
    d, ev = o.coords_move(0, 100.0)
    assert ev == 3 and abs(d - 2.5) < 2.5e-7
    eps = 0.5 * SURF_TOL
    o.coords_init([-1.0, 0.0 - eps, -0.5], _unit([1, 1, 0]))
    o.coords_place()
    assert o.coords_get(1)[2]["local"] == 4
    d, ev = o.coords_move(0, 100.0)
    assert abs(d - SQRT2 * 0.5) < 1e-7


# ---------------------------------------------------------------- MG data (baseMgNeutronDatabase_iTest.f90:44-130)
def _mg_from_gold(names):
    mats = [GOLD[n] for n in names]
    nG = mats[0]["numberOfGroups"]
    P0 = np.array([np.array(m["P0"]).reshape(nG, nG) for m in mats])       # rows = incident group
    prod = np.array([np.array(m["scatteringMultiplicity"]).reshape(nG, nG) for m in mats])
    cap = np.array([m["capture"] for m in mats])
    fis = np.array([m.get("fission", [0.0] * nG) for m in mats])
    nu = np.array([m.get("nu", [0.0] * nG) for m in mats])
    chi = np.array([m.get("chi", [0.0] * nG) for m in mats])
    d = problems.mg_data(nG, cap, P0, capture=cap, fission=fis, nu=nu, chi=chi, prod=prod)
    return d


def test_mg_database_itest_values(oracle_mod):
    gb = problems.GeometryBuilder()
    box = gb.surface(abi.BOX, 0, 0, 0, 1.0, 1.0, 1.0)
    gb.root_universe(box, 1, bc=[1] * 6)                     # only material 1 active (activate([1]))
    o = oracle_mod.Oracle()
    o.upload_geometry(gb.arrays())
    o.upload_mg(_mg_from_gold(["mgMat1", "mgMat2"]))
    tol = 1e-6
    assert abs(o.mg_info(1, 1)["total"] - 2.1) < tol       # getTrackingXS(MATERIAL_XS), G = 1
    assert abs(o.mg_info(2, 1)["total"] - 3.1) < tol       # getTotalMatXS(mat 2), G = 1
    assert abs(o.mg_info(1, 3)["total"] - 6.0) < tol
    assert abs(o.mg_info(1, 1)["majorant"] - 2.1) < tol
    m2 = o.mg_info(2, 1)
    assert abs(m2["scatter"] - 1.1) < tol and abs(m2["capture"] - 1.0) < tol
    assert abs(m2["fission"] - 1.0) < tol and abs(m2["nu_fission"] - 2.3) < tol
    m1 = o.mg_info(1, 4)
    assert abs(m1["total"] - 7.1) < tol and abs(m1["scatter"] - 3.1) < tol and abs(m1["capture"] - 4.0) < tol
    assert m1["fission"] == 0.0 and m1["nu_fission"] == 0.0


# ---------------------------------------------------------------- whole-cycle sanity of the restatement
def test_infinite_medium_flux_matches_analytic(oracle_mod):
    """2-group infinite medium, collision estimator: phi_1 = 1/(St1 - S11), phi_2 = phi_1 S12/(St2 - S22)."""
    p = problems.infinite_medium_2g()
    o = oracle_mod.Oracle(p)
    adm = o.upload_tally(p.tallies["flux"])
    m = 2024
    nb, n = 20, 5000
    for _ in range(nb):
        m, _ = o.fixed_source_cycle(adm, n, m)
    b = o.bins(adm)
    mean = b[:, 1] / nb / n
    sd = np.sqrt((b[:, 2] / nb - (b[:, 1] / nb) ** 2) / (nb - 1)) / n
    st = p.meta["sigma_t"]
    P0 = p.mg["p0"][0]
    phi1 = 1.0 / (st[0] - P0[0, 0])
    phi2 = phi1 * P0[0, 1] / (st[1] - P0[1, 1])
    assert abs(mean[0] - phi1) < 4 * sd[0] and abs(mean[1] - phi2) < 4 * sd[1]


def test_lattice_eigen_st_dt_agree(oracle_mod):
    """ST and DT are different estimators of the same k (SCONE's two transport operators)."""
    p = problems.lattice_17x17_7g()
    res = []
    for tr in (abi.TRANSPORT_ST, abi.TRANSPORT_DT):
        o = oracle_mod.Oracle(p, transport=tr)
        inact, act = o.upload_tally([]), o.upload_tally([])
        ia = o.upload_tally([abi.clerk(abi.CLERK_KEFF_ANALOG)])
        aa = o.upload_tally([abi.clerk(abi.CLERK_KEFF_IMPLICIT)])
        o.attach_tally(inact, ia)
        o.attach_tally(act, aa)
        o.eigen_init(4000, 99)
        for _ in range(4):
            o.eigen_cycle(inact, ia)
        for _ in range(8):
            o.eigen_cycle(act, aa)
        res.append(o.keff(aa))
    (k1, s1), (k2, s2) = res
    assert abs(k1 - k2) < 4 * math.hypot(s1, s2)


def test_batched_workload_shape():
    """The uneven batch has the stated distribution: group counts {1,2,4,7,16}, spheres of radius
    1-50 cm or 2-10 layer slabs, log-uniform history counts in [1e3, 1e6] (mean ~1.45e5)."""
    from scone_gb300 import problems
    b = problems.batched_uneven(n_problems=512, seed=31)
    groups = {p.meta["groups"] for p, *_ in b}
    assert groups == set(problems.GROUP_CHOICES)
    for p, pop, cycles, master in b:
        h = pop * cycles
        assert 995 <= h <= 1_000_005 and cycles == 10 and 0 < master < 2 ** 63
        if p.meta["kind"] == "sphere":
            assert 1.0 <= p.meta["radius"] <= 50.0
        else:
            assert 2 <= p.meta["layers"] <= 10
        assert p.mg["n_g"] == p.meta["groups"]
    logh = np.log10([pop * c for _, pop, c, _ in b])
    assert abs(logh.mean() - 4.5) < 0.15


def test_oracle_runs_batched_problem_kinds(oracle_mod):
    """Sphere and multi-slab problems run through the oracle's fixed-source cycle; the flux tally has
    one bin per group and every history ends (leakage through the vacuum boundary)."""
    from scone_gb300 import problems
    rng = np.random.default_rng(5)
    for kind in ("sphere", "slab"):
        for ng in (1, 16):
            p = problems.fixed_source_problem(rng, ng, kind)
            o = oracle_mod.Oracle(p, transport=abi.TRANSPORT_DT)
            a = o.upload_tally(p.tallies["flux"])
            m = 777
            for _ in range(2):
                m, st = o.fixed_source_cycle(a, 300, m)
            b = o.bins(a)
            assert b.shape == (ng, 3) and np.all(b[:, 1] >= 0) and b[0, 1] > 0
            assert st.n_histories == 300


def test_oracle_hybrid_tracking_limits(oracle_mod):
    """transportOperatorHT chooses per transit (transportOperatorHT_class.f90:49-81): with a cutoff near
    1 every transit in matter uses delta tracking, so the histories are those of transportOperatorDT.
    With a smaller cutoff both kinds occur and the histories differ from both operators' (a material
    whose total is the majorant has ratio 1 and takes delta tracking at any cutoff)."""
    p = problems.lattice_17x17_7g()
    n = 1500

    def run(transport, cutoff=0.0):
        o = oracle_mod.Oracle(p, transport=transport, ht_cutoff=cutoff)
        o.eigen_init(n, 0x5C3A84C9)
        bank, _ = o.eigen_bank(n)
        a = o.upload_tally(p.tallies["mesh"])
        o.transport_bank(a, bank, 31337, k_eff=1.0)
        return o.history_records(n)

    st, dt = run(abi.TRANSPORT_ST), run(abi.TRANSPORT_DT)
    hi = run(abi.TRANSPORT_HT, 0.999999)
    assert np.array_equal(hi[0], dt[0]) and np.array_equal(hi[1], dt[1])
    for c in (0.5, 1e-9):
        mid = run(abi.TRANSPORT_HT, c)
        assert not np.array_equal(mid[1], st[1]) and not np.array_equal(mid[1], dt[1])


def test_legendre_p1_sampler_moments(oracle_mod):
    """sampleLegendre_P1 (legendrePoly_func.f90:35-99) draws the linearly anisotropic cosine of
    multiScatterP1MG: for a = 3 P1/P0 the mean cosine is a/3 over the whole range |a| <= 3 (mixing of
    uniform, linear and delta parts), every draw lies in [-1, 1], and |a| > 3 is an error."""
    for a in (-2.5, -0.6, 0.0, 0.3, 0.99, 1.0, 2.0, 3.0):
        x, _ = oracle_mod.sample_legendre_p1(a, 0x1234567, 200000)
        assert np.all(np.abs(x) <= 1.0)
        assert abs(x.mean() - a / 3.0) < 5.0 * x.std() / np.sqrt(len(x)) + 1e-12, (a, x.mean())
        if abs(a) < 1.0:                     # density (1 + a mu)/2: second moment 1/3
            assert abs((x ** 2).mean() - 1.0 / 3.0) < 0.005
    with pytest.raises(RuntimeError):
        oracle_mod.sample_legendre_p1(3.5, 1, 10)


def test_p1_scattering_changes_leakage(oracle_mod):
    """Forward-peaked P1 scattering raises leakage from a finite sphere against P0 with the same
    cross sections (same RNG streams; only the scattering cosine differs)."""
    rng = np.random.default_rng(21)
    p = problems.fixed_source_problem(rng, 2, "sphere", radius=2.0)
    leak = {}
    for ratio in (None, 0.6):
        mg = dict(p.mg)
        if ratio is not None:
            mg["p1"] = ratio * np.asarray(mg["p0"])
        q = problems.Problem(p.geometry, mg, source=p.source, tallies=p.tallies)
        o = oracle_mod.Oracle(q, transport=abi.TRANSPORT_ST)
        a = o.upload_tally(q.tallies["flux"])
        m, st = o.fixed_source_cycle(a, 20000, 99)
        leak[ratio] = st.n_collisions / 20000.0      # fewer collisions per history = more leakage
    assert leak[0.6] < 0.95 * leak[None], leak


def _union_geometry(tokens_a, tokens_b):
    """Root box (half-width 6) -> cellUniverse of two cells given as token lists over surfaces
    1: sphere r 2 at the origin, 2: sphere r 2 at x = 3, 3: plane x = 1."""
    gb = problems.GeometryBuilder()
    box = gb.surface(abi.BOX, 0.0, 0.0, 0.0, 6.0, 6.0, 6.0)
    gb.surface(abi.SPHERE, 0.0, 0.0, 0.0, 2.0)
    gb.surface(abi.SPHERE, 3.0, 0.0, 0.0, 2.0)
    gb.surface(abi.XPLANE, 1.0)
    a = gb.cell(tokens_a)
    b = gb.cell(tokens_b)
    uni = gb.cell_universe([a, b], [1, 2])
    gb.root_universe(box, problems.uni_fill(uni), bc=[abi.BC_REFLECTIVE] * 6)
    return gb.arrays()


def test_union_cell_point_containment(oracle_mod):
    """unionCell (Geometry/Cells/unionCell_class.f90): unions, complements (De Morgan) and brackets
    decide containment as the boolean expression does, at random points.  Surface indices are
    1-based (the box is surface 1, the spheres 2 and 3, the plane 4)."""
    O, C, U, N = abi.CELL_OPEN, abi.CELL_CLOSE, abi.CELL_UNION, abi.CELL_COMPLEMENT
    in1 = lambda p: p[0] ** 2 + p[1] ** 2 + p[2] ** 2 < 4.0
    in2 = lambda p: (p[0] - 3.0) ** 2 + p[1] ** 2 + p[2] ** 2 < 4.0
    left = lambda p: p[0] < 1.0
    cases = [
        ([O, -2, U, -3, C], [N, O, -2, U, -3, C], lambda p: in1(p) or in2(p)),
        ([-2, U, -3], [2, 3], lambda p: in1(p) or in2(p)),                     # union at depth 0
        ([O, -2, U, -3, C, -4], [N, O, O, -2, U, -3, C, -4, C], lambda p: (in1(p) or in2(p)) and left(p)),
        ([N, O, 2, 3, C], [2, 3], lambda p: in1(p) or in2(p)),                 # # < 2 3 > = -2 : -3
        ([-2, N, -4], [N, O, -2, N, -4, C], lambda p: in1(p) and not left(p)),
    ]
    rng = np.random.default_rng(3)
    pts = rng.uniform(-5.5, 5.5, size=(400, 3))
    for ta, tb, truth in cases:
        g = _union_geometry(ta, tb)
        o = oracle_mod.Oracle()
        o.upload_geometry(g)
        for p in pts:
            m, _ = o.what_is_at(p)
            assert m == (1 if truth(p) else 2), (ta, p, m)


def test_union_cell_rejects_bad_definitions(oracle_mod):
    """Ambiguous precedence, unbalanced brackets and trailing operators are errors
    (unionCell%init, checkPrecedence)."""
    O, C, U, N = abi.CELL_OPEN, abi.CELL_CLOSE, abi.CELL_UNION, abi.CELL_COMPLEMENT
    for bad in ([-2, U, -3, -4], [O, -2, U, -3], [-2, U], [-2, N], [-2, -2, O, -3, C]):
        g = _union_geometry(bad, [2])
        o = oracle_mod.Oracle()
        with pytest.raises(RuntimeError):
            o.upload_geometry(g)


def _map_tallies(extra_x=None):
    """Collision clerks over the unionCell spheres: by material, by cell (cells listed in the
    materials' order), by the first cell with the `undefBin` rest bin, a lin x grid and the same x
    grid given as unstructured bounds."""
    step = 12.0 / 8
    bounds = np.array([-6.0 + i * step for i in range(9)])     # grid%init lin: min + (i - 1) step
    C_ = abi.CLERK_COLLISION
    return [
        abi.clerk(C_, axes=[(abi.AXIS_MATERIAL, 2, 0.0, 0.0), (abi.AXIS_GROUP, 2, 0.0, 0.0)]),
        abi.clerk(C_, axes=[abi.cell_axis([0, 1]), (abi.AXIS_GROUP, 2, 0.0, 0.0)]),
        abi.clerk(C_, axes=[abi.cell_axis([0], undef_bin=True)]),
        abi.clerk(C_, axes=[(abi.AXIS_X, 8, -6.0, 6.0)]),
        abi.clerk(C_, axes=[abi.unstruct_axis(abi.AXIS_X, bounds)]),
    ]


def test_cell_and_unstructured_maps(oracle_mod):
    """cellMap (Tallies/TallyMaps/Maps1D/cellMap_class.f90) and unstructured grids
    (SharedModules/grid_class.f90 `unstruct`, binaryFloorIdxClosed): a cell map over cells that hold
    one material each equals the material map; the rest bin holds what the listed cells do not; an
    unstructured grid with the bounds of a lin grid bins like the lin grid."""
    p = problems.union_cell_slab()
    o = oracle_mod.Oracle(p, transport=abi.TRANSPORT_ST)
    clerks = _map_tallies()
    a = o.upload_tally(clerks)
    o.fixed_source_cycle(a, 20000, 4242)
    b = o.bins(a)[:, 1]
    mat, cell, rest, lin, uns = b[0:4], b[4:8], b[8:10], b[10:18], b[18:26]
    assert mat.min() > 0
    np.testing.assert_array_equal(cell, mat)
    # material axis fastest: mat = [m1 g1, m2 g1, m1 g2, m2 g2]; rest bin = the other cell
    np.testing.assert_allclose(rest, [mat[0] + mat[2], mat[1] + mat[3]], rtol=1e-10)
    np.testing.assert_allclose(uns, lin, rtol=1e-10)
    np.testing.assert_allclose(lin.sum(), mat.sum(), rtol=1e-10)


def test_unstructured_grid_search(oracle_mod):
    """grid%search on unstructured bounds: a value on an inner bound opens the bin above it, the
    last bound closes the last bin, values outside the bounds map to no bin."""
    p = problems.union_cell_slab()
    o = oracle_mod.Oracle(p, transport=abi.TRANSPORT_ST)
    bounds = np.array([-1.0, 0.0, 0.5, 2.0])
    for v, want in [(-1.0, 1), (-0.5, 1), (0.0, 2), (0.49, 2), (0.5, 3), (2.0, 3), (2.5, 0), (-1.5, 0)]:
        assert o.grid_search(bounds, v) == want, v


def test_rotated_universe_enter_golden(oracle_mod):
    """universe%enter with `rotation (90 90 90)` and `origin (2 0 0)` (the axis map x -> z,
    y -> -y, z -> x): local positions, directions and cells as SCONE's cellUniverse test states them
    (Geometry/Universes/Tests/cellUniverse_test.f90:28-34,150-200)."""
    gb = problems.GeometryBuilder()
    box = gb.surface(abi.BOX, 0.0, 0.0, 0.0, 20.0, 20.0, 20.0)
    s1 = gb.surface(abi.SPHERE, 0.0, 0.0, 0.0, 2.0)
    s2 = gb.surface(abi.SPHERE, 4.0, 0.0, 0.0, 1.0)
    c1 = gb.cell([-(s1 + 1)])
    c2 = gb.cell([s1 + 1, s2 + 1])
    uni = gb.cell_universe([c1, c2], [1, 2], origin=(2.0, 0.0, 0.0))
    gb.rotate(uni, (90.0, 90.0, 90.0))
    gb.root_universe(box, problems.uni_fill(uni), bc=[abi.BC_VACUUM] * 6)
    o = oracle_mod.Oracle(problems.Problem(gb.arrays(), None))
    cases = [((0.0, 0.0, 3.0), (0.0, 0.0, 1.0), (1.0, 0.0, 0.0), (1.0, 0.0, 0.0), 1),
             ((2.0, 0.0, 1.0), (0.0, 1.0, 0.0), (-1.0, 0.0, 2.0), (0.0, -1.0, 0.0), 2),
             ((0.0, 0.0, 6.5), (1.0, 0.0, 0.0), (4.5, 0.0, 0.0), (0.0, 0.0, 1.0), 3)]
    for r, u, r_ref, u_ref, local in cases:
        o.coords_init(r, u)
        o.coords_place()
        rl, ul, info = o.coords_get(1)
        np.testing.assert_allclose(rl, r_ref, rtol=0, atol=1e-12)
        np.testing.assert_allclose(ul, u_ref, rtol=0, atol=1e-12)
        assert info["local"] == local


def test_rotation_matrix_rejections(oracle_mod):
    gb = problems.GeometryBuilder()
    box = gb.surface(abi.BOX, 0.0, 0.0, 0.0, 5.0, 5.0, 5.0)
    c = gb.cell([-(box + 1)])
    uni = gb.cell_universe([c], [1])
    gb.rotate(uni, (0.0, 200.0, 0.0))                             # theta outside [0, 180]
    gb.root_universe(box, problems.uni_fill(uni), bc=[abi.BC_VACUUM] * 6)
    with pytest.raises(Exception, match="rotation"):
        oracle_mod.Oracle(problems.Problem(gb.arrays(), None))


def test_rotated_pins_runs_and_rotation_matters(oracle_mod):
    """The rotated-universe problem transports; turning the pin universe changes its tallies."""
    p = problems.rotated_pins()
    o = oracle_mod.Oracle(p, transport=abi.TRANSPORT_ST)
    a = o.upload_tally(p.tallies["flux"])
    o.fixed_source_cycle(a, 5000, 1357)
    b1 = o.bins(a)[:, 1]
    g = dict(p.geometry)
    g["uni_rot"] = np.zeros_like(g["uni_rot"])
    q = problems.Problem(g, p.mg, source=p.source, tallies=p.tallies)
    o2 = oracle_mod.Oracle(q, transport=abi.TRANSPORT_ST)
    a2 = o2.upload_tally(q.tallies["flux"])
    o2.fixed_source_cycle(a2, 5000, 1357)
    b2 = o2.bins(a2)[:, 1]
    assert b1[:6].min() > 0
    assert not np.allclose(b1, b2)


def _ww_sphere():
    """A 2-group homogeneous sphere (radius 6 cm) and weight windows over x that rise toward the
    centre: particles moving out split, particles moving in are rouletted."""
    rng = np.random.default_rng(5)
    p = problems.fixed_source_problem(rng, 2, "sphere", radius=6.0)
    x = np.linspace(-6.0, 6.0, 13)
    centres = 0.5 * (x[1:] + x[:-1])
    lower = 0.4 / (1.0 + np.abs(centres))
    upper = 5.0 * lower
    desc = abi.collision(abi.COLL_IMP, ww_axes=[(abi.AXIS_X, 12, -6.0, 6.0)], ww_lower=lower, ww_upper=upper,
                         ww_const_survival=2.5, buffer_depth=64)
    return p, desc


def test_weight_windows_mg_unbiased(oracle_mod):
    """neutronMGimp with weight windows (weightWindowsField: split above wUpper, roulette below
    wLower to wLower * constSurvival) leaves the flux estimate unbiased against neutronMGstd."""
    p, desc = _ww_sphere()
    n = 20000
    res = {}
    for imp in (False, True):
        o = oracle_mod.Oracle(p, transport=abi.TRANSPORT_ST)
        if imp:
            o.set_collision(desc)
        a = o.upload_tally(p.tallies["flux"])
        o.fixed_source_cycle(a, n, 2024)
        res[imp] = o.bins(a)[:, 1]
    std, ww = res[False], res[True]
    assert std.min() > 0
    np.testing.assert_allclose(ww, std, rtol=0.05)
    assert not np.allclose(ww, std, rtol=1e-9)                 # the game did act


def test_ce_implicit_absorption_roulette_unbiased(oracle_mod):
    """neutronCEimp with implicit absorption, roulette and splitting: the flux tally agrees with
    neutronCEstd within statistics on the 3-layer CE slab."""
    p = problems.ce_slab_3layer(points=(2000, 4000))
    n = 4000
    res = {}
    for imp in (False, True):
        o = oracle_mod.Oracle(p, transport=abi.TRANSPORT_DT)
        if imp:
            o.set_collision(abi.collision(abi.COLL_IMP, imp_abs=True, roulette=True, split=True,
                                          min_wgt=0.25, max_wgt=1.25, av_wgt=0.5))
        a = o.upload_tally(p.tallies["flux"])
        o.fixed_source_cycle(a, n, 777)
        res[imp] = o.bins(a)[:, 1]
    std, imp = res[False], res[True]
    ok = std > 0.05 * std.max()
    np.testing.assert_allclose(imp[ok].sum(), std[ok].sum(), rtol=0.05)


def test_collision_options_rejected(oracle_mod):
    p, _ = _ww_sphere()
    o = oracle_mod.Oracle(p)
    with pytest.raises(Exception, match="roulette"):
        o.set_collision(abi.collision(abi.COLL_IMP, imp_abs=True))
    with pytest.raises(Exception, match="twice"):
        o.set_collision(abi.collision(abi.COLL_IMP, split=True, min_wgt=1.0, max_wgt=1.5))


def test_map_golden_vectors(oracle_mod):
    """spaceMap, energyMap and cellMap against the known answers of SCONE's own map tests
    (Tallies/TallyMaps/Maps1D/Tests/spaceMap_test.f90:88-140, energyMap_test.f90:25-181,
    cellMap_test.f90:28-128)."""
    gb = problems.GeometryBuilder()
    box = gb.surface(abi.BOX, 0.0, 0.0, 0.0, 5.0, 5.0, 5.0)
    z = [gb.surface(abi.ZPLANE, v) for v in (-1.3, 0.0, 1.0)]
    cells = [gb.cell([-(z[0] + 1), z[2] + 1]), gb.cell([-(z[0] + 1), -(z[2] + 1), z[1] + 1]),
             gb.cell([-(z[1] + 1), z[0] + 1]), gb.cell([-(z[0] + 1)])]   # the test's ids 2, 1, 5, 3
    uni = gb.cell_universe(cells, [1, 1, 1, 1])
    gb.root_universe(box, problems.uni_fill(uni), bc=[abi.BC_VACUUM] * 6)
    o = oracle_mod.Oracle(problems.Problem(gb.arrays(), None))
    # spaceMap: lin -10..10 in 20 bins, unstructured on [-10, -8, ..., 10]
    div = [-10.0, -8.0, -6.0, -4.0, -2.0, 0.0, 2.0, 4.0, 6.0, 8.0, 10.0]
    for ax in (abi.AXIS_X, abi.AXIS_Y, abi.AXIS_Z):
        for pos, lin, uns in ((0.5, 11, 6), (-10.1, 0, 0)):
            r = [0.0, 0.0, 0.0]
            r[ax - abi.AXIS_X] = pos
            assert o.map_point([(ax, 20, -10.0, 10.0)], r=r) == lin
            assert o.map_point([abi.unstruct_axis(ax, div)], r=r) == uns
    # energyMap: lin 0.01..10 (20), log 1e-7..10 (20), unstructured (25 bins)
    E_lin = [7.5774, 9.3652, 3.9223, 6.5548, 1.7119, 20.0]
    E_log = [0.0445008907555061, 1.79747463687278e-07, 1.64204055725811e-05, 2.34083673923110e-07,
             5.98486350302033e-07, 20.0]
    E_uns = [0.0761191517392624, 0.00217742635754091, 6.38548311340975e-08, 2.52734532533842,
             2.59031729968032e-11, 20.0]
    grid = [1e-11, 3e-8, 5.8e-8, 1.4e-7, 2.8e-7, 3.5e-7, 6.25e-7, 9.72e-7, 1.02e-6, 1.097e-6, 1.15e-6,
            1.855e-6, 4e-6, 9.877e-6, 1.5968e-5, 1.48728e-4, 5.53e-3, 9.118e-3, 0.111, 0.5, 0.821, 1.353,
            2.231, 3.679, 6.0655, 10.0]
    lin_ax = (abi.AXIS_ENERGY, 20, 0.01, 10.0, abi.GRID_LIN)
    log_ax = (abi.AXIS_ENERGY, 20, 1.0e-7, 10.0, abi.GRID_LOG)
    uns_ax = abi.unstruct_axis(abi.AXIS_ENERGY, grid)
    for ax, Es, want in ((lin_ax, E_lin, [16, 19, 8, 14, 4, 0]), (log_ax, E_log, [15, 1, 6, 1, 2, 0]),
                         (uns_ax, E_uns, [18, 16, 3, 23, 1, 0])):
        assert [o.map_point([ax], E=e, mg=False) for e in Es] == want
        assert o.map_point([ax], E=Es[0], mg=True) == 0              # MG particles map to no bin
    # cellMap over cells (2 5 3) by id, i.e. indices 0, 2, 3: cellIdx 1..4, and 0 (in no cell)
    no_undef = abi.cell_axis([0, 2, 3])
    undef = abi.cell_axis([0, 2, 3], undef_bin=True)
    assert [o.map_point([no_undef], cell=c) for c in (1, 2, 3, 4, 0)] == [1, 0, 2, 3, 0]
    assert [o.map_point([undef], cell=c) for c in (1, 2, 3, 4, 0)] == [1, 4, 2, 3, 4]


def test_multimap_golden_vectors(oracle_mod):
    """multiMap of three unstructured spaceMaps, first axis fastest: the known answers of SCONE's
    multiMap test (Tallies/TallyMaps/Tests/multiMap_test.f90:26-85)."""
    gb = problems.GeometryBuilder()
    box = gb.surface(abi.BOX, 0.0, 0.0, 0.0, 100.0, 100.0, 100.0)
    gb.root_universe(box, 1, bc=[abi.BC_VACUUM] * 6)
    o = oracle_mod.Oracle(problems.Problem(gb.arrays(), None))
    axes = [abi.unstruct_axis(abi.AXIS_X, [0.0, 1.0, 2.0]), abi.unstruct_axis(abi.AXIS_Y, [0.0, 2.0, 4.0, 6.0]),
            abi.unstruct_axis(abi.AXIS_Z, [0.0, 3.0, 6.0])]
    assert [abi.axis_bins(a) for a in axes] == [2, 3, 2]
    for r, want in (((0.1, 0.1, 0.1), 1), ((1.1, 5.1, 5.1), 12), ((1.1, 3.1, 2.1), 4),
                    ((-1.1, 5.1, 5.1), 0), ((1.1, 50.1, 5.1), 0), ((1.1, 5.1, -5.1), 0)):
        assert o.map_point(axes, r=r) == want, r


def test_openmp_eigen_cycle_equals_serial(oracle_mod):
    """The CPU baseline's eigenvalue cycle (OpenMP over histories, thread-private score memory, sites
    ordered by brood) gives the serial oracle's banks, master RNG state and k (tally sums to
    round-off: they are added in another order)."""
    p = problems.lattice_17x17_7g()
    res = []
    for omp in (False, True):
        o = oracle_mod.Oracle(p, transport=abi.TRANSPORT_DT)
        inact, act = o.upload_tally([]), o.upload_tally(p.tallies["mesh"])
        ia = o.upload_tally([abi.clerk(abi.CLERK_KEFF_ANALOG)])
        aa = o.upload_tally([abi.clerk(abi.CLERK_KEFF_IMPLICIT)])
        o.attach_tally(inact, ia)
        o.attach_tally(act, aa)
        o.eigen_init(5000, 0x5C3A84C9)
        ks = []
        for c in range(5):
            adm, atch = (inact, ia) if c < 2 else (act, aa)
            ks.append((o.eigen_cycle_omp(adm, atch, 4) if omp else o.eigen_cycle(adm, atch)).k_new)
        b, pop = o.eigen_bank(5000)
        res.append((np.array(ks), o.eigen_state()[0], b["r"][:pop].copy(), b["G"][:pop].copy(), o.bins(act)))
    (k0, m0, r0, g0, b0), (k1, m1, r1, g1, b1) = res
    np.testing.assert_allclose(k1, k0, rtol=1e-11)
    assert m0 == m1
    assert np.array_equal(r0, r1) and np.array_equal(g0, g1)
    np.testing.assert_allclose(b1, b0, rtol=1e-10, atol=1e-300)
