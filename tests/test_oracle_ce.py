"""Continuous-energy part of the CPU oracle, pinned to SCONE's own test values where they exist.

* H-1 (1001.03c) cross sections at the energies of aceNeutronDatabase_iTest.f90:183-197, from the
  ESZ block of IntegrationTestFiles/1001JEF311.ace (committed as a fixture);
* the floor-index rule of binaryFloorIdxClosed_Real (genericProcedures.f90:132-166);
* the unionised majorant bounds every active material's total (aceNeutronDatabase initMajorant);
* asymptoticScatter against its closed form, and the free-gas kernel (targetVelocity_constXS) by
  the equilibrium spectrum it must reach in a weakly absorbing infinite medium;
* ST and DT agree on the synthetic 3-layer slab, and the boundary planes see outward current only.
"""
import json
import math
import os

import numpy as np
import pytest

from scone_gb300 import abi, problems

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "scone_golden.json")))


def h1_problem():
    g = GOLD["h1_ace"]
    e = np.array(g["e"])
    xs = np.zeros((len(e), 4))
    xs[:, 0], xs[:, 1], xs[:, 3] = g["total"], g["elastic"], g["absorption"]
    ce = problems.ce_data([dict(e=e, xs=xs, A=g["aw"], kT=g["tz"])], [[(0, 1.0)]])
    gb = problems.GeometryBuilder()
    box = gb.surface(abi.BOX, 0.0, 0.0, 0.0, 1.0, 1.0, 1.0)
    gb.root_universe(box, 1, bc=[abi.BC_REFLECTIVE] * 6)
    return problems.Problem(gb.arrays(), None, ce=ce), e, xs


def test_h1_micro_xs_golden(oracle_mod):
    p, _, _ = h1_problem()
    o = oracle_mod.Oracle(p)
    TOL = 1.0e-6                                            # aceNeutronDatabase_iTest.f90:81
    assert abs(1.0 - 20.765855864000002 / o.ce_micro(0, 1.1e-6)[0]) < TOL
    m = o.ce_micro(0, 5.6e-3)
    assert m[2] == 0.0                                      # no inelastic
    assert abs(1.0 - 19.731020820000000 / m[0]) < TOL
    assert abs(1.0 - 19.730326000000000 / m[1]) < TOL
    assert abs(1.0 - 6.948036800000000e-04 / m[3]) < TOL


def test_floor_index_rule(oracle_mod):
    p, e, xs = h1_problem()
    o = oracle_mod.Oracle(p)
    for k in (0, 1, 17, 200, len(e) - 2):
        assert np.array_equal(o.ce_micro(0, e[k]), xs[k])        # f = 0 at a grid point
    assert np.array_equal(o.ce_micro(0, e[-1]), xs[-1])           # a(N) -> N-1 with f = 1
    for bad in (e[0] * 0.5, e[-1] * 2.0):
        with pytest.raises(RuntimeError):
            o.ce_micro(0, bad)


def slab(scale=0.02):
    return problems.ce_slab_3layer(scale=scale)


def test_union_majorant_bounds_material_totals(oracle_mod):
    p = slab()
    o = oracle_mod.Oracle(p)
    n = o.ce_union_size()
    sizes = p.meta["grid_points"]
    assert max(sizes) <= n <= sum(sizes) + 1
    rng = np.random.default_rng(5)
    for E in np.exp(rng.uniform(np.log(1e-11), np.log(20.0), 3000)):
        maj = o.ce_majorant(E)
        tot = max(o.ce_mat_total(m, E) for m in (1, 2, 3))
        assert maj >= tot * (1.0 - 1e-12)
        assert maj <= tot * (1.0 + 1e-6) * (1 + 1e-9) or maj <= tot * 2.0   # linear between points
    for E in p.ce["e"][:50]:
        maj = o.ce_majorant(E)
        tot = max(o.ce_mat_total(m, E) for m in (1, 2, 3))
        assert maj == pytest.approx(tot * (1.0 + 1e-6), rel=1e-12)


def test_asymptotic_scatter_closed_form(oracle_mod):
    for A in (1.0, 2.0, 12.0, 59.5):
        alpha = ((A - 1.0) / (A + 1.0)) ** 2
        E, mu = oracle_mod.asymptotic_scatter(1.0, 1.0, A)
        assert E == pytest.approx(1.0) and mu == pytest.approx(1.0)
        E, mu = oracle_mod.asymptotic_scatter(2.0, -1.0, A)
        assert E == pytest.approx(2.0 * alpha, abs=1e-15)
        for m in (-0.5, 0.0, 0.7):
            E, mu = oracle_mod.asymptotic_scatter(1.0, m, A)
            assert E == pytest.approx((1.0 + A * A + 2.0 * A * m) / (A + 1.0) ** 2)
            assert mu == pytest.approx(min(1.0, (1.0 + A * m) / math.sqrt(1.0 + A * A + 2.0 * A * m)))


def test_target_velocity_draws_and_scale(oracle_mod):
    kT, A = 2.53e-8, 1.0
    d = np.array([0.0, 0.0, 1.0])
    s = 12345
    v2 = []
    for _ in range(4000):
        v, s = oracle_mod.target_velocity(kT, d, A, kT, s)
        v2.append(v @ v)
    # E_t = A V_t^2 is the target's kinetic energy in units of kT... its mean over the
    # relative-speed-weighted Maxwellian lies between 1.5 kT (plain) and 2.5 kT
    m = np.mean(v2) * A / kT
    assert 1.5 < m < 2.6


def test_free_gas_reaches_equilibrium(oracle_mod):
    """With constant tabulated cross sections the free-gas kernel balances the collision density
    g(E) * E exp(-E/kT), g the Doppler factor of the constant-XS kernel (the
    dopplerCorrectionFactor of scatteringKernels_func.f90:248-270), so a collision estimator with
    constant Sigma reads phi(E) ~ g(E) E exp(-E/kT)."""
    from scipy.special import erf
    kT = problems.KT_293K
    p = problems.ce_infinite_medium(A=1.0, sigma_s=20.0, sigma_c=0.1, kT=kT)
    o = oracle_mod.Oracle(p, transport=abi.TRANSPORT_DT)
    nb = 40
    lo, hi = 1e-3 * kT, 30.0 * kT
    a = o.upload_tally([abi.clerk(abi.CLERK_COLLISION, axes=[(abi.AXIS_ENERGY, nb, lo, hi)])])
    bank = o.generate_source(2024, 3000)
    o.transport_bank(a, bank, 777)
    o.tally_cycle_end(a, 0.0)
    phi = o.bins(a)[:, 1]
    edges = np.geomspace(lo, hi, nb + 1) / kT

    def dens(x):
        al = np.sqrt(x)
        g = (1.0 + 0.5 / al**2) * erf(al) + np.exp(-al**2) / (al * np.sqrt(np.pi))
        return g * x * np.exp(-x)
    ref = np.array([np.trapezoid(dens(np.geomspace(edges[i], edges[i + 1], 64)),
                                 np.geomspace(edges[i], edges[i + 1], 64)) for i in range(nb)])
    phi_n, ref_n = phi / phi.sum(), ref / ref.sum()
    big = ref_n > 0.02
    assert np.max(np.abs(phi_n[big] / ref_n[big] - 1.0)) < 0.08
    mid = np.sqrt(edges[1:] * edges[:-1])
    assert np.sum(phi_n * mid) == pytest.approx(np.sum(ref_n * mid), rel=0.04)


def run_slab(oracle_mod, transport, n=500, batches=8):
    p = slab()
    o = oracle_mod.Oracle(p, transport=transport)
    a = o.upload_tally(p.tallies["current"])
    b = o.upload_tally([abi.clerk(abi.CLERK_COLLISION, axes=[(abi.AXIS_MATERIAL, 3, 0.0, 0.0)])])
    o.attach_tally(a, b)
    master = 4242
    for _ in range(batches):
        master, st = o.fixed_source_cycle(a, n, master)
    cur = o.bins(a)[:, 1].reshape(4, 200, 2)
    fb = o.bins(b)
    N = batches
    mean = fb[:, 1] / N
    sd = np.sqrt(np.maximum(fb[:, 2] / (N * (N - 1)) - mean**2 / (N - 1), 0.0))
    return cur, mean, sd, st


def test_slab_st_dt_agree_and_boundary_currents(oracle_mod):
    cs, ms, ss, sts = run_slab(oracle_mod, abi.TRANSPORT_ST)
    cd, md, sd, std = run_slab(oracle_mod, abi.TRANSPORT_DT)
    assert sts.n_collisions > 0 and std.n_collisions > 0
    for c in (cs, cd):
        assert c[0, :, 1].sum() == 0.0 and c[3, :, 0].sum() == 0.0   # nothing enters from vacuum
        assert c[0, :, 0].sum() > 0 and c[3, :, 1].sum() > 0
    # crossings per plane and direction: ST vs DT within 5 sigma (counts as Poisson, inflated 2x
    # for repeated crossings by one history)
    a, b = cs.sum(axis=1), cd.sum(axis=1)
    z = (a - b) / np.sqrt(2.0 * np.maximum(a + b, 1.0))
    assert np.all(np.abs(z) < 5.0), z
    # flux per material from batch statistics
    z = (ms - md) / np.sqrt(ss**2 + sd**2)
    assert np.all(np.abs(z) < 4.0), z
