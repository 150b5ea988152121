"""GPU parity for continuous-energy transport (neutronCEstd, aceNeutronDatabase lookups) against the
CPU oracle.

All-FP64 form: per-history bit-level agreement (real collisions and the RNG state at the end of
every history) and tallies equal to round-off (relative 1e-10; the surface-current clerk counts unit
weights, so its bins are exact).  Mixed form: statistical agreement with the FP64 form.
"""
import numpy as np
import pytest

from scone_gb300 import abi, problems

pytestmark = pytest.mark.gpu

SEED = 0x5C3A84C9
FORMS = [abi.FORM_EVENT, abi.FORM_HISTORY]
TRANSPORTS = [abi.TRANSPORT_ST, abi.TRANSPORT_DT, abi.TRANSPORT_ST_NOCACHE]


@pytest.fixture(scope="module")
def gpu_mod():
    from scone_gb300 import gpu
    gpu.load()
    return gpu


@pytest.fixture(scope="module")
def slab_small():
    return problems.ce_slab_3layer(scale=0.05)


@pytest.fixture(scope="module")
def slab_full():
    return problems.ce_slab_3layer()


def run_pair(gpu, orl, prob, transport, form, n, precision=abi.PREC_FP64):
    g = gpu.TransportOperatorGPU(prob, precision=precision, transport=transport, max_bank=max(n, 1024),
                                 record_histories=True, form=form)
    o = orl.Oracle(prob, transport=transport)
    bank = o.generate_source(SEED, n)
    res = []
    for t in (g, o):
        a = t.upload_tally(prob.tallies["current"])
        b = t.upload_tally(prob.tallies["flux"])
        t.attach_tally(a, b)
        _, st = t.transport_bank(a, bank, 987654321)
        t.tally_cycle_end(a, float(n))
        res.append((t, st, t.bins(a), t.bins(b)))
    return res


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("transport", TRANSPORTS)
def test_ce_slab_fp64_history_parity(gpu_mod, oracle_mod, slab_small, transport, form):
    n = 6000
    (g, sg, cg, fg), (o, so, co, fo) = run_pair(gpu_mod, oracle_mod, slab_small, transport, form, n)
    hg, rg = g.history_records(n)
    ho, ro = o.history_records(n)
    assert np.array_equal(hg, ho)
    assert np.array_equal(rg, ro)
    assert sg.n_events == so.n_events and sg.n_collisions == so.n_collisions
    assert np.array_equal(cg, co)                       # unit-weight crossings: exact
    np.testing.assert_allclose(fg, fo, rtol=1e-10, atol=0)


@pytest.mark.parametrize("transport", [abi.TRANSPORT_ST, abi.TRANSPORT_DT])
def test_ce_full_grids_fp64_parity(gpu_mod, oracle_mod, slab_full, transport):
    """Full-size grids (2e4-1e5 points per nuclide, ~5e5-point union grid): hashed searches give
    the reference's floor indices exactly."""
    n = 3000
    (g, sg, cg, fg), (o, so, co, fo) = run_pair(gpu_mod, oracle_mod, slab_full, transport, abi.FORM_HISTORY, n)
    hg, rg = g.history_records(n)
    ho, ro = o.history_records(n)
    assert np.array_equal(hg, ho)
    assert np.array_equal(rg, ro)
    assert np.array_equal(cg, co)
    np.testing.assert_allclose(fg, fo, rtol=1e-10, atol=0)


@pytest.mark.parametrize("transport", [abi.TRANSPORT_ST, abi.TRANSPORT_DT])
def test_ce_free_gas_fp64_parity(gpu_mod, oracle_mod, transport):
    """A = 1 scatterer near thermal energies: every collision samples a moving target."""
    p = problems.ce_infinite_medium(A=1.0, sigma_s=20.0, sigma_c=0.4)
    g = gpu_mod.TransportOperatorGPU(p, precision=abi.PREC_FP64, transport=transport, max_bank=4096,
                                     record_histories=True, form=abi.FORM_HISTORY)
    o = oracle_mod.Oracle(p, transport=transport)
    ax = [(abi.AXIS_ENERGY, 40, 1e-3 * problems.KT_293K, 30 * problems.KT_293K)]
    n = 2000
    bank = o.generate_source(SEED, n)
    out = []
    for t in (g, o):
        a = t.upload_tally([abi.clerk(abi.CLERK_COLLISION, axes=ax)])
        t.transport_bank(a, bank, 4321)
        t.tally_cycle_end(a, float(n))
        out.append((t.history_records(n), t.bins(a)))
    (hg, rg), bg = out[0]
    (ho, ro), bo = out[1]
    assert np.array_equal(hg, ho) and np.array_equal(rg, ro)
    np.testing.assert_allclose(bg, bo, rtol=1e-10, atol=0)


def test_ce_fixed_source_cycles_on_device(gpu_mod, oracle_mod, slab_small):
    """sg_fixed_source_cycle: point source with E sampled on the device, batches closed there."""
    p = slab_small
    g = gpu_mod.TransportOperatorGPU(p, precision=abi.PREC_FP64, transport=abi.TRANSPORT_DT, max_bank=4096,
                                     form=abi.FORM_HISTORY)
    o = oracle_mod.Oracle(p, transport=abi.TRANSPORT_DT)
    res = []
    for t in (g, o):
        a = t.upload_tally(p.tallies["current"])
        m = SEED
        for _ in range(3):
            m, _ = t.fixed_source_cycle(a, 2000, m)
        res.append((m, t.bins(a)))
    assert res[0][0] == res[1][0]
    assert np.array_equal(res[0][1], res[1][1])


def test_ce_mixed_matches_fp64_statistically(gpu_mod, slab_full):
    """Mixed form (FP32 tables and kinematics) against the FP64 form on the full slab: per-plane
    current totals and per-material flux from 10 batches agree within 4 sigma."""
    p = slab_full
    out = {}
    for prec in (abi.PREC_FP64, abi.PREC_MIXED):
        g = gpu_mod.TransportOperatorGPU(p, precision=prec, transport=abi.TRANSPORT_DT, max_bank=1 << 16,
                                         form=abi.FORM_HISTORY)
        a = g.upload_tally(p.tallies["current"])
        b = g.upload_tally([abi.clerk(abi.CLERK_COLLISION, axes=[(abi.AXIS_MATERIAL, 3, 0.0, 0.0)])])
        g.attach_tally(a, b)
        m = 11 if prec == abi.PREC_FP64 else 13
        N = 10
        for _ in range(N):
            m, _ = g.fixed_source_cycle(a, 20000, m)
        fb = g.bins(b)
        mean = fb[:, 1] / N
        sd = np.sqrt(np.maximum(fb[:, 2] / (N * (N - 1)) - mean**2 / (N - 1), 0.0))
        cb = g.bins(a)
        cm = cb[:, 1].reshape(4, 200, 2).sum(axis=1) / N
        out[prec] = (mean, sd, cm)
    (m64, s64, c64), (mmx, smx, cmx) = out[abi.PREC_FP64], out[abi.PREC_MIXED]
    z = (m64 - mmx) / np.sqrt(s64**2 + smx**2)
    assert np.all(np.abs(z) < 4.0), z
    z = (c64 - cmx) * N / np.sqrt(2.0 * np.maximum((c64 + cmx) * N, 1.0))   # counts, 2x for re-crossings
    assert np.all(np.abs(z) < 5.0), z
    assert np.all(cmx[c64 == 0] == 0)


def _history_parity(gpu_mod, oracle_mod, p, transport, n, tally, master=2468):
    g = gpu_mod.TransportOperatorGPU(p, precision=abi.PREC_FP64, transport=transport, max_bank=max(n, 4096),
                                     record_histories=True, form=abi.FORM_HISTORY)
    o = oracle_mod.Oracle(p, transport=transport)
    bank = o.generate_source(SEED, n)
    out = []
    for t in (g, o):
        a = t.upload_tally(tally)
        _, st = t.transport_bank(a, bank, master)
        t.tally_cycle_end(a, float(n))
        out.append((t.history_records(n), t.bins(a), st))
    ((hg, rg), bg, sg), ((ho, ro), bo, so) = out
    assert np.array_equal(hg, ho) and np.array_equal(rg, ro)
    assert sg.n_events == so.n_events
    np.testing.assert_allclose(bg, bo, rtol=1e-10, atol=0)
    g.close()
    return bg


@pytest.mark.parametrize("transport", [abi.TRANSPORT_ST, abi.TRANSPORT_DT])
def test_ace_tables_drive_the_ce_kernels(gpu_mod, oracle_mod, transport, tmp_path):
    """The CE slab's ten nuclides written as ACE type-1 tables into one library file, read back as
    aceNeutronDatabase reads them (aceNeutronNuclide%init, aceNeutronNuclide_class.f90:737) and
    uploaded: GPU histories equal the oracle's on the same tables, per history, FP64."""
    from scone_gb300 import ace
    slab = problems.ce_slab_3layer(scale=0.05)
    ce = slab.ce
    path = str(tmp_path / "slab.ace")
    nucs = []
    for k in range(len(ce["A"])):
        a, b = int(ce["nuc_ptr"][k]), int(ce["nuc_ptr"][k + 1])
        e, xs = ce["e"][a:b], ce["xs"][a:b]
        line = ace.write_table(path, f"{1001 + 1000 * k}.90c", float(ce["A"][k]), float(ce["kT"][k]), e, xs[:, 0],
                               xs[:, 1], xs[:, 3], ext_mode="a")
        r = ace.nuclide(path, line)
        np.testing.assert_allclose(r["xs"], xs, rtol=1e-10, atol=0)
        nucs.append(dict(e=r["e"], xs=r["xs"], A=r["A"], kT=r["kT"]))
    mats = [[(int(ce["mat_nuc"][j]), float(ce["mat_dens"][j])) for j in range(ce["mat_ptr"][m], ce["mat_ptr"][m + 1])]
            for m in range(len(ce["mat_ptr"]) - 1)]
    p = problems.Problem(slab.geometry, None, ce=problems.ce_data(nucs, mats), source=slab.source,
                         tallies=slab.tallies)
    bins = _history_parity(gpu_mod, oracle_mod, p, transport, 4000, p.tallies["current"])
    assert bins[:, 1].sum() > 0


@pytest.mark.parametrize("transport", [abi.TRANSPORT_ST, abi.TRANSPORT_DT])
def test_scone_h1_table_on_the_device(gpu_mod, oracle_mod, transport):
    """SCONE's own H-1 table (IntegrationTestFiles/1001JEF311.ace, 1001.03c, committed under
    tests/golden) uploaded to the device: hydrogen in an all-reflective box, a 1 MeV source slowing
    down to thermal energies through free-gas scattering (A < 1 always samples a moving target,
    neutronCEstd_class.f90:340-384): per-history FP64 parity with the oracle and equal spectra."""
    import os
    from scone_gb300 import ace
    r = ace.nuclide(os.path.join(os.path.dirname(__file__), "golden", "scone_h1_1001_03c.ace"))
    assert r["zaid"] == "1001.03c" and r["A"] < 1.0
    ce = problems.ce_data([dict(e=r["e"], xs=r["xs"], A=r["A"], kT=r["kT"])], [[(0, 0.0669)]])
    gb = problems.GeometryBuilder()
    box = gb.surface(abi.BOX, 0.0, 0.0, 0.0, 50.0, 50.0, 50.0)
    gb.root_universe(box, 1, bc=[abi.BC_REFLECTIVE] * 6)
    ax = [(abi.AXIS_ENERGY, 60, 1.0e-11, 2.0)]
    p = problems.Problem(gb.arrays(), None, ce=ce, source=dict(r=(0.0, 0.0, 0.0), E=1.0))
    bins = _history_parity(gpu_mod, oracle_mod, p, transport, 1500, [abi.clerk(abi.CLERK_COLLISION, axes=ax)])
    assert (bins[:, 1] > 0).sum() > 30                         # the spectrum spans the slowing-down range


@pytest.mark.parametrize("where", ["top", "repeated"])
@pytest.mark.parametrize("transport", [abi.TRANSPORT_ST, abi.TRANSPORT_DT])
def test_ce_lookup_edges_fp64_parity(gpu_mod, oracle_mod, transport, where):
    """The grid lookups at their edges, per history against the oracle: nuclide 0 gets a repeated
    interior grid point (a step in its cross sections), and every history starts exactly on a grid
    point -- the top of every grid (20 MeV: binaryFloorIdxClosed's closed end takes the last
    interval) or the repeated point (the floor index is the later of the two)."""
    p = problems.ce_slab_3layer(scale=0.05)
    ce = dict(p.ce)
    ptr, e, xs = np.asarray(ce["nuc_ptr"]), np.asarray(ce["e"]), np.asarray(ce["xs"])
    k = int(ptr[1]) // 2
    ce["e"] = np.insert(e, k + 1, e[k])
    ce["xs"] = np.insert(xs, k + 1, xs[k] * 1.5, axis=0)
    ptr2 = ptr.copy()
    ptr2[1:] += 1
    ce["nuc_ptr"] = ptr2
    E = 20.0 if where == "top" else float(e[k])
    q = problems.Problem(p.geometry, None, name="ce_slab_edges", ce=ce, source=dict(r=(15.0, 0.0, 0.0), E=E),
                         tallies=p.tallies)
    _history_parity(gpu_mod, oracle_mod, q, transport, 3000, q.tallies["current"])
