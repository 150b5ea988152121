"""GPU parity: libsconegpu against the CPU oracle (a restatement of SCONE's algorithm).

All-FP64 form: bit-level agreement per history (number of real collisions and the RNG state at the
end of every history, i.e. every draw in SCONE's order), identical fission banks, and tallies equal
to round-off (scores are summed in a different order: relative tolerance 1e-10).
Mixed form: statistical agreement with the FP64 form (k within 4 sigma, flux z-scores).
"""
import numpy as np
import pytest

from scone_gb300 import abi, problems

pytestmark = pytest.mark.gpu

SEED = 0x5C3A84C9


@pytest.fixture(scope="module")
def gpu_mod():
    from scone_gb300 import gpu
    gpu.load()
    return gpu


FORMS = [abi.FORM_EVENT, abi.FORM_HISTORY]


def make_pair(gpu, orl, prob, transport=abi.TRANSPORT_ST, precision=abi.PREC_FP64, max_bank=1 << 18,
              form=abi.FORM_EVENT, ht_cutoff=0.0):
    g = gpu.TransportOperatorGPU(prob, precision=precision, transport=transport, max_bank=max_bank,
                                 record_histories=True, form=form, ht_cutoff=ht_cutoff)
    o = orl.Oracle(prob, transport=transport, ht_cutoff=ht_cutoff)
    return g, o


ALL_TRANSPORTS = [abi.TRANSPORT_ST, abi.TRANSPORT_DT, abi.TRANSPORT_ST_NOCACHE, abi.TRANSPORT_HT,
                  abi.TRANSPORT_HT_NOCACHE]


def test_point_source_bank_bitexact(gpu_mod, oracle_mod):
    p = problems.infinite_medium_2g()
    g, o = make_pair(gpu_mod, oracle_mod, p)
    bg = g.generate_source(SEED, 5000)
    bo = o.generate_source(SEED, 5000)
    for k in ("G", "wgt"):
        assert np.array_equal(bg[k], bo[k]), k
    assert np.array_equal(bg["r"], bo["r"])
    np.testing.assert_allclose(bg["dir"], bo["dir"], rtol=0, atol=1e-15)


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("transport", ALL_TRANSPORTS)
def test_infinite_medium_fp64_history_parity(gpu_mod, oracle_mod, transport, form):
    p = problems.infinite_medium_2g()
    g, o = make_pair(gpu_mod, oracle_mod, p, transport, form=form)
    n = 20000
    bank = o.generate_source(SEED, n)
    ag = g.upload_tally(p.tallies["flux"])
    ao = o.upload_tally(p.tallies["flux"])
    master = 987654321
    _, sg = g.transport_bank(ag, bank, master)
    _, so = o.transport_bank(ao, bank, master)
    cg, rg = g.history_records(n)
    co, ro = o.history_records(n)
    assert np.array_equal(cg, co)
    assert np.array_equal(rg, ro)
    assert sg.n_events == so.n_events and sg.n_collisions == so.n_collisions
    for t in (g, o):
        t.tally_cycle_end(ag if t is g else ao, float(n))
    bg, bo = g.bins(ag), o.bins(ao)
    np.testing.assert_allclose(bg, bo, rtol=1e-10, atol=0)


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("transport,cutoff", [(t, 0.0) for t in ALL_TRANSPORTS] +
                         [(abi.TRANSPORT_HT, 0.5), (abi.TRANSPORT_HT, 0.3)])
def test_lattice_fp64_bank_parity(gpu_mod, oracle_mod, transport, cutoff, form):
    p = problems.lattice_17x17_7g()
    g, o = make_pair(gpu_mod, oracle_mod, p, transport, form=form, ht_cutoff=cutoff)
    n = 4000
    o.eigen_init(n, SEED)
    bank, pop = o.eigen_bank(n)
    assert pop == n
    ag = g.upload_tally(p.tallies["mesh"] + [abi.clerk(abi.CLERK_KEFF_IMPLICIT)])
    ao = o.upload_tally(p.tallies["mesh"] + [abi.clerk(abi.CLERK_KEFF_IMPLICIT)])
    master = 1122334455
    ng, sg = g.transport_bank(ag, bank, master, k_eff=1.05)
    no, so = o.transport_bank(ao, bank, master, k_eff=1.05)
    cg, rg = g.history_records(n)
    co, ro = o.history_records(n)
    assert np.array_equal(cg, co)
    assert np.array_equal(rg, ro)
    assert sg.n_next == so.n_next > 0
    m = so.n_next
    for k in ("G", "wgt", "brood_id"):
        assert np.array_equal(ng[k][:m], no[k][:m]), k
    # continuous values carry the <= 1 ulp log/sin/cos differences between CUDA and glibc
    np.testing.assert_allclose(ng["r"][:m], no["r"][:m], rtol=0, atol=1e-9)
    np.testing.assert_allclose(ng["dir"][:m], no["dir"][:m], rtol=0, atol=1e-12)
    g.tally_cycle_end(ag, float(m), 1.05)
    o.tally_cycle_end(ao, float(m), 1.05)
    np.testing.assert_allclose(g.bins(ag), o.bins(ao), rtol=1e-10, atol=1e-300)


def _eigen(t, p, pop, n_in, n_act):
    inact = t.upload_tally([])
    act = t.upload_tally(p.tallies["mesh"])
    ia = t.upload_tally([abi.clerk(abi.CLERK_KEFF_ANALOG)])
    aa = t.upload_tally([abi.clerk(abi.CLERK_KEFF_IMPLICIT)])
    t.attach_tally(inact, ia)
    t.attach_tally(act, aa)
    t.eigen_init(pop, SEED)
    ks = []
    for _ in range(n_in):
        ks.append(t.eigen_cycle(inact, ia).k_new)
    for _ in range(n_act):
        ks.append(t.eigen_cycle(act, aa).k_new)
    return np.array(ks), t.keff(aa), t.bins(act)


@pytest.mark.parametrize("form", FORMS)
def test_lattice_eigen_fp64_cycles(gpu_mod, oracle_mod, form):
    p = problems.lattice_17x17_7g()
    g, o = make_pair(gpu_mod, oracle_mod, p, form=form)
    kg, keg, bg = _eigen(g, p, 3000, 3, 3)
    ko, keo, bo = _eigen(o, p, 3000, 3, 3)
    np.testing.assert_allclose(kg, ko, rtol=1e-10)
    mg, _ = g.eigen_state()
    mo, _ = o.eigen_state()
    assert mg == mo
    bgk, _ = g.eigen_bank(3000)
    bok, _ = o.eigen_bank(3000)
    np.testing.assert_allclose(bgk["r"], bok["r"], rtol=0, atol=1e-9)
    np.testing.assert_allclose(bg, bo, rtol=1e-8, atol=1e-300)


@pytest.mark.parametrize("form,transport", [(abi.FORM_EVENT, abi.TRANSPORT_ST), (abi.FORM_HISTORY, abi.TRANSPORT_ST),
                                            (abi.FORM_HISTORY, abi.TRANSPORT_ST_NOCACHE),
                                            (abi.FORM_HISTORY, abi.TRANSPORT_DT)])
def test_lattice_mixed_vs_fp64_statistics(gpu_mod, form, transport):
    p = problems.lattice_17x17_7g()
    res = {}
    for prec in (abi.PREC_FP64, abi.PREC_MIXED):
        t = gpu_mod.TransportOperatorGPU(p, precision=prec, max_bank=1 << 19, form=form, transport=transport)
        ks, (k, sd), bins = _eigen(t, p, 100000, 5, 10)
        res[prec] = (k, sd, bins)
    k64, s64, b64 = res[abi.PREC_FP64]
    k32, s32, b32 = res[abi.PREC_MIXED]
    assert abs(k64 - k32) < 4.0 * np.hypot(s64, s32), (k64, s64, k32, s32)
    n = 10
    m64, m32 = b64[:, 1] / n, b32[:, 1] / n
    v64 = (b64[:, 2] / n - m64 ** 2) / (n - 1)
    v32 = (b32[:, 2] / n - m32 ** 2) / (n - 1)
    ok = (v64 + v32) > 0
    z = (m64[ok] - m32[ok]) / np.sqrt(v64[ok] + v32[ok])
    # the variances come from consecutive cycles, whose fission sources are correlated (strongly in
    # this reflective lattice), so they understate the true variance and z spreads wider than 1 for
    # equal distributions; a bias shows in the mean
    assert abs(z.mean()) < 0.2 and z.std() < 1.6, (z.mean(), z.std())


@pytest.mark.parametrize("form", FORMS)
def test_fixed_source_device_cycle_matches_oracle(gpu_mod, oracle_mod, form):
    p = problems.infinite_medium_2g()
    g, o = make_pair(gpu_mod, oracle_mod, p, form=form)
    ag = g.upload_tally(p.tallies["flux"])
    ao = o.upload_tally(p.tallies["flux"])
    mg = mo = 4242
    for _ in range(3):
        mg, _ = g.fixed_source_cycle(ag, 10000, mg)
        mo, _ = o.fixed_source_cycle(ao, 10000, mo)
    assert mg == mo
    np.testing.assert_allclose(g.bins(ag), o.bins(ao), rtol=1e-10)


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("transport", [abi.TRANSPORT_ST, abi.TRANSPORT_DT])
def test_p1_scattering_fp64_history_parity(gpu_mod, oracle_mod, transport, form):
    """multiScatterP1MG (linearly anisotropic scattering, PN P1): per-history bit-level agreement
    with the oracle, with coefficients that use all three branches of sampleLegendre_P1
    (|3 P1/P0| < 1 and between 1 and 3)."""
    rng = np.random.default_rng(29)
    p = problems.fixed_source_problem(rng, 4, "slab", layers=4)
    mg = dict(p.mg)
    p0 = np.asarray(mg["p0"])
    mg["p1"] = p0 * rng.uniform(-0.9, 0.9, size=p0.shape)          # 3 P1/P0 in (-2.7, 2.7)
    q = problems.Problem(p.geometry, mg, source=p.source, tallies=p.tallies)
    g, o = make_pair(gpu_mod, oracle_mod, q, transport, form=form)
    n = 20000
    bank = o.generate_source(SEED, n)
    ag, ao = g.upload_tally(q.tallies["flux"]), o.upload_tally(q.tallies["flux"])
    _, sg = g.transport_bank(ag, bank, 24680)
    _, so = o.transport_bank(ao, bank, 24680)
    cg, rg = g.history_records(n)
    co, ro = o.history_records(n)
    assert np.array_equal(cg, co) and np.array_equal(rg, ro)
    g.tally_cycle_end(ag, float(n))
    o.tally_cycle_end(ao, float(n))
    np.testing.assert_allclose(g.bins(ag), o.bins(ao), rtol=1e-10, atol=0)


@pytest.mark.parametrize("world", [2, 3])
def test_fixed_source_shards_sum_to_single_process(gpu_mod, oracle_mod, world):
    """sg_fixed_source_cycle_shard: the ranks of a population split (run here one after another on
    one GPU, each on its own handle, nothing shared) sum to the single-process oracle run."""
    from scone_gb300 import replicas
    p = problems.infinite_medium_2g()
    n, cycles = 30001, 3
    total = None
    for rank in range(world):
        g = gpu_mod.TransportOperatorGPU(p, precision=abi.PREC_FP64, transport=abi.TRANSPORT_ST, max_bank=n,
                                         form=abi.FORM_HISTORY)
        a = g.upload_tally(p.tallies["flux"])
        replicas.fixed_source_shard(g, a, n, rank, world, 777, cycles, gpu_mod.rng_skip)
        c = g.bins(a)[:, 1]
        total = c if total is None else total + c
        g.close()
    o = oracle_mod.Oracle(p, transport=abi.TRANSPORT_ST)
    ao = o.upload_tally(p.tallies["flux"])
    m = 777
    for _ in range(cycles):
        m, _ = o.fixed_source_cycle(ao, n, m)
    np.testing.assert_allclose(total, o.bins(ao)[:, 1], rtol=1e-10, atol=0)


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("transport", [abi.TRANSPORT_ST, abi.TRANSPORT_DT, abi.TRANSPORT_HT])
def test_union_cell_fp64_history_parity(gpu_mod, oracle_mod, transport, form):
    """unionCell geometry (a union of two spheres and its complement): per-history bit-level
    agreement with the oracle and equal tallies."""
    p = problems.union_cell_slab()
    g, o = make_pair(gpu_mod, oracle_mod, p, transport, form=form)
    n = 20000
    bank = o.generate_source(SEED, n)
    ag, ao = g.upload_tally(p.tallies["flux"]), o.upload_tally(p.tallies["flux"])
    g.transport_bank(ag, bank, 13579)
    o.transport_bank(ao, bank, 13579)
    cg, rg = g.history_records(n)
    co, ro = o.history_records(n)
    assert np.array_equal(cg, co) and np.array_equal(rg, ro)
    g.tally_cycle_end(ag, float(n))
    o.tally_cycle_end(ao, float(n))
    bg, bo = g.bins(ag), o.bins(ao)
    assert bg[:, 1].reshape(2, 2).sum(axis=1).min() > 0          # both cells are visited
    np.testing.assert_allclose(bg, bo, rtol=1e-10, atol=0)


def test_union_cell_bad_definition_is_rejected(gpu_mod):
    O, C, U = abi.CELL_OPEN, abi.CELL_CLOSE, abi.CELL_UNION
    gb = problems.GeometryBuilder()
    box = gb.surface(abi.BOX, 0.0, 0.0, 0.0, 6.0, 6.0, 6.0)
    s1 = gb.surface(abi.SPHERE, 0.0, 0.0, 0.0, 2.0)
    s2 = gb.surface(abi.SPHERE, 3.0, 0.0, 0.0, 2.0)
    a = gb.cell([-(s1 + 1), U, -(s2 + 1), s1 + 1])             # mixes union and intersection
    b = gb.cell([O, s1 + 1, C])
    uni = gb.cell_universe([a, b], [1, 2])
    gb.root_universe(box, problems.uni_fill(uni), bc=[abi.BC_REFLECTIVE] * 6)
    t = gpu_mod.TransportOperatorGPU(max_bank=16)
    with pytest.raises(gpu_mod.SconeGpuError, match="ambiguous"):
        t.upload_geometry(gb.arrays())


@pytest.mark.parametrize("form", FORMS)
def test_file_source_cycles_match_oracle(gpu_mod, oracle_mod, form, tmp_path):
    """fileSource: a bank written with printToFile's layout, read back and used as the source of
    fixed-source cycles (particle int(xi N) + 1 per history) gives the oracle's results."""
    p = problems.infinite_medium_2g()
    o0 = oracle_mod.Oracle(p)
    seed_bank = o0.generate_source(SEED, 500)
    rng = np.random.default_rng(5)
    seed_bank["r"][:] = rng.uniform(-9.0, 9.0, size=(500, 3))   # spread inside the reflective box
    seed_bank["G"][:] = rng.integers(1, 3, 500)
    stem = str(tmp_path / "src")
    gpu_mod.write_bank_file(stem, seed_bank, binary=True)
    fb = gpu_mod.read_bank_file(stem + ".bin")
    g = gpu_mod.TransportOperatorGPU(p, precision=abi.PREC_FP64, transport=abi.TRANSPORT_DT, max_bank=20000,
                                     form=form)
    o = oracle_mod.Oracle(p, transport=abi.TRANSPORT_DT)
    res = []
    for t in (g, o):
        t.set_file_source(fb)
        a = t.upload_tally(p.tallies["flux"])
        m = 99
        for _ in range(3):
            m, _ = t.fixed_source_cycle(a, 10000, m)
        res.append((m, t.bins(a)))
    assert res[0][0] == res[1][0]
    np.testing.assert_allclose(res[0][1], res[1][1], rtol=1e-10, atol=0)


def _map_clerks():
    """Collision and track clerks over the unionCell spheres binned by cell (with and without the
    rest bin), by x on an unstructured grid and on a lin grid."""
    C_, T_ = abi.CLERK_COLLISION, abi.CLERK_TRACK
    xb = np.array([-6.0, -2.5, -0.3, 0.0, 1.0, 3.3, 6.0])
    return [
        abi.clerk(C_, axes=[abi.cell_axis([1, 0]), (abi.AXIS_GROUP, 2, 0.0, 0.0)]),
        abi.clerk(T_, axes=[abi.cell_axis([0], undef_bin=True), abi.unstruct_axis(abi.AXIS_X, xb)]),
        abi.clerk(C_, axes=[abi.unstruct_axis(abi.AXIS_X, xb), (abi.AXIS_Y, 3, -6.0, 6.0, abi.GRID_LIN)]),
        abi.clerk(T_, resp=(abi.RESP_FLUX, abi.MACRO_TOTAL), axes=[abi.cell_axis([1])]),
    ]


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("transport", [abi.TRANSPORT_ST, abi.TRANSPORT_DT])
def test_cell_and_grid_maps_fp64_parity(gpu_mod, oracle_mod, transport, form):
    """cellMap and unstructured / lin grids on the device against the oracle: equal tallies."""
    p = problems.union_cell_slab()
    g, o = make_pair(gpu_mod, oracle_mod, p, transport, form=form)
    n = 20000
    bank = o.generate_source(SEED, n)
    clerks = _map_clerks()
    ag, ao = g.upload_tally(clerks), o.upload_tally(clerks)
    g.transport_bank(ag, bank, 24680)
    o.transport_bank(ao, bank, 24680)
    cg, rg = g.history_records(n)
    co, ro = o.history_records(n)
    assert np.array_equal(cg, co) and np.array_equal(rg, ro)
    g.tally_cycle_end(ag, float(n))
    o.tally_cycle_end(ao, float(n))
    bg, bo = g.bins(ag), o.bins(ao)
    assert bg[:4, 1].min() > 0
    np.testing.assert_allclose(bg, bo, rtol=1e-10, atol=0)


def test_cell_and_grid_maps_mixed(gpu_mod, oracle_mod):
    """The mixed form (FP32 grid search) on the same maps: within 3 % of the FP64 form per bin of
    the cell map and the total of the unstructured grid."""
    p = problems.union_cell_slab()
    out = {}
    for prec in (abi.PREC_FP64, abi.PREC_MIXED):
        g = gpu_mod.TransportOperatorGPU(p, precision=prec, transport=abi.TRANSPORT_ST, max_bank=1 << 18)
        a = g.upload_tally(_map_clerks())
        g.fixed_source_cycle(a, 200000, 777)
        out[prec] = g.bins(a)[:, 1]
        g.close()
    f, m = out[abi.PREC_FP64], out[abi.PREC_MIXED]
    np.testing.assert_allclose(m[:4], f[:4], rtol=0.03)
    np.testing.assert_allclose(m.sum(), f.sum(), rtol=0.03)


def test_bad_map_axes_are_rejected(gpu_mod):
    p = problems.union_cell_slab()
    g = gpu_mod.TransportOperatorGPU(p, max_bank=16)
    C_ = abi.CLERK_COLLISION
    for ax, msg in [(abi.unstruct_axis(abi.AXIS_X, [0.0, 2.0, 1.0]), "not sorted"),
                    (abi.cell_axis([5]), "lacks"),
                    ((abi.AXIS_X, 4, 0.0, 1.0, abi.GRID_LOG), "lin or unstruct"),
                    ((abi.AXIS_ENERGY, 4, 0.0, 1.0, abi.GRID_LOG), "0 < min")]:
        with pytest.raises(gpu_mod.SconeGpuError, match=msg):
            g.upload_tally([abi.clerk(C_, axes=[ax])])
    g.close()


def test_heap_threshold_window_and_radix_agree(gpu_mod, oracle_mod, monkeypatch):
    """normSize_Repr's heap threshold found by the window select and by the radix select alone
    (SCONE_GB300_NO_WINDOW_SELECT=1) gives the same cycles as the oracle."""
    p = problems.lattice_17x17_7g()
    o = oracle_mod.Oracle(p)
    ko, _, _ = _eigen(o, p, 20000, 2, 2)
    for flag in ("0", "1"):
        monkeypatch.setenv("SCONE_GB300_NO_WINDOW_SELECT", flag)
        g = gpu_mod.TransportOperatorGPU(p, max_bank=1 << 16)
        kg, _, _ = _eigen(g, p, 20000, 2, 2)
        g.close()
        np.testing.assert_allclose(kg, ko, rtol=1e-10)


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("transport", [abi.TRANSPORT_ST, abi.TRANSPORT_DT, abi.TRANSPORT_ST_NOCACHE])
def test_rotated_universes_fp64_history_parity(gpu_mod, oracle_mod, transport, form):
    """Rotated cell and pin universes (universe `rotation`): per-history bit-level agreement with the
    oracle and equal tallies."""
    p = problems.rotated_pins()
    g, o = make_pair(gpu_mod, oracle_mod, p, transport, form=form)
    n = 20000
    bank = o.generate_source(SEED, n)
    ag, ao = g.upload_tally(p.tallies["flux"]), o.upload_tally(p.tallies["flux"])
    g.transport_bank(ag, bank, 97531)
    o.transport_bank(ao, bank, 97531)
    cg, rg = g.history_records(n)
    co, ro = o.history_records(n)
    assert np.array_equal(cg, co) and np.array_equal(rg, ro)
    g.tally_cycle_end(ag, float(n))
    o.tally_cycle_end(ao, float(n))
    np.testing.assert_allclose(g.bins(ag), o.bins(ao), rtol=1e-10, atol=0)


def test_rotated_universes_mixed_statistics(gpu_mod):
    """The mixed form on rotated universes agrees with the FP64 form within statistics."""
    p = problems.rotated_pins()
    out = {}
    for prec in (abi.PREC_FP64, abi.PREC_MIXED):
        t = gpu_mod.TransportOperatorGPU(p, precision=prec, transport=abi.TRANSPORT_ST, max_bank=1 << 18)
        a = t.upload_tally(p.tallies["flux"])
        t.fixed_source_cycle(a, 200000, 4321)
        out[prec] = t.bins(a)[:, 1]
        t.close()
    np.testing.assert_allclose(out[abi.PREC_MIXED][:12], out[abi.PREC_FP64][:12], rtol=0.03)


def _ww_sphere():
    rng = np.random.default_rng(5)
    p = problems.fixed_source_problem(rng, 2, "sphere", radius=6.0)
    x = np.linspace(-6.0, 6.0, 13)
    centres = 0.5 * (x[1:] + x[:-1])
    lower = 0.4 / (1.0 + np.abs(centres))
    desc = abi.collision(abi.COLL_IMP, ww_axes=[(abi.AXIS_X, 12, -6.0, 6.0)], ww_lower=lower,
                         ww_upper=5.0 * lower, ww_const_survival=2.5, buffer_depth=64)
    return p, desc


@pytest.mark.parametrize("transport", [abi.TRANSPORT_ST, abi.TRANSPORT_DT])
def test_weight_windows_mg_fp64_history_parity(gpu_mod, oracle_mod, transport):
    """neutronMGimp with weight windows (splitting into the history's buffer, roulette) on the device
    against the oracle: per-history collision counts and final RNG states, and tallies."""
    p, desc = _ww_sphere()
    g, o = make_pair(gpu_mod, oracle_mod, p, transport, form=abi.FORM_HISTORY)
    g.set_collision(desc)
    o.set_collision(desc)
    n = 20000
    bank = o.generate_source(SEED, n)
    ag, ao = g.upload_tally(p.tallies["flux"]), o.upload_tally(p.tallies["flux"])
    g.transport_bank(ag, bank, 8642)
    o.transport_bank(ao, bank, 8642)
    cg, rg = g.history_records(n)
    co, ro = o.history_records(n)
    assert np.array_equal(cg, co) and np.array_equal(rg, ro)
    g.tally_cycle_end(ag, float(n))
    o.tally_cycle_end(ao, float(n))
    np.testing.assert_allclose(g.bins(ag), o.bins(ao), rtol=1e-10, atol=0)


@pytest.mark.parametrize("form", FORMS)
def test_ce_imp_fp64_history_parity(gpu_mod, oracle_mod, form):
    """neutronCEimp with implicit absorption and roulette (and splitting in the history-loop form)
    on the CE slab: per-history agreement with the oracle and equal tallies."""
    p = problems.ce_slab_3layer(points=(2000, 4000))
    desc = abi.collision(abi.COLL_IMP, imp_abs=True, roulette=True, split=(form == abi.FORM_HISTORY),
                         min_wgt=0.25, max_wgt=1.25, av_wgt=0.5)
    g, o = make_pair(gpu_mod, oracle_mod, p, abi.TRANSPORT_DT, form=form)
    g.set_collision(desc)
    o.set_collision(desc)
    n = 5000
    bank = o.generate_source(SEED, n)
    ag, ao = g.upload_tally(p.tallies["flux"]), o.upload_tally(p.tallies["flux"])
    g.transport_bank(ag, bank, 1122)
    o.transport_bank(ao, bank, 1122)
    cg, rg = g.history_records(n)
    co, ro = o.history_records(n)
    assert np.array_equal(cg, co) and np.array_equal(rg, ro)
    g.tally_cycle_end(ag, float(n))
    o.tally_cycle_end(ao, float(n))
    np.testing.assert_allclose(g.bins(ag), o.bins(ao), rtol=1e-10, atol=0)


def test_weight_windows_mixed_statistics(gpu_mod):
    """Mixed form with weight windows against the FP64 form and against analog transport."""
    p, desc = _ww_sphere()
    out = {}
    for key, prec, imp in (("f64", abi.PREC_FP64, True), ("mx", abi.PREC_MIXED, True), ("std", abi.PREC_FP64, False)):
        t = gpu_mod.TransportOperatorGPU(p, precision=prec, transport=abi.TRANSPORT_ST, max_bank=1 << 18,
                                         form=abi.FORM_HISTORY)
        if imp:
            t.set_collision(desc)
        a = t.upload_tally(p.tallies["flux"])
        t.fixed_source_cycle(a, 200000, 55)
        out[key] = t.bins(a)[:, 1]
        t.close()
    np.testing.assert_allclose(out["mx"], out["f64"], rtol=0.02)
    np.testing.assert_allclose(out["f64"], out["std"], rtol=0.02)


def test_splitting_needs_history_form(gpu_mod):
    p, desc = _ww_sphere()
    t = gpu_mod.TransportOperatorGPU(p, max_bank=1 << 12, form=abi.FORM_EVENT)
    t.set_collision(desc)
    a = t.upload_tally(p.tallies["flux"])
    with pytest.raises(gpu_mod.SconeGpuError, match="history-loop"):
        t.fixed_source_cycle(a, 1000, 1)
    t.close()


def _fixed_bank_parity(gpu_mod, oracle_mod, p, transport, form, n, master, k_eff=1.0, tally="flux"):
    """One gen loop over the same source bank on the device and in the oracle, FP64: per-history
    collision counts and end RNG states identical, fission banks identical (when fissile), tallies
    equal to round-off.  Returns the device bins."""
    g, o = make_pair(gpu_mod, oracle_mod, p, transport, form=form, max_bank=max(1 << 18, 4 * n))
    bank = o.generate_source(SEED, n)
    ag, ao = g.upload_tally(p.tallies[tally]), o.upload_tally(p.tallies[tally])
    ng, sg = g.transport_bank(ag, bank, master, k_eff=k_eff)
    no, so = o.transport_bank(ao, bank, master, k_eff=k_eff)
    cg, rg = g.history_records(n)
    co, ro = o.history_records(n)
    assert np.array_equal(cg, co)
    assert np.array_equal(rg, ro)
    assert sg.n_events == so.n_events and sg.n_collisions == so.n_collisions
    assert sg.n_next == so.n_next
    m = so.n_next
    for k in ("G", "wgt", "brood_id"):
        assert np.array_equal(ng[k][:m], no[k][:m]), k
    np.testing.assert_allclose(ng["r"][:m], no["r"][:m], rtol=0, atol=1e-9)
    g.tally_cycle_end(ag, float(n))
    o.tally_cycle_end(ao, float(n))
    bg, bo = g.bins(ag), o.bins(ao)
    np.testing.assert_allclose(bg, bo, rtol=1e-10, atol=1e-300)
    g.close()
    return bg, so


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("transport", ALL_TRANSPORTS)
def test_scone_test_lat_fp64_history_parity(gpu_mod, oracle_mod, transport, form):
    """SCONE's own test_lat geometry (IntegrationTestFiles/Geometry/test_lat, geometryStd_iTest.f90):
    squareCylinder root with reflective x and periodic y boundaries, a pin and a square pin in a 2x2
    lattice; fissile regions give fission sites.  Per-history and bank parity with the oracle."""
    p = problems.scone_test_lat_problem()
    bins, st = _fixed_bank_parity(gpu_mod, oracle_mod, p, transport, form, 20000, 97531, k_eff=1.1)
    assert st.n_next > 0
    assert (bins[:, 1] > 0).sum() >= 60                          # every mesh cell of every group is reached


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("transport", ALL_TRANSPORTS)
def test_plane_cells_periodic_box_fp64_history_parity(gpu_mod, oracle_mod, transport, form):
    """General planes (plane_class.f90:144-186) cutting a cellUniverse, inside a box with periodic x
    faces (box_class.f90 explicitBC / transformBC periodic branches): per-history parity."""
    p = problems.plane_cells()
    bins, _ = _fixed_bank_parity(gpu_mod, oracle_mod, p, transport, form, 20000, 86420)
    assert bins[:4, 1].min() > 0                                   # both materials, both groups


@pytest.mark.parametrize("problem", ["scone_test_lat", "plane_cells"])
@pytest.mark.parametrize("transport", [abi.TRANSPORT_ST, abi.TRANSPORT_DT])
def test_scone_geometries_mixed_statistics(gpu_mod, problem, transport):
    """The mixed form on squareCylinder/periodic and general-plane geometries agrees with the FP64
    form within statistics: per-bin z-scores of 10 cycles of 20 000 histories (the gen loop over the
    same point-source bank, fission sites discarded)."""
    p = problems.scone_test_lat_problem() if problem == "scone_test_lat" else problems.plane_cells()
    out = {}
    n, cycles = 20000, 10
    for prec in (abi.PREC_FP64, abi.PREC_MIXED):
        t = gpu_mod.TransportOperatorGPU(p, precision=prec, transport=transport, max_bank=1 << 18,
                                         form=abi.FORM_HISTORY)
        a = t.upload_tally(p.tallies["flux"])
        bank = t.generate_source(SEED, n)
        for c in range(cycles):
            t.transport_bank(a, bank, 2468 + 7919 * c, k_eff=1.1, next_cap=1 << 18)
            t.tally_cycle_end(a, float(n), 1.1)
        out[prec] = t.bins(a)
        t.close()
    b64, b32 = out[abi.PREC_FP64], out[abi.PREC_MIXED]
    m64, m32 = b64[:, 1] / cycles, b32[:, 1] / cycles
    v64 = np.maximum(b64[:, 2] / cycles - m64 ** 2, 0) / (cycles - 1)
    v32 = np.maximum(b32[:, 2] / cycles - m32 ** 2, 0) / (cycles - 1)
    ok = (v64 + v32) > 0
    z = (m64[ok] - m32[ok]) / np.sqrt(v64[ok] + v32[ok])
    assert ok.sum() >= 4                                      # DT scores no track-length bins
    assert np.abs(z).max() < 5.0 and abs(z.mean()) < 0.5, (z.mean(), np.abs(z).max())


@pytest.mark.parametrize("transport", [abi.TRANSPORT_ST, abi.TRANSPORT_DT])
def test_lattice_fp64_parity_large_population(gpu_mod, oracle_mod, transport):
    """FP64 per-history parity on 1e5 lattice histories (a converged-shape fission bank, the mesh
    tally and k-implicit clerks): every history's collision count and end RNG state, the fission
    bank and the bins."""
    p = problems.lattice_17x17_7g()
    n = 100000
    g, o = make_pair(gpu_mod, oracle_mod, p, transport, form=abi.FORM_HISTORY, max_bank=1 << 19)
    o.eigen_init(n, SEED)
    bank, pop = o.eigen_bank(n)
    assert pop == n
    clerks = p.tallies["mesh"] + [abi.clerk(abi.CLERK_KEFF_IMPLICIT)]
    ag, ao = g.upload_tally(clerks), o.upload_tally(clerks)
    ng, sg = g.transport_bank(ag, bank, 5551212, k_eff=1.07, next_cap=1 << 19)
    no, so = o.transport_bank(ao, bank, 5551212, k_eff=1.07, next_cap=1 << 19)
    cg, rg = g.history_records(n)
    co, ro = o.history_records(n)
    assert np.array_equal(cg, co)
    assert np.array_equal(rg, ro)
    assert sg.n_events == so.n_events and sg.n_next == so.n_next > 0
    m = so.n_next
    for k in ("G", "wgt", "brood_id"):
        assert np.array_equal(ng[k][:m], no[k][:m]), k
    np.testing.assert_allclose(ng["r"][:m], no["r"][:m], rtol=0, atol=1e-9)
    g.tally_cycle_end(ag, float(m), 1.07)
    o.tally_cycle_end(ao, float(m), 1.07)
    np.testing.assert_allclose(g.bins(ag), o.bins(ao), rtol=1e-10, atol=1e-300)
    g.close()


def _pinned_bank(src, n, cap=None):
    """A HostBank whose arrays live in page-locked host memory (torch pin_memory), filled from src."""
    import torch
    cap = cap or n
    arrs = {}
    for k, shape, dt in (("wgt", (cap,), torch.float64), ("r", (cap, 3), torch.float64),
                         ("dir", (cap, 3), torch.float64), ("G", (cap,), torch.int32),
                         ("time", (cap,), torch.float64), ("brood_id", (cap,), torch.int32)):
        t = torch.zeros(shape, dtype=dt).pin_memory()
        if src is not None:
            t[:n].copy_(torch.from_numpy(np.ascontiguousarray(src[k][:n])))
        arrs[k] = t
    hb = abi.HostBank(cap, {k: v.numpy() for k, v in arrs.items()})
    hb._pinned = arrs                                      # keeps the page-locked memory alive
    return hb


@pytest.mark.parametrize("pinned", [False, True])
def test_eigen_cycle_bank_equals_resident_cycles(gpu_mod, pinned):
    """sg_eigen_cycle_bank (host dungeons: bank in, normalised bank out, pRNG and k passed through)
    gives the device-resident sg_eigen_cycle's k, pRNG and banks, FP64, cycle after cycle; with
    page-locked banks the kernels read the input in place."""
    p = problems.lattice_17x17_7g()
    pop = 5000
    res = gpu_mod.TransportOperatorGPU(p, precision=abi.PREC_FP64, max_bank=1 << 16, form=abi.FORM_HISTORY)
    host = gpu_mod.TransportOperatorGPU(p, precision=abi.PREC_FP64, max_bank=1 << 16, form=abi.FORM_HISTORY)
    adm = {}
    for t in (res, host):
        inact, act = t.upload_tally([]), t.upload_tally(p.tallies["mesh"])
        ia = t.upload_tally([abi.clerk(abi.CLERK_KEFF_ANALOG)])
        aa = t.upload_tally([abi.clerk(abi.CLERK_KEFF_IMPLICIT)])
        t.attach_tally(inact, ia)
        t.attach_tally(act, aa)
        adm[id(t)] = (inact, ia, act, aa)
    res.eigen_init(pop, SEED)
    b0, _ = res.eigen_bank(pop)
    master, k = res.eigen_state()
    k_end = 1.0
    mk = (lambda src, n, cap=None: _pinned_bank(src, n, cap)) if pinned else \
        (lambda src, n, cap=None: abi.HostBank(cap or n) if src is None else abi.HostBank(n, src.head(n)))
    bank = mk(b0, pop)
    out = mk(None, pop, pop)
    for c in range(6):
        inact, ia, act, aa = adm[id(res)]
        st_r = res.eigen_cycle(inact if c < 3 else act, ia if c < 3 else aa)
        inact, ia, act, aa = adm[id(host)]
        master, k_new, st_h = host.eigen_cycle_bank(inact if c < 3 else act, ia if c < 3 else aa, bank, pop,
                                                    master, k, k_end, out)
        k_end = k = k_new
        # k sums scores added atomically in another order: equal to round-off
        assert abs(st_h.k_new - st_r.k_new) <= 1e-12 * st_r.k_new and st_h.n_next == st_r.n_next, c
        assert st_h.n_events == st_r.n_events
        mr, kr = res.eigen_state()
        assert master == mr and abs(k - kr) <= 1e-12 * kr
        br, _ = res.eigen_bank(pop)
        for key in ("G", "brood_id", "wgt", "r", "dir"):
            assert np.array_equal(out[key][:pop], br[key][:pop]), (c, key)
        bank, out = out, bank
    np.testing.assert_allclose(host.bins(adm[id(host)][2]), res.bins(adm[id(res)][2]), rtol=1e-12, atol=1e-300)
    res.close()
    host.close()


def test_transport_bank_reads_page_locked_banks_in_place(gpu_mod, oracle_mod):
    """sg_transport_bank on a page-locked host bank (read in place by the kernels) and on the same
    bank in pageable memory (copied first): identical fission banks and bins."""
    p = problems.lattice_17x17_7g()
    n = 20000
    o = oracle_mod.Oracle(p)
    o.eigen_init(n, SEED)
    bank, _ = o.eigen_bank(n)
    out = []
    for pinned in (False, True):
        g = gpu_mod.TransportOperatorGPU(p, precision=abi.PREC_MIXED, transport=abi.TRANSPORT_DT, max_bank=1 << 17,
                                         form=abi.FORM_HISTORY)
        a = g.upload_tally(p.tallies["mesh"] + [abi.clerk(abi.CLERK_KEFF_IMPLICIT)])
        b = _pinned_bank(bank, n) if pinned else abi.HostBank(n, bank.head(n))
        nxt, st = g.transport_bank(a, b, 31337, k_eff=1.02, next_cap=1 << 17)
        g.tally_cycle_end(a, float(st.n_next), 1.02)
        out.append((nxt.head(st.n_next), g.bins(a)))
        g.close()
    (b0, t0), (b1, t1) = out
    for k in ("G", "brood_id", "wgt", "r", "dir", "time"):
        assert np.array_equal(b0[k], b1[k]), k
    np.testing.assert_allclose(t1, t0, rtol=1e-10, atol=1e-300)


@pytest.mark.parametrize("precision", [abi.PREC_FP64, abi.PREC_MIXED])
@pytest.mark.parametrize("form,transport", [(abi.FORM_HISTORY, abi.TRANSPORT_DT), (abi.FORM_HISTORY, abi.TRANSPORT_ST),
                                            (abi.FORM_HISTORY, abi.TRANSPORT_HT), (abi.FORM_EVENT, abi.TRANSPORT_DT)])
def test_reflective_box_never_leaks(gpu_mod, precision, form, transport):
    """The 17x17 lattice sits in an all-reflective box, so no history may end as a leak: the
    k-implicit clerk's leakage bin stays exactly zero over 1e6 histories.  (Delta-tracking flights
    that leave the box are brought back by the transform BC; a transform that also reflected a
    coordinate lying just inside another face would leave the point outside, which the mixed form
    then scored as a leak about once per 1e5 histories.)"""
    p = problems.lattice_17x17_7g()
    n = 1000000
    t = gpu_mod.TransportOperatorGPU(p, precision=precision, transport=transport, max_bank=1 << 21, form=form)
    t.eigen_init(n, SEED)
    bank, pop = t.eigen_bank(n)
    assert pop == n
    a = t.upload_tally([abi.clerk(abi.CLERK_KEFF_IMPLICIT)])
    nxt, st = t.transport_bank(a, bank, 8675309, k_eff=1.08, next_cap=1 << 21)
    assert st.n_next > 0.9 * n
    t.tally_cycle_end(a, float(st.n_next), 1.08)
    b = t.bins(a)
    assert b[3, 1] == 0.0, b[:, 1]                        # bins: prod, scatter prod, abs, leak, k
    assert b[2, 1] > 0.0
    t.close()


@pytest.mark.parametrize("transport", [abi.TRANSPORT_DT, abi.TRANSPORT_ST])
def test_lattice_mixed_k_unbiased_correlated(gpu_mod, transport):
    """Correlated sampling: both precision forms transport the same converged 1e6 bank with the
    same RNG streams, cycle after cycle, so most histories follow the same path and k_mixed - k_FP64
    has a standard error of a few 1e-7: a bias of the mixed form shows far below the statistical
    error of either k.  (A boundary transform that leaked a few histories per 1e5 moved it by
    -1.6e-5.)"""
    p = problems.lattice_17x17_7g()
    pop = 1000000
    ops = {prec: gpu_mod.TransportOperatorGPU(p, precision=prec, transport=transport, max_bank=3 * pop,
                                              form=abi.FORM_HISTORY)
           for prec in (abi.PREC_FP64, abi.PREC_MIXED)}
    fp = ops[abi.PREC_FP64]
    inact = fp.upload_tally([])
    ia = fp.upload_tally([abi.clerk(abi.CLERK_KEFF_ANALOG)])
    fp.attach_tally(inact, ia)
    fp.eigen_init(pop, SEED)
    for _ in range(20):
        fp.eigen_cycle(inact, ia)
    bank, n = fp.eigen_bank(pop)
    k0 = fp.eigen_state()[1]
    dk = []
    for c in range(8):
        ks = {}
        for prec, t in ops.items():
            a = t.upload_tally([abi.clerk(abi.CLERK_KEFF_IMPLICIT)])
            _, st = t.transport_bank(a, bank, 1000003 * (c + 1), k_eff=k0, next_cap=3 * pop)
            t.tally_cycle_end(a, float(st.n_next), k0)
            b = t.bins(a)
            assert b[3, 1] == 0.0                               # no leakage from a reflective box
            ks[prec] = b[4, 1]
        dk.append(ks[abi.PREC_MIXED] - ks[abi.PREC_FP64])
    dk = np.array(dk)
    se = dk.std(ddof=1) / np.sqrt(len(dk))
    assert abs(dk.mean()) < 4.0 * se + 2e-6, (dk.mean(), se)
    for t in ops.values():
        t.close()
