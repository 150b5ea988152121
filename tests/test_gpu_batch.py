"""GPU parity of the batched and served forms (sg_batch_*, sg_serve_*).

Every problem of a batch must give what SCONE's fixedSourcePhysicsPackage gives for that problem
alone: the oracle runs each problem's cycles one after another, the batched kernel runs every cycle
of every problem in one launch.  Histories use the same RNG streams in both, so the all-FP64 form
agrees to round-off (scores are summed in a different order: relative 1e-10).  The mixed form is
compared with the FP64 form statistically.
"""
import numpy as np
import pytest

from scone_gb300 import abi, problems

pytestmark = pytest.mark.gpu

RTOL = 1e-10


@pytest.fixture(scope="module")
def gpu_mod():
    from scone_gb300 import gpu
    gpu.load()
    return gpu


def small_batch(seed=3, n=12, pop=(200, 1500), cycles=3):
    """A mixed batch with every group count and both geometry kinds."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        n_g = problems.GROUP_CHOICES[i % len(problems.GROUP_CHOICES)]
        kind = "sphere" if i % 2 == 0 else "slab"
        p = problems.fixed_source_problem(rng, n_g, kind)
        out.append((p, int(rng.integers(pop[0], pop[1])), cycles, int(rng.integers(1, 2 ** 62))))
    return out


def oracle_bins(orl, batch, transport):
    res = []
    for p, pop, cycles, master in batch:
        o = orl.Oracle(p, transport=transport)
        a = o.upload_tally(p.tallies["flux"])
        m = master
        for _ in range(cycles):
            m, _ = o.fixed_source_cycle(a, pop, m)
        res.append(o.bins(a))
        o.close()
    return res


def load_batch(gpu, batch, precision, transport, **kw):
    B = gpu.BatchGPU(precision=precision, transport=transport, max_problems=max(64, len(batch)),
                     arena_bytes=kw.pop("arena_bytes", 256 << 20), max_work_items=1 << 16)
    slots = [B.add(p, pop, cycles, master) for p, pop, cycles, master in batch]
    return B, slots


@pytest.mark.parametrize("transport", [abi.TRANSPORT_ST, abi.TRANSPORT_DT, abi.TRANSPORT_ST_NOCACHE,
                                       abi.TRANSPORT_HT])
def test_batched_fp64_matches_oracle(gpu_mod, oracle_mod, transport):
    batch = small_batch()
    ref = oracle_bins(oracle_mod, batch, transport)
    B, slots = load_batch(gpu_mod, batch, abi.PREC_FP64, transport)
    st = B.run(slots)
    assert st.n_histories == sum(pop * c for _, pop, c, _ in batch)
    for s, r in zip(slots, ref):
        got = B.bins(s)
        assert np.all(got[:, 0] == 0.0)                  # BIN is cleared by every cycle close
        np.testing.assert_allclose(got[:, 1:], r[:, 1:], rtol=RTOL, atol=0)


@pytest.mark.parametrize("form", [abi.FORM_EVENT, abi.FORM_HISTORY])
def test_plain_forms_match_batched(gpu_mod, form):
    """One problem per launch sequence (sg_fixed_source_cycle's path) against one launch for all."""
    batch = small_batch(seed=5)
    B, slots = load_batch(gpu_mod, batch, abi.PREC_FP64, abi.TRANSPORT_DT)
    B.run(slots)
    a = [B.bins(s) for s in slots]
    for s in slots:
        B.clear_tally(s)
    st = B.run_plain(slots, form=form)
    assert st.n_histories == sum(pop * c for _, pop, c, _ in batch)
    for s, x in zip(slots, a):
        np.testing.assert_allclose(B.bins(s), x, rtol=RTOL, atol=0)


def test_results_do_not_depend_on_launch_shape(gpu_mod):
    batch = small_batch(seed=7)
    B, slots = load_batch(gpu_mod, batch, abi.PREC_FP64, abi.TRANSPORT_ST)
    ref = None
    for item, block, order, per in [(1024, 128, 1, 0), (32, 64, 0, 1), (4096, 96, 0, 2), (256, 32, 1, 0)]:
        for s in slots:
            B.clear_tally(s)
        B.set_tuning(item_histories=item, block_threads=block, order=order, blocks_per_sm=per)
        B.run(slots)
        got = [B.bins(s) for s in slots]
        if ref is None:
            ref = got
        else:
            for g, r in zip(got, ref):
                np.testing.assert_allclose(g, r, rtol=RTOL, atol=0)


def test_mixed_form_agrees_with_fp64(gpu_mod):
    """Precision form against the all-FP64 form on the same histories: per-bin z-scores of the means
    and the relative errors (within 10 % of the FP64 ones)."""
    rng = np.random.default_rng(11)
    batch = []
    for i, n_g in enumerate(problems.GROUP_CHOICES * 2):
        p = problems.fixed_source_problem(rng, n_g, "sphere" if i % 2 else "slab")
        batch.append((p, 4000, 10, int(rng.integers(1, 2 ** 62))))
    res = {}
    for prec in (abi.PREC_FP64, abi.PREC_MIXED):
        B, slots = load_batch(gpu_mod, batch, prec, abi.TRANSPORT_DT)
        B.run(slots)
        res[prec] = [B.bins(s) for s in slots]
        B.close()
    zs = []
    for a, b, (_, pop, cycles, _) in zip(res[abi.PREC_FP64], res[abi.PREC_MIXED], batch):
        n = cycles
        ma, mb = a[:, 1] / n, b[:, 1] / n
        va = np.maximum(a[:, 2] / n - ma ** 2, 0) / (n - 1)
        vb = np.maximum(b[:, 2] / n - mb ** 2, 0) / (n - 1)
        ok = (va > 0) & (vb > 0)
        # the two forms follow the same RNG streams, so their estimates are strongly correlated:
        # differences far below the statistical error
        zs.extend(((ma - mb)[ok] / np.sqrt(va + vb)[ok]).tolist())
        rel_a, rel_b = np.sqrt(va[ok]) / ma[ok], np.sqrt(vb[ok]) / mb[ok]
        assert np.all(np.abs(rel_b / rel_a - 1.0) < 0.10)
    zs = np.array(zs)
    assert np.all(np.abs(zs) < 1.0), np.abs(zs).max()


def test_arena_admission_by_budget(gpu_mod):
    """A full arena refuses a problem (SG_ERR_OOM); removing one frees room for it."""
    rng = np.random.default_rng(13)
    B = gpu_mod.BatchGPU(precision=abi.PREC_MIXED, transport=abi.TRANSPORT_DT, max_problems=64,
                         arena_bytes=4 << 20, max_work_items=1 << 12)
    p = problems.fixed_source_problem(rng, 16, "slab", layers=10)
    slots = []
    while True:
        s = B.try_add(p, 100, 3, 99)
        if s is None:
            break
        slots.append(s)
        assert len(slots) < 64
    used, cap = B.memory()
    assert 0 < used <= cap and len(slots) >= 2
    B.remove(slots.pop())
    s = B.try_add(p, 100, 3, 99)
    assert s is not None
    slots.append(s)
    B.run(slots)
    first = B.bins(slots[0])
    for s in slots[1:]:                                   # identical problems and seeds
        np.testing.assert_allclose(B.bins(s), first, rtol=RTOL, atol=0)


def test_autotune_keeps_results(gpu_mod):
    batch = small_batch(seed=17, n=10)
    B, slots = load_batch(gpu_mod, batch, abi.PREC_MIXED, abi.TRANSPORT_DT)
    best = B.autotune(slots)
    assert best["item_histories"] >= 32 and best["block_threads"] in (32, 64, 96, 128)
    assert all(np.all(B.bins(s) == 0.0) for s in slots)   # tallies cleared after tuning
    B.run(slots)
    a = [B.bins(s) for s in slots]
    for s in slots:
        B.clear_tally(s)
    B.set_tuning(item_histories=1024, block_threads=128, order=1, blocks_per_sm=0)
    B.run(slots)
    for s, x in zip(slots, a):
        np.testing.assert_allclose(B.bins(s), x, rtol=1e-9, atol=0)


def test_autotune_plain_keeps_results(gpu_mod):
    """Queue thresholds of the event form change scheduling only: FP64 results stay the same."""
    batch = small_batch(seed=23, n=6)
    B, slots = load_batch(gpu_mod, batch, abi.PREC_FP64, abi.TRANSPORT_ST)
    B.run_plain(slots, form=abi.FORM_EVENT)
    ref = [B.bins(s) for s in slots]
    best = B.autotune_plain(slots)
    assert best["rounds_per_check"] >= 1 and best["tail_divisor"] >= 1 and best["tail_min"] >= 0
    assert all(np.all(B.bins(s) == 0.0) for s in slots)
    B.run_plain(slots, form=abi.FORM_EVENT)
    for s, r in zip(slots, ref):
        np.testing.assert_allclose(B.bins(s), r, rtol=RTOL, atol=0)


@pytest.mark.parametrize("precision", [abi.PREC_FP64, abi.PREC_MIXED])
def test_served_result_alone_equals_result_in_mix(gpu_mod, precision):
    """Continuous batching: a request served alone and the same request admitted while others are
    on the device give the same tallies (same histories; only the summation order differs)."""
    batch = small_batch(seed=19, n=16, pop=(500, 4000), cycles=4)
    B, slots = load_batch(gpu_mod, batch, precision, abi.TRANSPORT_DT)
    B.set_tuning(item_histories=256)
    probe = slots[3]
    # alone
    B.serve_start(2048)
    B.submit(probe)
    done = []
    while not done:
        done += B.pump(wait=True)
    assert done[0][0] == probe and done[0][1] > 0
    alone = B.bins(probe)
    # in the mix: others first, the probe arrives while they run, more arrive after it; the waves
    # leave room for other streams' kernels meanwhile (smaller grid, same results)
    B.serve_share(2, True)
    for s in slots[:3]:
        B.submit(s)
    B.pump()
    B.submit(probe)
    for s in slots[4:]:
        B.submit(s)
        B.pump()
    seen = {}
    while len(seen) < len(slots):
        for s, lat in B.pump(wait=True):
            seen[s] = lat
    _, active, waves = B.serve_status()
    assert active == 0 and waves > 3
    B.serve_stop()
    np.testing.assert_allclose(B.bins(probe), alone, rtol=RTOL, atol=0)
    assert all(lat > 0 for lat in seen.values())
    # and both equal the batched form
    for s in slots:
        B.clear_tally(s)
    B.run([probe])
    np.testing.assert_allclose(B.bins(probe), alone, rtol=RTOL, atol=0)
