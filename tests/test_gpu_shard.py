"""An eigenvalue cycle split over processes on the GPU (SCONE with MPI): sg_normalise_shard against
the oracle's restatement of normSize_Repr's per-process part, and whole split runs (the processes
as threads of this program, each with its own handle on this one GPU, exchanging on the host
through ThreadComm) against the single-process run of sg_eigen_cycle.  No kernel waits on another
handle's kernels: every exchange is a host-side step between launches."""
import numpy as np
import pytest

from scone_gb300 import abi, problems, replicas

from test_replicas_eigen import KEYS, SEED, _check, _run_single, _sites, _split_at_broods, run_threads

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu_mod():
    from scone_gb300 import gpu
    gpu.load()
    return gpu


@pytest.mark.parametrize("world", [1, 3])
@pytest.mark.parametrize("k_eff,tot_pop", [(1.0, 15000), (3.0, 15000), (8.0, 15000), (1.0, None)])
def test_normalise_shard_matches_oracle(gpu_mod, oracle_mod, world, k_eff, tot_pop):
    """Every process's normalised sites, bit for bit, and their concatenation equal to the
    single-process normSize_Repr."""
    p = problems.lattice_17x17_7g()
    o = oracle_mod.Oracle(p, transport=abi.TRANSPORT_DT)
    bank, m = _sites(o, p, 20000, k_eff)
    tp = tot_pop or m
    master = 0x1D0C9B5E3A17F42 & ((1 << 63) - 1)
    single, ns = o.normalise(bank, m, tp, master, 20 * tp)
    g = gpu_mod.TransportOperatorGPU(p, precision=abi.PREC_FP64, transport=abi.TRANSPORT_DT, max_bank=1 << 18,
                                     form=abi.FORM_HISTORY)
    before, parts = 0, []
    for piece, lo_h in _split_at_broods(bank, m, world):
        og, ng = g.normalise_shard(piece, piece.n, before, m, tp, master, 20 * tp)
        oo, no = o.normalise_shard(piece, piece.n, before, m, tp, master, 20 * tp)
        before += piece.n
        assert ng == no
        for k in KEYS + ("brood_id",):
            assert np.array_equal(og[k][:ng], oo[k][:no]), k
        parts.append((og, ng, lo_h))
    for k in KEYS:
        assert np.array_equal(np.concatenate([b[k][:n] for b, n, _ in parts]), single[k][:ns]), k
    g.close()


@pytest.mark.parametrize("precision", [abi.PREC_FP64, abi.PREC_MIXED])
@pytest.mark.parametrize("world", [2, 3])
def test_split_eigen_cycles_equal_single_process(gpu_mod, precision, world):
    """Five lattice cycles from k0 = 3 (duplication in the first cycle, dropping after), the
    population split over 2 or 3 processes: the concatenated banks and the RNG state equal the
    single-process run's, k and the (synchronised) mesh tally to round-off."""
    p = problems.lattice_17x17_7g()
    pop, cycles, k0 = 30000, 5, 3.0

    def op():
        return gpu_mod.TransportOperatorGPU(p, precision=precision, transport=abi.TRANSPORT_DT, max_bank=1 << 18,
                                            form=abi.FORM_HISTORY)

    ops = [op() for _ in range(world)]
    shards = run_threads(ops, p, pop, cycles, k0, gpu_mod.rng_skip)
    one = op()
    single = _run_single(one, p, pop, cycles, k0)
    _check(shards, single, pop)
    for t in ops + [one]:
        t.close()
