"""An eigenvalue cycle split over processes (SCONE with MPI, eigenPhysicsPackage_class.f90:203-303):
normSize_Repr's per-process part (particleDungeon_class.f90:431-590), loadBalancing (:593-700) and
the sum of the k attachment's scores (scoreMemory%reduceBins, scoreMemory_class.f90:403-432), on the
CPU with the oracle as every process's transport operator.  The split run must give the
single-process run's banks (concatenated in process order), RNG state and k."""
import os
import socket
import threading

import numpy as np
import pytest

from scone_gb300 import abi, problems, replicas

SEED = 0x5C3A84C9
KEYS = ("r", "dir", "wgt", "G", "time")


def _sites(o, p, n, k_eff, master=77):
    """Fission sites of n lattice histories, sorted by brood (the input of normSize_Repr)."""
    o.eigen_init(n, SEED)
    bank, _ = o.eigen_bank(n)
    a = o.upload_tally([])
    nxt, st = o.transport_bank(a, bank, master, k_eff=k_eff, next_cap=8 * n)
    return nxt, int(st.n_next)


def _split_at_broods(bank, m, world):
    """The sites of `world` processes that ran contiguous shares of the histories: cut at brood
    boundaries, each piece's brood IDs renumbered from 1 (as each process numbers its histories)."""
    brood = bank["brood_id"][:m]
    nh = int(brood.max())
    pieces = []
    for r in range(world):
        lo_h = replicas.offset(nh, r, world)
        hi_h = lo_h + replicas.workshare(nh, r, world)
        sel = (brood > lo_h) & (brood <= hi_h)
        d = {k: v[:m][sel].copy() for k, v in bank.a.items()}
        d["brood_id"] = d["brood_id"] - lo_h
        pieces.append((abi.HostBank(int(sel.sum()), d), lo_h))
    return pieces


@pytest.mark.parametrize("world", [1, 2, 3])
@pytest.mark.parametrize("k_eff,tot_pop", [(1.0, 1500), (3.0, 1500), (8.0, 1500), (1.0, None)])
def test_normalise_pieces_equal_single_process(oracle_mod, world, k_eff, tot_pop):
    """Each process normalises its own sites against the threshold over all processes' draws: the
    pieces, concatenated, are the single-process normSize_Repr result.  k_eff 3 and 8 leave fewer
    sites than the population (duplicates, and full copies at 8); tot_pop None keeps the count."""
    p = problems.lattice_17x17_7g()
    o = oracle_mod.Oracle(p, transport=abi.TRANSPORT_DT)
    bank, m = _sites(o, p, 2000, k_eff)
    tp = tot_pop or m
    master = 0x2545F4914F6CDD1D & ((1 << 63) - 1)
    single, ns = o.normalise(bank, m, tp, master, 20 * tp)
    assert ns == tp
    got = {k: [] for k in KEYS + ("brood_id",)}
    before = 0
    for piece, lo_h in _split_at_broods(bank, m, world):
        out, n_out = o.normalise_shard(piece, piece.n, before, m, tp, master, 20 * tp)
        before += piece.n
        for k in KEYS:
            got[k].append(out[k][:n_out])
        got["brood_id"].append(out["brood_id"][:n_out] + lo_h)
    for k in KEYS + ("brood_id",):
        assert np.array_equal(np.concatenate(got[k]), single[k][:ns]), k


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _setup(op, p):
    admin = op.upload_tally(p.tallies["mesh"])
    atch = op.upload_tally([abi.clerk(abi.CLERK_KEFF_IMPLICIT)])
    op.attach_tally(admin, atch)
    return admin, atch


def _run_shard(op, comm, p, pop, cycles, k0, skip):
    admin, atch = _setup(op, p)
    bank, master, k = replicas.eigen_shard_init(op, comm, pop, SEED, k0)
    k_end = 1.0
    ks = []
    for _ in range(cycles):
        bank, master, k_new, _ = replicas.eigen_cycle_shard(op, comm, admin, atch, bank, pop, master, k, k_end,
                                                            skip, sync=(admin,), next_cap=16 * pop)
        k = k_end = k_new
        ks.append(k_new)
    return bank, master, ks, op.bins(admin)


def _run_single(op, p, pop, cycles, k0):
    admin, atch = _setup(op, p)
    op.eigen_init(pop, SEED, k0)
    ks = [op.eigen_cycle(admin, atch).k_new for _ in range(cycles)]
    bank, n = op.eigen_bank(pop)
    assert n == pop
    master, _ = op.eigen_state()
    return bank, master, ks, op.bins(admin)


def _check(shards, single, pop):
    bank1, master1, ks1, bins1 = single
    assert all(s[1] == master1 for s in shards)
    for k in KEYS:
        got = np.concatenate([s[0][k][:s[0].n] for s in shards])
        assert got.shape[0] == pop and np.array_equal(got, bank1[k][:pop]), k
    for s in shards:
        np.testing.assert_allclose(s[2], ks1, rtol=1e-13, atol=0)
        np.testing.assert_allclose(s[3], bins1, rtol=1e-11, atol=1e-300)


def _gloo_rank(rank, world, port, pop, cycles, k0, out):
    import torch.distributed as dist
    from oracle import oracle
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    p = problems.lattice_17x17_7g()
    o = oracle.Oracle(p, transport=abi.TRANSPORT_DT)
    bank, master, ks, bins = _run_shard(o, replicas.TorchComm(), p, pop, cycles, k0, oracle.rng_skip)
    np.savez(f"{out}_{rank}.npz", master=np.uint64(master), ks=np.array(ks), bins=bins,
             **{k: bank[k][:bank.n] for k in KEYS})
    dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_gloo_eigen_cycles_equal_single_process(oracle_mod, tmp_path, world):
    """World-size 2 and 3 over gloo: five cycles of the lattice from k0 = 3 (the first cycle
    duplicates sites, the later ones drop them), every exchange through torch.distributed."""
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    pop, cycles, k0 = 1200, 5, 3.0
    out = str(tmp_path / "rank")
    mp.start_processes(_gloo_rank, args=(world, _free_port(), pop, cycles, k0, out), nprocs=world, join=True,
                       start_method="spawn")
    shards = []
    for r in range(world):
        z = np.load(f"{out}_{r}.npz")
        n = z["r"].shape[0]
        bank = abi.HostBank(n, dict({k: z[k] for k in KEYS}, brood_id=np.zeros(n, np.int32)))
        shards.append((bank, int(z["master"]), list(z["ks"]), z["bins"]))
    p = problems.lattice_17x17_7g()
    single = _run_single(oracle_mod.Oracle(p, transport=abi.TRANSPORT_DT), p, pop, cycles, k0)
    _check(shards, single, pop)


def run_threads(ops, p, pop, cycles, k0, skip):
    """Every process of a split run as a thread of this program (ThreadComm); results per rank."""
    comms = replicas.ThreadComm.group(len(ops))
    res, errs = [None] * len(ops), []

    def body(r):
        try:
            res[r] = _run_shard(ops[r], comms[r], p, pop, cycles, k0, skip)
        except BaseException as e:          # reported by the test, not lost in the thread
            errs.append(e)
            comms[r].sh.barrier.abort()

    th = [threading.Thread(target=body, args=(r,)) for r in range(len(ops))]
    for t in th:
        t.start()
    for t in th:
        t.join()
    if errs:
        raise errs[0]
    return res


def test_thread_comm_eigen_cycles_equal_single_process(oracle_mod):
    """The same split run with the processes as threads (ThreadComm), world size 4."""
    p = problems.lattice_17x17_7g()
    pop, cycles, k0 = 1000, 4, 3.0
    ops = [oracle_mod.Oracle(p, transport=abi.TRANSPORT_DT) for _ in range(4)]
    shards = run_threads(ops, p, pop, cycles, k0, oracle_mod.rng_skip)
    single = _run_single(oracle_mod.Oracle(p, transport=abi.TRANSPORT_DT), p, pop, cycles, k0)
    _check(shards, single, pop)


def test_load_balance_moves_particles_to_neighbours():
    """loadBalancing alone: shares of 5, 1 and 6 particles of a 12-particle population end as
    getWorkshare's 4, 4, 4, the particles in their global order."""
    comms = replicas.ThreadComm.group(3)
    pops = [5, 1, 6]
    start = np.cumsum([0] + pops)
    banks = []
    for r in range(3):
        n = pops[r]
        ids = np.arange(start[r], start[r] + n, dtype=np.float64)
        banks.append(abi.HostBank(n, dict(r=np.repeat(ids[:, None], 3, 1), dir=np.zeros((n, 3)), wgt=ids,
                                          time=np.zeros(n), E=np.zeros(n), G=np.ones(n, np.int32),
                                          brood_id=np.arange(1, n + 1, dtype=np.int32))))
    out = [None] * 3
    th = [threading.Thread(target=lambda r=r: out.__setitem__(r, replicas.load_balance(comms[r], banks[r], pops[r],
                                                                                        12, pops)))
          for r in range(3)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    assert [b.n for b in out] == [4, 4, 4]
    assert np.array_equal(np.concatenate([b["wgt"] for b in out]), np.arange(12, dtype=np.float64))


def _balance(pops, tot):
    comms = replicas.ThreadComm.group(len(pops))
    start = np.cumsum([0] + pops)
    out, errs = [None] * len(pops), []

    def body(r):
        n = pops[r]
        ids = np.arange(start[r], start[r] + n, dtype=np.float64)
        bank = abi.HostBank(n, dict(r=np.repeat(ids[:, None], 3, 1), dir=np.zeros((n, 3)), wgt=ids,
                                    time=np.zeros(n), E=np.zeros(n), G=np.ones(n, np.int32),
                                    brood_id=np.ones(n, np.int32)))
        try:
            out[r] = replicas.load_balance(comms[r], bank, n, tot, pops)
        except RuntimeError as e:
            errs.append(e)
            comms[r].sh.barrier.abort()
            for q in comms[r].sh.boxes.values():        # wake a neighbour blocked on a receive
                q.put(np.zeros((0, 11)))

    th = [threading.Thread(target=body, args=(r,)) for r in range(len(pops))]
    for t in th:
        t.start()
    for t in th:
        t.join(timeout=60)
    return out, errs


def test_load_balance_from_a_middle_rank_holding_everything():
    """All 12 particles on the middle one of 3 ranks: it passes 4 up and 4 down in one exchange."""
    out, errs = _balance([0, 12, 0], 12)
    assert not errs
    assert [b.n for b in out] == [4, 4, 4]
    assert np.array_equal(np.concatenate([b["wgt"] for b in out]), np.arange(12, dtype=np.float64))


def test_load_balance_refuses_what_neighbour_passes_cannot_settle():
    """All particles on the first of 3 ranks: the second would have to pass particles up before it
    has received them.  SCONE's nearest-neighbour scheme assumes shares near the workshare (what
    normSize_Repr leaves); here the exchange fails with an error instead of passing garbage."""
    out, errs = _balance([12, 0, 0], 12)
    assert errs and "more particles than it holds" in str(errs[0])
