"""Multi-process split of a cycle (SCONE's MPI getWorkshare/getOffset) with world size 2 over gloo,
on the CPU: each rank transports its share with the oracle, the score memory is summed across
ranks (the only exchange), and the sum equals the single-process run."""
import os
import socket

import numpy as np
import pytest

from scone_gb300 import replicas


def test_shares_partition_the_population():
    for n in (1, 2, 7, 1000, 100001):
        for world in (1, 2, 3, 4, 8):
            shares = [replicas.workshare(n, r, world) for r in range(world)]
            offs = [replicas.offset(n, r, world) for r in range(world)]
            assert sum(shares) == n
            assert offs[0] == 0
            for r in range(1, world):
                assert offs[r] == offs[r - 1] + shares[r - 1]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, n, cycles, out):
    import torch
    import torch.distributed as dist
    from oracle import oracle
    from scone_gb300 import abi, problems
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    p = problems.infinite_medium_2g()
    o = oracle.Oracle(p, transport=abi.TRANSPORT_DT)
    a = o.upload_tally(p.tallies["flux"])
    replicas.fixed_source_shard(o, a, n, rank, world, 4242, cycles, oracle.rng_skip)
    csum = torch.tensor(o.bins(a)[:, 1].copy())
    dist.all_reduce(csum, op=dist.ReduceOp.SUM)
    if rank == 0:
        np.save(out, csum.numpy())
    dist.destroy_process_group()


def test_two_ranks_sum_to_one(tmp_path):
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    from oracle import oracle
    from scone_gb300 import abi, problems
    oracle.build()
    n, cycles = 3001, 3
    out = str(tmp_path / "csum.npy")
    mp.start_processes(_rank, args=(2, _free_port(), n, cycles, out), nprocs=2, join=True, start_method="spawn")
    summed = np.load(out)
    p = problems.infinite_medium_2g()
    o = oracle.Oracle(p, transport=abi.TRANSPORT_DT)
    a = o.upload_tally(p.tallies["flux"])
    m = 4242
    for _ in range(cycles):
        m, _ = o.fixed_source_cycle(a, n, m)
    single = o.bins(a)[:, 1]
    np.testing.assert_allclose(summed, single, rtol=1e-12, atol=0)
