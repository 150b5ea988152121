"""Splitting a cycle's histories over processes, as SCONE does with MPI.

Histories are independent within a cycle, so N processes (one per GPU) each transport a contiguous
share of the population with no exchange inside the cycle: process r takes getWorkshare(N) histories
starting after getOffset(N) (SharedModules/mpi_func.f90:133-159), its master RNG strided by that
offset once at the start (fixedSourcePhysicsPackage_class.f90:131), and every cycle strides by the
total population.  The union of all processes' histories is then the single-process run's, history
by history.  A fixed-source run exchanges only the sum of the score memory
(scoreMemory%collectDistributed, Tallies/scoreMemory_class.f90:443-467).

An eigenvalue cycle exchanges three things between its gen loop and the next
(eigenPhysicsPackage_class.f90:203-303): the running scores of the synchronised tallies, the k
attachment among them (scoreMemory%reduceBins, :403-432), summed before they are closed; the
fission-site counts of all processes, from which every process normalises its own sites against the
same threshold (normSize_Repr, ParticleObjects/particleDungeon_class.f90:431-590, sg_normalise_shard);
and particles passed between neighbouring processes until each holds its workshare of the next
cycle (loadBalancing, :593-700).  The next cycle's banks, concatenated in process order, are the
single-process run's.

The exchanges go through a small communicator: `TorchComm` over torch.distributed (CPU tensors, so
the gloo backend; one process per GPU), or `ThreadComm` for processes emulated as threads of one
program.  Neither moves device memory: the banks cross on the host, as the C ABI's banks do.
"""
import queue
import threading

import numpy as np

from . import abi

RNG_STRIDE = 152917


def workshare(n, rank, world):
    """getWorkshare: (N + rank) / worldSize."""
    return (n + rank) // world


def offset(n, rank, world):
    """getOffset: N / worldSize * rank + max(0, mod(N, worldSize) + rank - worldSize)."""
    return n // world * rank + max(0, n % world + rank - world)


def rank_master(master, n, rank, world, skip):
    """The master state process `rank` starts from: master strided by its offset.  `skip` is the
    RNG skip-ahead (gpu.rng_skip or the oracle's)."""
    return skip(master, RNG_STRIDE * offset(n, rank, world))


def fixed_source_shard(op, admin, n, rank, world, master, cycles, skip):
    """`cycles` fixed-source cycles of this process's share on a transport operator `op` (the GPU
    handle or the oracle); returns the final master state."""
    share = workshare(n, rank, world)
    m = rank_master(master, n, rank, world, skip)
    for _ in range(cycles):
        m, _ = op.fixed_source_cycle(admin, share, m, total=n)
    return m


# ------------------------------------------------------------------ communicators
class TorchComm:
    """The exchanges of an eigenvalue cycle over torch.distributed (an initialised process group
    whose backend moves CPU tensors, e.g. gloo)."""

    def __init__(self, group=None):
        import torch.distributed as dist
        self.dist, self.group = dist, group
        self.rank, self.world = dist.get_rank(group), dist.get_world_size(group)

    def allreduce(self, x):
        import torch
        t = torch.from_numpy(np.array(x, dtype=np.float64, copy=True))
        self.dist.all_reduce(t, group=self.group)
        return t.numpy()

    def allgather(self, v):
        import torch
        out = [torch.zeros(1, dtype=torch.int64) for _ in range(self.world)]
        self.dist.all_gather(out, torch.tensor([int(v)], dtype=torch.int64), group=self.group)
        return [int(t.item()) for t in out]

    def send(self, arr, dst):
        import torch
        self.dist.send(torch.from_numpy(np.ascontiguousarray(arr)), dst, group=self.group)

    def recv(self, src, shape):
        import torch
        t = torch.zeros(shape, dtype=torch.float64)
        self.dist.recv(t, src, group=self.group)
        return t.numpy()


class ThreadComm:
    """Processes emulated as threads of one program: `ThreadComm.group(world)` returns one
    communicator per rank.  Sums run in rank order, so every rank gets the same value."""

    class _Shared:
        def __init__(self, world):
            self.world = world
            self.barrier = threading.Barrier(world)
            self.slots = [None] * world
            self.boxes = {(a, b): queue.Queue() for a in range(world) for b in range(world)}

    def __init__(self, shared, rank):
        self.sh, self.rank, self.world = shared, rank, shared.world

    @classmethod
    def group(cls, world):
        sh = cls._Shared(world)
        return [cls(sh, r) for r in range(world)]

    def _gather(self, v):
        self.sh.barrier.wait()
        self.sh.slots[self.rank] = v
        self.sh.barrier.wait()
        out = list(self.sh.slots)
        self.sh.barrier.wait()
        return out

    def allreduce(self, x):
        parts = self._gather(np.array(x, dtype=np.float64, copy=True))
        tot = parts[0].copy()
        for p in parts[1:]:
            tot = tot + p
        return tot

    def allgather(self, v):
        return [int(x) for x in self._gather(int(v))]

    def send(self, arr, dst):
        self.sh.boxes[(self.rank, dst)].put(np.array(arr, copy=True))

    def recv(self, src, shape):
        a = self.sh.boxes[(src, self.rank)].get(timeout=600)
        if a.shape != tuple(shape):
            raise RuntimeError(f"recv: expected {shape} from rank {src}, got {a.shape}")
        return a


# ------------------------------------------------------------------ eigenvalue cycles
_COLS = 11   # r(3), dir(3), wgt, time, E, G, brood_id


def _pack(bank, n):
    a = bank.a
    return np.concatenate([a["r"][:n], a["dir"][:n], a["wgt"][:n, None], a["time"][:n, None], a["E"][:n, None],
                           a["G"][:n, None].astype(np.float64), a["brood_id"][:n, None].astype(np.float64)], axis=1)


def _unpack(x):
    n = x.shape[0]
    return abi.HostBank(n, dict(r=x[:, 0:3], dir=x[:, 3:6], wgt=x[:, 6], time=x[:, 7], E=x[:, 8],
                                G=x[:, 9].astype(np.int32), brood_id=x[:, 10].astype(np.int32)))


def load_balance(comm, bank, n, tot_pop, pops):
    """particleDungeon%loadBalancing (particleDungeon_class.f90:593-700): after normalisation
    process r holds sites pops[:r].sum() .. pops[:r+1].sum() of the concatenated bank; particles go
    to or come from the neighbours until it holds getOffset(tot_pop) .. the next process's offset.
    The top end is settled first, then the bottom end, as SCONE does, so blocking exchanges resolve
    from the last process down."""
    rank, world = comm.rank, comm.world
    x = _pack(bank, n)
    lo = sum(pops[:rank])
    hi = lo + pops[rank]
    t_lo = offset(tot_pop, rank, world)
    t_hi = tot_pop if rank == world - 1 else offset(tot_pop, rank + 1, world)
    ex = hi - t_hi
    if ex > x.shape[0]:
        raise RuntimeError("loadBalancing: a process would pass on more particles than it holds")
    if ex > 0:
        comm.send(x[x.shape[0] - ex:], rank + 1)
        x = x[:x.shape[0] - ex]
    elif ex < 0:
        x = np.concatenate([x, comm.recv(rank + 1, (-ex, _COLS))])
    ex = lo - t_lo
    if -ex > x.shape[0]:
        raise RuntimeError("loadBalancing: a process would pass on more particles than it holds")
    if ex < 0:
        comm.send(x[:-ex], rank - 1)
        x = x[-ex:]
    elif ex > 0:
        x = np.concatenate([comm.recv(rank - 1, (ex, _COLS)), x])
    return _unpack(x)


def eigen_shard_init(op, comm, tot_pop, master, k0=1.0):
    """This process's share of the initial fission source (generateInitialState,
    eigenPhysicsPackage_class.f90:348-366): particle i of the population from master + stride(i),
    the process taking getWorkshare after getOffset.  Returns (bank, master, k0), master strided by
    tot_pop as the single-process run leaves it."""
    op.eigen_init(tot_pop, master, k0)
    full, _ = op.eigen_bank(tot_pop)
    o = offset(tot_pop, comm.rank, comm.world)
    share = workshare(tot_pop, comm.rank, comm.world)
    bank = abi.HostBank(share, {k: v[o:o + share].copy() for k, v in full.a.items()})
    m, _ = op.eigen_state()
    return bank, m, k0


def eigen_cycle_shard(op, comm, admin, atch, bank, tot_pop, master, k_new, k_end, skip, sync=(), next_cap=None):
    """One eigenvalue cycle (eigenPhysicsPackage_class.f90:203-303) of this process's share `bank`
    on a transport operator `op` (the GPU handle or the oracle).  `master` is the master process's
    RNG state, `k_new` the k the gen loop uses and `k_end` end%k_eff; `atch` is the k attachment,
    whose scores are summed over processes before it closes, as are those of the admins in `sync`
    (tallies with mpiSync).  Every admin must close each cycle (batch size 1).  Returns
    (bank, master, k, stats): the next share after normalisation and load balancing, the master
    strided as in the single-process run, and k from the summed attachment."""
    rank, world = comm.rank, comm.world
    n = bank.n
    start_w = float(np.sum(bank.a["wgt"][:n]))
    op.tally_cycle_start(admin, start_w)
    rm = skip(master, RNG_STRIDE * offset(tot_pop, rank, world))
    cap = next_cap or max(4 * n, 16)
    nxt, st = op.transport_bank(admin, bank, rm, k_eff=k_new, next_cap=cap)
    master = skip(master, RNG_STRIDE * (tot_pop + 1))                       # :257
    end_w = float(comm.allreduce([st.end_weight])[0])
    for a in [atch] + [x for x in sync if x != atch]:                       # reduceBins over processes
        op.set_scores(a, comm.allreduce(op.get_scores(a)))
    op.tally_cycle_end(admin, end_w, k_end)                                 # :261
    pops = comm.allgather(st.n_next)
    tot_sites = sum(pops)
    if tot_sites == 0:
        raise RuntimeError("normSize: empty fission bank")
    normed, m = op.normalise_shard(nxt, st.n_next, sum(pops[:rank]), tot_sites, tot_pop, master,
                                   max(cap, 2 * tot_pop // world + 16))    # :269
    new_pops = comm.allgather(m)
    if sum(new_pops) != tot_pop:
        raise RuntimeError("normSize: normalisation failed")
    share = load_balance(comm, normed, m, tot_pop, new_pops)
    master = skip(master, RNG_STRIDE)                                       # stride(1), :275
    k, _ = op.keff(atch)                                                    # :289-298
    return share, master, k, st
