"""Splitting a cycle's histories over processes, as SCONE does with MPI.

Histories are independent within a cycle, so N processes (one per GPU) each transport a contiguous
share of the population with no exchange inside the cycle: process r takes getWorkshare(N) histories
starting after getOffset(N) (SharedModules/mpi_func.f90:133-159), its master RNG strided by that
offset once at the start (fixedSourcePhysicsPackage_class.f90:131), and every cycle strides by the
total population.  The union of all processes' histories is then the single-process run's, history
by history; the only exchange is the sum of the score memory (scoreMemory%collectDistributed,
Tallies/scoreMemory_class.f90:443-467).
"""
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
