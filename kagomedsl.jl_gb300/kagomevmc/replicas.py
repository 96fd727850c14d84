"""Independent-replica scale-out (one process per GPU, no data-path collective).

Walker chains are independent, so N GPUs run N replicas of a batch with
distinct seeds.  The only exchange is a final reduction of a few scalars
per rank: the slowest rank's elapsed time and the summed counts / energy
sums.  The transport is the caller's: ``reduce_run`` takes an ``allreduce``
callable (bench.py passes one over torch.distributed, NCCL on GPUs and gloo
on CPU; a Julia host would pass MPI's), so this package needs no
communication library.
"""
from __future__ import annotations

SEED_STRIDE = 104729  # a prime: replica r draws from key seed + r * SEED_STRIDE


def shard(total: int, rank: int, world: int):
    """Contiguous split of `total` walkers: (first, count) for `rank`."""
    base, extra = divmod(total, world)
    first = rank * base + min(rank, extra)
    return first, base + (1 if rank < extra else 0)


def replica_seed(seed: int, rank: int) -> int:
    return (int(seed) + SEED_STRIDE * int(rank)) & 0xFFFFFFFFFFFFFFFF


def reduce_run(elapsed_ms: float, sums: dict, allreduce=None) -> tuple:
    """Max of elapsed_ms and sum of every entry of `sums` over all ranks.

    allreduce(values, op) -> list of floats, op "max" or "sum", reduces a
    list of floats over every rank; None (one process) returns the inputs.
    Returns (elapsed_ms_max, sums_total).
    """
    keys = sorted(sums)
    if allreduce is None:
        return float(elapsed_ms), {k: float(sums[k]) for k in keys}
    t = allreduce([float(elapsed_ms)], "max")
    s = allreduce([float(sums[k]) for k in keys], "sum")
    return float(t[0]), {k: float(v) for k, v in zip(keys, s)}
