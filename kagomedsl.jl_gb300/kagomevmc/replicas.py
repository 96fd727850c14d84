"""Independent-replica scale-out (one process per GPU, no data-path collective).

Walker chains are independent, so N GPUs run N replicas of a batch with
distinct seeds.  The only exchange is a final reduction of a few scalars
per rank: the slowest rank's elapsed time and the summed counts / energy
sums.  torch.distributed carries that reduction (NCCL on GPUs, gloo on CPU).
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


def reduce_run(elapsed_ms: float, sums: dict, device=None) -> tuple:
    """Max of elapsed_ms and sum of every entry of `sums` over all ranks.

    Returns (elapsed_ms_max, sums_total).  With no process group (one
    process) it returns its inputs.
    """
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(elapsed_ms), {k: float(v) for k, v in sums.items()}
    keys = sorted(sums)
    dev = device if device is not None else "cpu"
    t = torch.tensor([float(elapsed_ms)], dtype=torch.float64, device=dev)
    s = torch.tensor([float(sums[k]) for k in keys], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(s, op=dist.ReduceOp.SUM)
    return float(t[0]), {k: float(v) for k, v in zip(keys, s.tolist())}
