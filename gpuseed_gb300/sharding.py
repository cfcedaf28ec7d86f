"""Read sharding across processes (one GPU each) -- no collective on the data path.

The reference processes reads in independent batches on one GPU
(seed_gen.cu:2910-3790) and numbers them from 1 across batches (:3632).  Across
N processes the same holds: process r takes a contiguous range of reads, seeds
it against its own replica of the index, and writes its records with the read
numbers of its range; concatenating the shards in rank order gives exactly the
single-process output.  Only timings are reduced across ranks (max of the
elapsed times, sum of the reads).
"""
from __future__ import annotations


def shard_range(n_reads: int, rank: int, world: int) -> tuple[int, int]:
    """Contiguous [lo, hi) of the reads owned by `rank`; sizes differ by at most one."""
    if world <= 0 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside world of {world}")
    base, extra = divmod(n_reads, world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def first_read_number(n_reads: int, rank: int, world: int) -> int:
    """1-based number of the first read of `rank`'s shard in the records."""
    return shard_range(n_reads, rank, world)[0] + 1


def reduce_timing(dist, elapsed_s: float, reads: int, device=None) -> tuple[float, float]:
    """(max elapsed over ranks, total reads over ranks); plain values without a group."""
    if dist is None:
        return elapsed_s, float(reads)
    import torch
    t = torch.tensor([elapsed_s], dtype=torch.float64, device=device)
    n = torch.tensor([float(reads)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(n, op=dist.ReduceOp.SUM)
    return float(t.item()), float(n.item())
