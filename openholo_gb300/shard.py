"""Work split across ranks for N > 1 GPUs of one node.

One process per GPU, each generating its own frames: the units of the
hologram path (frames, and the frames of a batch) are independent, so ranks
share no data and no collective runs on the data path.  The only
cross-rank step is the timing reduction (the slowest rank's time).
"""
from __future__ import annotations


def shard_range(n: int, rank: int, world: int) -> tuple[int, int]:
    """[lo, hi) of n units for `rank` of `world`: contiguous blocks whose
    sizes differ by at most one (the first n % world ranks take one more)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside a world of {world}")
    if n < 0:
        raise ValueError("negative unit count")
    base, extra = divmod(n, world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def shard(units, rank: int, world: int):
    """This rank's contiguous share of a sequence of units."""
    lo, hi = shard_range(len(units), rank, world)
    return units[lo:hi]


def rank_seed(base: int, rank: int) -> int:
    """Seed of a rank's synthetic inputs: distinct frames per rank (weak scaling)."""
    return base + rank


def max_over_ranks(value: float, dist=None, device=None) -> float:
    """The largest `value` over all ranks of the default process group (the
    benchmark's slowest-rank time); `value` itself without a group."""
    if dist is None or not dist.is_available() or not dist.is_initialized():
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
