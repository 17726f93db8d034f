"""Target sharding across ranks (one process per GPU).

Targets are independent once the sources are known, so a multi-GPU transfer
gives each rank a contiguous slice of the targets (in the caller's order or
in Morton order) and the whole source cloud; each rank builds its own tree
and operator, and no data-path collective is needed.  The caller gathers the
target slices if it needs them in one place.
"""
from __future__ import annotations


def target_shard(n_targets: int, rank: int, world: int) -> tuple[int, int]:
    """[begin, end) of rank's slice: sizes differ by at most one, in rank order."""
    if world < 1 or not (0 <= rank < world):
        raise ValueError("rank must lie in [0, world)")
    if n_targets < 0:
        raise ValueError("n_targets must be >= 0")
    base, extra = divmod(n_targets, world)
    begin = rank * base + min(rank, extra)
    return begin, begin + base + (1 if rank < extra else 0)
