"""Target sharding across ranks (one process per GPU).

Targets are independent once the sources are known, so a multi-GPU transfer
gives each rank one contiguous Morton-ordered slice of the targets and the
whole source cloud; each rank builds its own tree and operator, and no
data-path collective is needed.  A slice is contiguous in space (a run of the
Morton curve), so each rank's queries touch a compact region of the source
tree.  Within a slice the targets keep the caller's order, so with one rank
the shard is the whole target set in its own order.  ``assemble`` puts the
slices' results back in the caller's order, for a caller that needs them in
one place (the gather is the caller's, not the transfer's).
"""
from __future__ import annotations

import numpy as np

_BITS = 21  # bits per axis of the 63-bit Morton codes


def slice_bounds(n: int, rank: int, world: int) -> tuple[int, int]:
    """[begin, end) of rank's share of n items: sizes differ by at most one, in rank order."""
    if world < 1 or not (0 <= rank < world):
        raise ValueError("rank must lie in [0, world)")
    if n < 0:
        raise ValueError("n must be >= 0")
    base, extra = divmod(n, world)
    begin = rank * base + min(rank, extra)
    return begin, begin + base + (1 if rank < extra else 0)


def _spread3(v: np.ndarray) -> np.ndarray:
    """Bits 0..20 of v moved to bits 0, 3, 6, ..., 60."""
    v = v.astype(np.uint64) & np.uint64(0x1FFFFF)
    v = (v | (v << np.uint64(32))) & np.uint64(0x1F00000000FFFF)
    v = (v | (v << np.uint64(16))) & np.uint64(0x1F0000FF0000FF)
    v = (v | (v << np.uint64(8))) & np.uint64(0x100F00F00F00F00F)
    v = (v | (v << np.uint64(4))) & np.uint64(0x10C30C30C30C30C3)
    v = (v | (v << np.uint64(2))) & np.uint64(0x1249249249249249)
    return v


def morton_codes(points: np.ndarray) -> np.ndarray:
    """63-bit Morton codes of an (n, 3) point array in its own bounding box."""
    p = np.asarray(points, dtype=np.float64)
    if p.ndim != 2 or p.shape[1] != 3:
        raise ValueError("points must be an (n, 3) array")
    if len(p) == 0:
        return np.zeros(0, np.uint64)
    if not np.all(np.isfinite(p)):
        raise ValueError("point coordinates must be finite")
    lo, hi = p.min(0), p.max(0)
    ext = np.where(hi > lo, hi - lo, 1.0)
    top = (1 << _BITS) - 1
    q = np.clip(np.floor((p - lo) / ext * top), 0, top).astype(np.uint64)
    return (_spread3(q[:, 0]) << np.uint64(2)) | (_spread3(q[:, 1]) << np.uint64(1)) | _spread3(q[:, 2])


def target_shard(targets: np.ndarray, rank: int, world: int) -> np.ndarray:
    """Indices (ascending) of the targets in rank's Morton-ordered slice.

    The targets are ranked by (Morton code, index) and cut into `world`
    contiguous runs whose sizes differ by at most one; every rank computes
    the same cut from the same target array, so the shards partition the
    targets with no communication.
    """
    n = len(targets)
    b, e = slice_bounds(n, rank, world)
    if world == 1:
        return np.arange(n, dtype=np.int64)
    order = np.argsort(morton_codes(targets), kind="stable")
    return np.sort(order[b:e])


def assemble(parts, shards, n: int) -> np.ndarray:
    """The full (n, ...) result from every rank's part and shard indices."""
    parts = [np.asarray(p) for p in parts]
    shape = (n,) + parts[0].shape[1:] if parts else (n,)
    dtype = parts[0].dtype if parts else np.float64
    out = np.empty(shape, dtype)
    seen = np.zeros(n, bool)
    for p, s in zip(parts, shards):
        s = np.asarray(s)
        if len(p) != len(s):
            raise ValueError("a part and its shard differ in length")
        if seen[s].any():
            raise ValueError("shards overlap")
        seen[s] = True
        out[s] = p
    if not seen.all():
        raise ValueError("shards do not cover every target")
    return out
