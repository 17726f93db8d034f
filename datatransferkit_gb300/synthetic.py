"""Seeded synthetic point clouds and fields of the MLS transfer workloads.

All generators run on the host with numpy's PCG64 (``default_rng(seed)``) so
that every machine sees identical bits; callers copy to the device.

Workloads (sizes, seeds):
  plain_cpu     10,000 sources / 10,000 targets U[0,1]^3 (seeds 1, 2),
                Quadratic3, Wendland<2>, k = 20
  fp64_scale    2,000,000 sources U[0,1]^3 (seed 3); 126^3 targets on a
                jittered grid ((i + 0.5 + u) / 126, u ~ U[-0.25, 0.25], seed 4),
                Quadratic3, Wendland<2>, k = 32
  batched       256 problems, sizes log-uniform in [1e3, 1e5] (seed 5);
                sources from an 8-cluster Gaussian mixture (sigma log-uniform
                in [0.02, 0.2], clipped to [0,1]^3, seed 5 + problem id),
                targets U[0,1]^3 of equal count, radius search r = 0.05,
                Linear3 / Quadratic3 alternating by problem id, Wendland<2>
  mixed         8,000,000 sources / 8,000,000 targets U[0,1]^3 (seeds 6, 7),
                Quadratic3, Wendland<4>, k = 32; smooth field and a tanh
                front of width 0.01
  adjoint       1,000,000 sources / 1,000,000 targets U[0,1]^3 (seeds 8, 9),
                Quadratic3, Wendland<2>, k = 32
"""
from __future__ import annotations

import numpy as np


def uniform_points(n: int, seed: int) -> np.ndarray:
    return np.random.default_rng(seed).random((n, 3))


def jittered_grid(m: int, seed: int, jitter: float = 0.25) -> np.ndarray:
    rng = np.random.default_rng(seed)
    i = np.arange(m, dtype=np.float64)
    g = np.stack(np.meshgrid(i, i, i, indexing="ij"), axis=-1).reshape(-1, 3)
    u = rng.uniform(-jitter, jitter, size=g.shape)
    return (g + 0.5 + u) / m


def smooth_field(p: np.ndarray) -> np.ndarray:
    """f(x, y, z) = sin(2 pi x) cos(2 pi y) + z^2."""
    return np.sin(2 * np.pi * p[:, 0]) * np.cos(2 * np.pi * p[:, 1]) + p[:, 2] ** 2


def front_field(p: np.ndarray, width: float = 0.01) -> np.ndarray:
    """g(x, y, z) = tanh((x - 0.5) / width)."""
    return np.tanh((p[:, 0] - 0.5) / width)


def gaussian_mixture(n: int, seed: int, clusters: int = 8, sigma=(0.02, 0.2)) -> np.ndarray:
    rng = np.random.default_rng(seed)
    centers = rng.random((clusters, 3))
    sig = np.exp(rng.uniform(np.log(sigma[0]), np.log(sigma[1]), clusters))
    lab = rng.integers(0, clusters, n)
    p = centers[lab] + rng.standard_normal((n, 3)) * sig[lab, None]
    return np.clip(p, 0.0, 1.0)


def batched_problems(n_problems: int = 256, seed: int = 5, lo: float = 1e3, hi: float = 1e5):
    """List of dicts (src, tgt, basis id) of the batched uneven workload."""
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(lo), np.log(hi), n_problems)).astype(np.int64)
    out = []
    for p, n in enumerate(sizes):
        src = gaussian_mixture(int(n), seed + p)
        tgt = np.random.default_rng(10_000 + seed + p).random((int(n), 3))
        out.append(dict(src=src, tgt=tgt, basis=1 if p % 2 == 0 else 2))
    return out


def cluster_problem(n_targets: int, n_in_radius: int, radius: float, rank: int = 0,
                    seed: int = 0):
    """Isolated clusters around each target (tstMeshfreeOperators.cpp:41-77 layout).

    Cluster i is centred at i * ceil(4 radius) (+ an offset per rank); its
    target lies within +-radius/2 of the centre and its n_in_radius sources
    within +-radius, so each target's nearest n_in_radius sources are its own.
    """
    rng = np.random.default_rng(seed)
    offset = n_targets * radius * 10.0 * rank
    tgt = np.zeros((n_targets, 3))
    src = np.zeros((n_targets * n_in_radius, 3))
    for i in range(n_targets):
        c = i * np.ceil(4 * radius) + offset
        tgt[i] = c + 0.5 * rng.uniform(-radius, radius, 3)
        src[i * n_in_radius:(i + 1) * n_in_radius] = c + rng.uniform(-radius, radius, (n_in_radius, 3))
    return src, tgt


def grid_points(n, offset) -> np.ndarray:
    """Integer grid n[0] x n[1] x n[2] shifted by offset (tstMeshfreeOperators.cpp:105-127)."""
    pts = [(offset[0] + i, offset[1] + j, offset[2] + k)
           for i in range(n[0]) for j in range(n[1]) for k in range(n[2])]
    return np.asarray(pts, dtype=np.float64).reshape(-1, 3)


def polynomial_of_basis(size: int):
    """The test polynomials of tstMeshfreeOperators.cpp:178-199 by basis size."""
    if size == 1:
        return lambda p: np.full(len(p), 3.0)
    if size == 4:
        return lambda p: 4 + 2 * p[:, 0] + 3 * p[:, 1] - 2 * p[:, 2]
    return lambda p: (2 + 3 * p[:, 0] - 5 * p[:, 1] + 2 * p[:, 2] + 3 * p[:, 0] ** 2
                      + 4 * p[:, 0] * p[:, 1] - 2 * p[:, 0] * p[:, 2] + p[:, 1] ** 2
                      - 3 * p[:, 1] * p[:, 2] + 4 * p[:, 2] ** 2)
