"""GPU kNN / radius search against the oracle: neighbour sets bit-exact.

Rows are compared entry by entry: the GPU returns the min(k, n_src) smallest
(d2, source index) keys in ascending order, as the oracle does.
"""
import numpy as np
import pytest
import torch

import datatransferkit_gb300 as dtk
from datatransferkit_gb300 import synthetic as syn
from oracle import cpu

pytestmark = pytest.mark.gpu


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def gpu_knn(src, tgt, k, layout="right"):
    s, t = dev(src), dev(tgt)
    if layout == "left":  # LayoutLeft: (i, d) at d*n + i
        s = s.t().contiguous().t()
        t = t.t().contiguous().t()
    off, idx = dtk.knn_search(s, t, k)
    return off.cpu().numpy(), idx.cpu().numpy()


@pytest.mark.parametrize("k", [1, 4, 10, 20, 32])
def test_knn_uniform_bit_exact(k):
    src = syn.uniform_points(20000, 31)
    tgt = syn.uniform_points(5000, 32)
    off, idx = gpu_knn(src, tgt, k)
    o2, i2, _ = cpu.knn(src, tgt, k)
    assert np.array_equal(off, o2)
    assert np.array_equal(idx, i2)


def test_knn_layout_left_matches_layout_right():
    src = syn.uniform_points(3000, 1)
    tgt = syn.uniform_points(700, 2)
    a = gpu_knn(src, tgt, 16, "right")
    b = gpu_knn(src, tgt, 16, "left")
    assert np.array_equal(a[1], b[1])


def test_knn_ties_grid_line_duplicates():
    src = syn.grid_points((40, 40, 1), (0.0, 0.0, 0.0))
    tgt = np.concatenate([syn.grid_points((6, 6, 1), (17.5, 17.5, 0.0)),
                          syn.grid_points((3, 3, 1), (19.0, 19.0, 0.0))])
    for k in (1, 4, 10, 32):
        off, idx = gpu_knn(src, tgt, k)
        assert np.array_equal(idx, cpu.knn(src, tgt, k)[1]), k
    src = np.concatenate([syn.uniform_points(500, 3)] * 3)  # every point three times
    tgt = syn.uniform_points(300, 4)
    assert np.array_equal(gpu_knn(src, tgt, 32)[1], cpu.knn(src, tgt, 32)[1])


def test_knn_small_and_degenerate_clouds():
    rng = np.random.default_rng(5)
    for n_src in (1, 2, 5, 31, 32, 33, 64, 65):
        src = rng.random((n_src, 3))
        tgt = rng.random((50, 3)) * 2 - 0.5  # some targets outside the source box
        for k in (1, 4, 32):
            off, idx = gpu_knn(src, tgt, k)
            o2, i2, _ = cpu.knn(src, tgt, k)
            assert np.array_equal(off, o2) and np.array_equal(idx, i2), (n_src, k)
    flat = np.zeros((1000, 3))
    flat[:, :2] = rng.random((1000, 2))
    tgt = rng.random((200, 3))
    assert np.array_equal(gpu_knn(flat, tgt, 20)[1], cpu.knn(flat, tgt, 20)[1])
    same = np.ones((100, 3))  # all sources identical
    assert np.array_equal(gpu_knn(same, tgt, 10)[1], cpu.knn(same, tgt, 10)[1])


def test_knn_clustered_sources():
    src = syn.gaussian_mixture(30000, 7)
    tgt = syn.uniform_points(4000, 8)
    assert np.array_equal(gpu_knn(src, tgt, 32)[1], cpu.knn(src, tgt, 32)[1])


def test_knn_empty_targets():
    off, idx = gpu_knn(syn.uniform_points(10, 1), np.zeros((0, 3)), 4)
    assert off.tolist() == [0] and idx.size == 0


def test_knn_large_coordinates_offset():
    src = syn.uniform_points(5000, 9) * 1e-3 + 1e6
    tgt = syn.uniform_points(500, 10) * 1e-3 + 1e6
    assert np.array_equal(gpu_knn(src, tgt, 20)[1], cpu.knn(src, tgt, 20)[1])


def test_knn_near_ties_resolved_exactly():
    # shells of sources whose distances to their centre agree to ~1e-9
    # (relative): the 32-bit keys of the sorting networks collide and the
    # exact network decides; the centres and their twins 1e-12 away run as
    # consecutive, seeded queries
    rng = np.random.default_rng(12)
    centres = 0.2 + 0.6 * rng.random((40, 3))
    parts = []
    for c in centres:
        u = rng.standard_normal((120, 3))
        u /= np.linalg.norm(u, axis=1)[:, None]
        r = 0.01 * (1 + 1e-9 * rng.integers(0, 50, 120))
        parts.append(c + u * r[:, None])
    src = np.concatenate(parts + [syn.uniform_points(20000, 13)])
    tgt = np.concatenate([centres, centres + 1e-12 * rng.standard_normal(centres.shape)])
    for k in (16, 32):
        assert np.array_equal(gpu_knn(src, tgt, k)[1], cpu.knn(src, tgt, k)[1]), k


def test_knn_deep_and_degenerate_trees():
    # the leaves are Morton cells of at most 32 points: runs of identical codes
    # (split by position), a geometric sequence (a deep key trie), a cluster
    # of extent 1e-9 inside a unit cloud, and targets on, near and far from all
    rng = np.random.default_rng(14)
    geo = np.zeros((400, 3))
    geo[:, 0] = 2.0 ** -np.arange(400) * 0.9
    dup = np.concatenate([np.tile([[0.3, 0.3, 0.3]], (700, 1)), np.tile([[0.7, 0.2, 0.9]], (45, 1))])
    tiny = 0.5 + 1e-9 * rng.random((300, 3))
    src = np.concatenate([geo, dup, tiny, rng.random((6000, 3))])
    tgt = np.concatenate([src[::37], [[0.3, 0.3, 0.3], [0.5, 0.5, 0.5], [0.0, 0.0, 0.0], [3.0, -2.0, 0.5]],
                          rng.random((500, 3))])
    for k in (1, 7, 32):
        assert np.array_equal(gpu_knn(src, tgt, k)[1], cpu.knn(src, tgt, k)[1]), k


@pytest.mark.parametrize("kind", ["uniform", "clustered", "duplicates"])
def test_knn_chunked_queries_bit_exact(kind):
    """300k targets: warps take chunks of Morton-consecutive queries, and each
    chunk's later queries scan the leaf list collected after its first query
    (they traverse the tree when the list overflowed, and search again when
    the list's bound is not proven): clustered sources leave uniform targets
    far from most leaves, duplicates give zero k-th distances."""
    rng = np.random.default_rng(21)
    n = 300_000
    if kind == "uniform":
        src, tgt = syn.uniform_points(400_000, 22), syn.uniform_points(n, 23)
    elif kind == "clustered":
        src, tgt = syn.gaussian_mixture(400_000, 24), syn.uniform_points(n, 25)
    else:
        spots = rng.random((40, 3))
        src = np.concatenate([syn.uniform_points(200_000, 26), np.repeat(spots, 100, axis=0)])
        tgt = np.concatenate([syn.uniform_points(n - 4000, 27), np.repeat(spots, 100, axis=0)])
    assert np.array_equal(gpu_knn(src, tgt, 32)[1], cpu.knn(src, tgt, 32)[1])


def test_radius_sets_bit_exact():
    src = syn.gaussian_mixture(20000, 11)
    tgt = syn.uniform_points(3000, 12)
    r = 0.05
    s, t = dev(src), dev(tgt)
    op = dtk.MovingLeastSquaresOperator(None, s, t, dtk.Wendland(2),
                                        dtk.MultivariatePolynomialBasis(dtk.Linear, 3), radius=r)
    off, idx, _ = op.csr()
    off, idx = off.cpu().numpy(), idx.cpu().numpy()
    o2, i2, _ = cpu.radius(src, tgt, r)
    assert np.array_equal(off, o2)
    for i in range(len(tgt)):
        assert np.array_equal(np.sort(idx[off[i]:off[i + 1]]), np.sort(i2[o2[i]:o2[i + 1]])), i


def test_knn_in_a_cluster_sharing_one_morton_code():
    # 400 sources inside a cube of side 1e-9 (one 30-bit Morton code: the
    # run is split between leaves by position) in a unit cloud, and targets
    # inside the cube, off the sources: a search may only start in a subtree
    # whose cell holds no point outside it, else it would miss the sibling
    # leaves of the same code
    rng = np.random.default_rng(21)
    cube = 0.5 + 1e-9 * rng.random((400, 3))
    src = np.concatenate([rng.random((5000, 3)), cube, rng.random((3000, 3))])
    tgt = np.concatenate([0.5 + 1e-9 * rng.random((300, 3)), rng.random((200, 3))])
    for k in (1, 4, 32):
        assert np.array_equal(gpu_knn(src, tgt, k)[1], cpu.knn(src, tgt, k)[1]), k
