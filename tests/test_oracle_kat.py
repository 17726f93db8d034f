"""The reference's known-answer tests, run on the CPU oracle (pins the oracle).

Ported from packages/Meshfree/test (paths inside the DataTransferKit project):
  tstMeshfreeOperators.cpp:130-448           same_npoints_and_basis, grid, line,
                                              single_point_in_radius
  tstMeshfreeOperatorsSimpleProblem.cpp:113-147  corner_cases
  tstSVD.cpp:67-150                          full_rank, rank_deficient
  tstCompactlySupportedRadialBasisFunctions.cpp:52-108  polynomial_rbf, wrap_rbf
  tstMultivariatePolynomialBasis.cpp:60-84  3D basis values
  tstNearestNeighborOperator.cpp:141-273      k = 1 on structured / mixed clouds
Inputs come from the project's own seeded generators (std::default_random_engine
is implementation-defined); the properties checked and tolerances are the
reference's.
"""
import numpy as np
import pytest
from numpy.polynomial import polynomial as P

from oracle import cpu
from datatransferkit_gb300 import synthetic as syn

BASES = [0, 1, 2]
SIZE = {0: 1, 1: 4, 2: 10}


def rel_close(a, b, tol):
    a, b = np.asarray(a), np.asarray(b)
    assert a.shape == b.shape
    err = np.abs(a - b) / np.maximum(np.abs(b), 1e-300)
    small = np.abs(b) < 1e-300
    assert np.all(np.where(small, np.abs(a - b) <= tol, err <= tol)), (a, b, err.max())


@pytest.mark.parametrize("basis", BASES)
def test_same_npoints_and_basis(basis):
    m = SIZE[basis]
    f = syn.polynomial_of_basis(m)
    src, tgt = syn.cluster_problem(10, m, 0.5, seed=101)
    r = cpu.mls_transfer(src, tgt, f(src), 0, basis)
    rel_close(r["target"], f(tgt), 1e-7)


@pytest.mark.parametrize("basis", BASES)
def test_grid(basis):
    f = syn.polynomial_of_basis(SIZE[basis])
    src = syn.grid_points((40, 40, 1), (0.0, 0.0, 0.0))
    tgt = syn.grid_points((1, 1, 1), (19.0, 19.0, 0.0))
    r = cpu.mls_transfer(src, tgt, f(src), 0, basis)
    rel_close(r["target"], f(tgt), 1e-14)


@pytest.mark.parametrize("basis", BASES)
def test_line(basis):
    f = syn.polynomial_of_basis(SIZE[basis])
    src = syn.grid_points((40, 1, 1), (0.0, 0.0, 0.0))
    tgt = syn.grid_points((39, 1, 1), (0.5, 0.0, 0.0))
    r = cpu.mls_transfer(src, tgt, f(src), 0, basis)
    rel_close(r["target"], f(tgt), 1e-14)


@pytest.mark.parametrize("basis", BASES)
def test_single_point_in_radius(basis):
    f = syn.polynomial_of_basis(SIZE[basis])
    src, tgt = syn.cluster_problem(10, 1, 0.5, seed=102)
    r = cpu.mls_transfer(src, tgt, f(src), 0, basis)
    assert np.all(np.isfinite(r["target"]))


def test_corner_cases():
    r = cpu.mls_transfer(np.array([[1.0, 1, 1], [2.0, 2, 2]]), np.array([[1.5, 1.5, 1.5]]),
                         np.array([255.0, 255.0]), 0, 1)
    rel_close(r["target"], [255.0], 1e-12)
    assert len(r["idx"]) == 2  # nnz per row = min(k, n_src)
    r = cpu.mls_transfer(np.array([[1.0, 1, 1]]), np.zeros((0, 3)), np.array([255.0]), 0, 1)
    assert r["target"].shape == (0,)


def check_identity(mats, pinv, deficient=()):
    prod = np.einsum("bik,bkj->bij", pinv, mats)
    n = mats.shape[1]
    for i in range(n):
        for j in range(n):
            if i == j and i not in deficient:
                rel_close(prod[:, i, i], np.ones(len(mats)), 1e-12)
            else:
                rel_close(prod[:, i, j] + 1, np.ones(len(mats)), 1e-12)


def test_svd_full_rank():
    a = np.random.default_rng(7).uniform(-1000, 1000, (10, 32, 32))
    p, under = cpu.svd_pinv(a)
    assert under == 0
    check_identity(a, p)


def test_svd_rank_deficient():
    a = np.random.default_rng(8).uniform(-1000, 1000, (10, 40, 40))
    a[:, :, 3] = 0.0
    p, under = cpu.svd_pinv(a)
    assert under == 10
    check_identity(a, p, deficient={3})


RBF_POLYS = {
    0: P.polypow([1.0, -1.0], 2),
    1: P.polymul(P.polypow([1.0, -1.0], 4), [1.0, 4.0]),
    2: P.polymul(P.polypow([1.0, -1.0], 6), [3.0, 18.0, 35.0]),
    3: P.polymul(P.polypow([1.0, -1.0], 8), [1.0, 8.0, 25.0, 32.0]),
    4: P.polymul(P.polypow([1.0, -1.0], 4), [4.0, 16.0, 12.0, 3.0]),
    5: P.polymul(P.polypow([1.0, -1.0], 6), [6.0, 36.0, 82.0, 72.0, 30.0, 5.0]),
}


@pytest.mark.parametrize("rbf", sorted(RBF_POLYS))
def test_polynomial_rbf(rbf):
    x = np.arange(10) / 10.0
    rel_close(cpu.rbf(rbf, x), P.polyval(x, RBF_POLYS[rbf]), 1e-8)


def test_buhmann_values_finite_and_unit_at_zero():
    x = np.array([1e-12, 0.25, 0.5, 0.75, 0.9])
    for r in (6, 7, 8):
        v = cpu.rbf(r, x)
        assert np.all(np.isfinite(v))
    assert abs(cpu.rbf(7, np.array([0.0]))[0] - 1.0) < 1e-15
    assert abs(cpu.rbf(8, np.array([0.0]))[0] - 1.0) < 1e-15


def test_wrap_rbf_scaling():
    # RadialBasisFunction<RBF>(radius)(x) = rbf(x / radius): with radius 2, a
    # Wendland<0> weight at distance 1 equals the raw function at 0.5.
    assert cpu.rbf(0, np.array([1.0 / 2.0]))[0] == (1 - 0.5) ** 2


def test_basis_3d():
    b = cpu.basis(2, np.array([[0.0, 1.0, 2.0]]))
    assert np.array_equal(b[0], [1, 0, 1, 2, 0, 0, 0, 1, 2, 4])
    assert np.array_equal(cpu.basis(1, np.array([[0.0, 1.0, 2.0]]))[0], [1, 0, 1, 2])
    assert np.array_equal(cpu.basis(0, np.array([[0.0, 0.0, 0.0]]))[0], [1])


def structured_cloud(L, n, o=(0.0, 0.0, 0.0)):
    pts = np.zeros((n[0] * n[1] * n[2], 3))
    for i in range(n[0]):
        for j in range(n[1]):
            for k in range(n[2]):
                pts[i + j * n[0] + k * n[0] * n[1]] = (o[0] + i * L[0] / n[0], o[1] + j * L[1] / n[1],
                                                       o[2] + k * L[2] / n[2])
    return pts


def test_nearest_structured_clouds():
    src = structured_cloud((2.0, 3.0, 5.0), (7, 11, 13))
    off, idx, _ = cpu.knn(src, src, 1)
    out = src[idx, 0]
    rel_close(out, src[:, 0], 1e-14)


def test_nearest_mixed_clouds():
    Lx, nx = 17.0, 29
    src = structured_cloud((Lx, 19.0, 23.0), (nx, 31, 37))
    tgt = np.random.default_rng(3).random((41, 3)) * [Lx, 19.0, 23.0]
    off, idx, _ = cpu.knn(src, tgt, 1)
    ref = np.round(tgt[:, 0] / Lx * nx) * Lx / nx
    ref[ref == Lx] -= Lx / nx
    rel_close(src[idx, 0], ref, 1e-14)


@pytest.mark.parametrize("k", [1, 4, 10, 20, 32])
def test_knn_grid_index_matches_brute_force(k):
    rng = np.random.default_rng(k)
    src = rng.random((1500, 3))
    src[100:120] = src[0]  # duplicate points (distance ties)
    tgt = np.concatenate([rng.random((300, 3)), src[:20], rng.random((20, 3)) * 3 - 1])
    a = cpu.knn(src, tgt, k)
    b = cpu.knn(src, tgt, k, brute=True)
    assert np.array_equal(a[1], b[1]) and np.array_equal(a[2], b[2])


def test_knn_ties_broken_by_index():
    src = syn.grid_points((40, 40, 1), (0.0, 0.0, 0.0))
    tgt = np.array([[19.5, 19.5, 0.0]])
    off, idx, d2 = cpu.knn(src, tgt, 10)
    # rows ascend in (d2, index)
    keys = list(zip(d2, idx))
    assert keys == sorted(keys)
    assert d2[0] == d2[3] == 0.5  # four equidistant sources come first, by index


def test_radius_search_matches_brute_force():
    rng = np.random.default_rng(4)
    src = syn.gaussian_mixture(4000, 4)
    tgt = rng.random((500, 3))
    r = 0.05
    off, idx, d2 = cpu.radius(src, tgt, r)
    for i in range(len(tgt)):
        d = ((src - tgt[i]) ** 2)
        dd = (d[:, 0] + d[:, 1]) + d[:, 2]
        expect = np.nonzero(np.sqrt(dd) <= r)[0]
        got = idx[off[i]:off[i + 1]]
        assert np.array_equal(np.sort(got), expect)
