"""NearestNeighborOperator on the GPU (the reference's tstNearestNeighborOperator.cpp
cases on one rank, and the k = 1 search against the oracle), and rank-2
(multi-component) fields for both operators.

Nearest indices are bit-exact against the oracle's k = 1 search (ties to the
smaller source index).  Values: the reference's 1e-14 relative checks.
Rank-2 MLS applies: each component within 1e-14 of sum_j |c_j v_j| of the
rank-1 apply of that column (two summation orders of one row) in the FP64
form; within 2^-40 in the mixed form, whose rank-1 apply sums in double-float
arithmetic on the FP32 pipe (a 2^-48 unit per term, up to 32 terms)."""
import numpy as np
import pytest
import torch

import datatransferkit_gb300 as dtk
from datatransferkit_gb300 import synthetic as syn
from oracle import cpu
from tests.test_oracle_kat import structured_cloud

pytestmark = pytest.mark.gpu


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def test_unique_source_point():
    # tstNearestNeighborOperator.cpp:85-139 on one rank: the source at
    # (comm_size, ...), the target at (comm_rank, ...)
    op = dtk.NearestNeighborOperator(None, dev(np.full((1, 3), 1.0)), dev(np.zeros((1, 3))))
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    op.apply(dev(np.array([255.0])), out)
    assert out.cpu().tolist() == [255.0]


def test_structured_clouds():
    # tstNearestNeighborOperator.cpp:141-204: the target is the source cloud
    src = structured_cloud((2.0, 3.0, 5.0), (7, 11, 13))
    op = dtk.NearestNeighborOperator(None, dev(src), dev(src))
    out = torch.empty(len(src), dtype=torch.float64, device="cuda")
    op.apply(dev(src[:, 0]), out)
    np.testing.assert_allclose(out.cpu().numpy(), src[:, 0], rtol=1e-14)


def test_mixed_clouds():
    # tstNearestNeighborOperator.cpp:206-273: random targets, structured sources
    Lx, nx = 17.0, 29
    src = structured_cloud((Lx, 19.0, 23.0), (nx, 31, 37))
    tgt = np.random.default_rng(3).random((41, 3)) * [Lx, 19.0, 23.0]
    op = dtk.NearestNeighborOperator(None, dev(src), dev(tgt))
    out = torch.empty(len(tgt), dtype=torch.float64, device="cuda")
    op.apply(dev(src[:, 0]), out)
    ref = np.round(tgt[:, 0] / Lx * nx) * Lx / nx
    ref[ref == Lx] -= Lx / nx
    np.testing.assert_allclose(out.cpu().numpy(), ref, rtol=1e-14)


@pytest.mark.parametrize("layout", ["right", "left"])
def test_indices_match_oracle_and_ties(layout):
    src = syn.uniform_points(50000, 21)
    tgt = syn.uniform_points(20000, 22)
    s, t = dev(src), dev(tgt)
    if layout == "left":
        s, t = s.t().contiguous().t(), t.t().contiguous().t()
    op = dtk.NearestNeighborOperator(None, s, t)
    _, idx, _ = cpu.knn(src, tgt, 1)
    assert np.array_equal(op.indices.cpu().numpy(), idx)
    # integer grid with targets on cell centres: 8 equidistant sources, the smallest index wins
    grid = syn.grid_points((6, 6, 6), (0.0, 0.0, 0.0))
    centres = syn.grid_points((5, 5, 5), (0.5, 0.5, 0.5))
    op = dtk.NearestNeighborOperator(None, dev(grid), dev(centres))
    _, idx, _ = cpu.knn(grid, centres, 1, brute=True)
    assert np.array_equal(op.indices.cpu().numpy(), idx)


def test_rank2_fields_nearest():
    src = syn.uniform_points(3000, 23)
    tgt = syn.uniform_points(1000, 24)
    op = dtk.NearestNeighborOperator(None, dev(src), dev(tgt))
    vals = np.random.default_rng(5).standard_normal((len(src), 5))
    idx = op.indices.cpu().numpy()
    for v in (dev(vals), dev(vals.T.copy()).t()):  # LayoutRight, LayoutLeft
        out = torch.empty((len(tgt), 5), dtype=torch.float64, device="cuda")
        op.apply(v, out)
        assert np.array_equal(out.cpu().numpy(), vals[idx])
    out_left = torch.empty((5, len(tgt)), dtype=torch.float64, device="cuda").t()
    op.apply(dev(vals), out_left)
    assert np.array_equal(out_left.cpu().numpy(), vals[idx])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("n_comp", [1, 3, 7])
def test_rank2_fields_mls(precision, n_comp):
    src = syn.uniform_points(20000, 25)
    tgt = syn.uniform_points(4000, 26)
    op = dtk.MovingLeastSquaresOperator(None, dev(src), dev(tgt), dtk.Wendland(2),
                                        dtk.MultivariatePolynomialBasis(dtk.Quadratic, 3), k=32,
                                        precision=precision)
    vals = np.random.default_rng(6).standard_normal((len(src), n_comp))
    off, idx, coeff = (t.cpu().numpy() for t in op.csr())
    mag = np.stack([cpu.apply(off, idx, np.abs(coeff.astype(np.float64)), np.abs(vals[:, c]))
                    for c in range(n_comp)], 1)
    ref = np.empty((len(tgt), n_comp))
    for c in range(n_comp):
        y = torch.empty(len(tgt), dtype=torch.float64, device="cuda")
        op.apply(dev(vals[:, c]), y)
        ref[:, c] = y.cpu().numpy()
    for v in (dev(vals), dev(vals.T.copy()).t()):
        out = torch.empty((len(tgt), n_comp), dtype=torch.float64, device="cuda")
        op.apply(v, out)
        tol = 1e-14 if precision == "fp64" else 2.0 ** -40
        assert np.all(np.abs(out.cpu().numpy() - ref) <= tol * mag + 1e-300)


def test_preconditions():
    src = dev(syn.uniform_points(100, 27))
    tgt = dev(syn.uniform_points(10, 28))
    with pytest.raises(dtk.InvalidArgument):
        dtk.NearestNeighborOperator(None, src[:0], tgt)  # DTK_CHECK( !search_tree.empty() )
    with pytest.raises(dtk.Unsupported):
        dtk.NearestNeighborOperator(2, src, tgt)  # more than one rank
    op = dtk.NearestNeighborOperator(None, src, tgt)
    with pytest.raises(dtk.InvalidArgument):
        op.apply(torch.zeros(99, dtype=torch.float64, device="cuda"),
                 torch.zeros(10, dtype=torch.float64, device="cuda"))
    with pytest.raises(dtk.InvalidArgument):
        op.apply(torch.zeros(100, dtype=torch.float64, device="cuda"),
                 torch.zeros(11, dtype=torch.float64, device="cuda"))
    with pytest.raises(dtk.InvalidArgument):  # component counts differ
        op.apply(torch.zeros((100, 2), dtype=torch.float64, device="cuda"),
                 torch.zeros((10, 3), dtype=torch.float64, device="cuda"))
    empty = dtk.NearestNeighborOperator(None, src, tgt[:0])
    empty.apply(torch.zeros(100, dtype=torch.float64, device="cuda"),
                torch.zeros(0, dtype=torch.float64, device="cuda"))
