"""FP64 form of the GPU MLS operator against the oracle and the golden fixtures.

The FP64 form runs the reference algorithm (same Jacobi pivots, rotations and
absolute DBL_EPSILON stop and truncation).  Neighbour indices are bit-exact.
Tolerance on values: relative L2 of target values, and per row
max|c - c_ref| / max|c_ref| on coefficients, each <= max(1e-12, 100 * spread),
where spread is the distance between the oracle and its own
multiply-add-contracted build on the same inputs: how far the reference code
itself moves between two valid compilations.  On the benchmark clouds
(k = 20/32, quadratic) the spread is ~1e-14 and the bound is 1e-12; on the
reference's deliberately degenerate known-answer layouts (k = basis size,
rank-one moments) the reference is itself only reproducible to its spread.
"""
from pathlib import Path

import numpy as np
import pytest
import torch

import datatransferkit_gb300 as dtk
from datatransferkit_gb300 import _capi
from datatransferkit_gb300 import synthetic as syn
from oracle import cpu

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"
BASIS = {0: dtk.MultivariatePolynomialBasis(dtk.Constant, 3),
         1: dtk.MultivariatePolynomialBasis(dtk.Linear, 3),
         2: dtk.MultivariatePolynomialBasis(dtk.Quadratic, 3)}
RBF = [dtk.Wendland(0), dtk.Wendland(2), dtk.Wendland(4), dtk.Wendland(6), dtk.Wu(2), dtk.Wu(4),
       dtk.Buhmann(2), dtk.Buhmann(3), dtk.Buhmann(4)]
TOL = 1e-12
SPREAD_FACTOR = 100.0


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def run_gpu(src, tgt, values, rbf, basis, k=None, radius=None, precision="fp64"):
    op = dtk.MovingLeastSquaresOperator(None, dev(src), dev(tgt), RBF[rbf], BASIS[basis], k=k,
                                        radius=radius, precision=precision)
    out = torch.full((len(tgt),), np.nan, dtype=torch.float64, device="cuda")
    op.apply(dev(values), out)
    off, idx, coeff = op.csr()
    return dict(target=out.cpu().numpy(), offset=off.cpu().numpy(), idx=idx.cpu().numpy(),
                coeff=coeff.double().cpu().numpy(), under=op.underdetermined, op=op)


def rel_l2(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def tolerances(src, tgt, offset, idx, rbf, basis, values, coeff_ref):
    sc, st = cpu.rounding_spread(src, tgt, offset, idx, rbf, basis, values, coeff_ref)
    return max(TOL, SPREAD_FACTOR * sc), max(TOL, SPREAD_FACTOR * st)


def assert_coeff_close(c, c_ref, offset, tol):
    for i in range(len(offset) - 1):
        a, b = c[offset[i]:offset[i + 1]], c_ref[offset[i]:offset[i + 1]]
        if len(b):
            assert np.abs(a - b).max() <= tol * max(np.abs(b).max(), 1e-300), i


@pytest.mark.parametrize("name", sorted(p.stem for p in GOLDEN.glob("*.npz")
                                        if p.stem not in ("svd", "rbf_basis")))
def test_golden_fixture(name):
    g = dict(np.load(GOLDEN / f"{name}.npz"))
    r = run_gpu(g["src"], g["tgt"], g["values"], int(g["rbf"]), int(g["basis"]), k=int(g["k"]))
    assert np.array_equal(r["idx"], g["idx"])
    tc, tt = tolerances(g["src"], g["tgt"], g["offset"], g["idx"], int(g["rbf"]), int(g["basis"]),
                        g["values"], g["coeff"])
    if tc <= TOL:  # rank decisions are only reproducible where the values are
        assert r["under"] == int(g["underdetermined"])
    assert_coeff_close(r["coeff"], g["coeff"], g["offset"], tc)
    assert rel_l2(r["target"], g["target"]) <= tt


@pytest.mark.parametrize("basis", [0, 1, 2])
def test_reference_known_answers(basis):
    m = BASIS[basis].size
    f = syn.polynomial_of_basis(m)
    src, tgt = syn.cluster_problem(10, m, 0.5, seed=201)
    r = run_gpu(src, tgt, f(src), 0, basis)
    np.testing.assert_allclose(r["target"], f(tgt), rtol=1e-7)  # same_npoints_and_basis
    src = syn.grid_points((40, 40, 1), (0.0, 0.0, 0.0))
    tgt = syn.grid_points((1, 1, 1), (19.0, 19.0, 0.0))
    r = run_gpu(src, tgt, f(src), 0, basis)
    np.testing.assert_allclose(r["target"], f(tgt), rtol=1e-14)  # grid
    src = syn.grid_points((40, 1, 1), (0.0, 0.0, 0.0))
    tgt = syn.grid_points((39, 1, 1), (0.5, 0.0, 0.0))
    r = run_gpu(src, tgt, f(src), 0, basis)
    np.testing.assert_allclose(r["target"], f(tgt), rtol=1e-14)  # line
    src, tgt = syn.cluster_problem(10, 1, 0.5, seed=202)
    r = run_gpu(src, tgt, f(src), 0, basis)
    assert np.all(np.isfinite(r["target"]))  # single_point_in_radius


def test_corner_cases():
    r = run_gpu(np.array([[1.0, 1, 1], [2.0, 2, 2]]), np.array([[1.5, 1.5, 1.5]]),
                np.array([255.0, 255.0]), 0, 1)
    np.testing.assert_allclose(r["target"], [255.0], rtol=1e-12)
    op = dtk.MovingLeastSquaresOperator(None, dev(np.array([[1.0, 1, 1]])), dev(np.zeros((0, 3))))
    out = torch.empty(0, dtype=torch.float64, device="cuda")
    op.apply(dev(np.array([255.0])), out)
    assert op.nnz == 0


@pytest.mark.parametrize("rbf", range(9))
@pytest.mark.parametrize("basis", [0, 1, 2])
def test_all_rbfs_and_bases_against_oracle(rbf, basis):
    src = syn.uniform_points(6000, 40 + rbf)
    tgt = syn.uniform_points(1500, 60 + basis)
    vals = syn.smooth_field(src)
    r = run_gpu(src, tgt, vals, rbf, basis, k=16)
    ref = cpu.mls_transfer(src, tgt, vals, rbf, basis, k=16)
    assert np.array_equal(r["idx"], ref["idx"])
    tc, tt = tolerances(src, tgt, ref["offset"], ref["idx"], rbf, basis, vals, ref["coeff"])
    if tc <= TOL:
        assert r["under"] == ref["underdetermined"]
    assert_coeff_close(r["coeff"], ref["coeff"], ref["offset"], tc)
    assert rel_l2(r["target"], ref["target"]) <= tt


@pytest.mark.parametrize("k", [10, 20, 32])
def test_benchmark_density_against_oracle(k):
    # a 0.1^3 window of the 2M-point density of the FP64-at-scale workload
    src = syn.uniform_points(2000, 70) * 0.1
    tgt = 0.02 + syn.uniform_points(800, 71) * 0.06
    vals = syn.smooth_field(src)
    r = run_gpu(src, tgt, vals, 1, 2, k=k)
    ref = cpu.mls_transfer(src, tgt, vals, 1, 2, k=k)
    assert np.array_equal(r["idx"], ref["idx"])
    tc, tt = tolerances(src, tgt, ref["offset"], ref["idx"], 1, 2, vals, ref["coeff"])
    assert_coeff_close(r["coeff"], ref["coeff"], ref["offset"], tc)
    assert rel_l2(r["target"], ref["target"]) <= tt
    if k >= 20:  # the benchmark neighbourhoods: the plain 1e-12 bound holds
        assert rel_l2(r["target"], ref["target"]) <= TOL


@pytest.mark.parametrize("log", [0, 40])
def test_rotation_log_and_formed_u_agree(log):
    """Row 0 of the pseudo-inverse from the rotation log (the default) against
    U formed for every matrix (log 0: the reference's product order) and U
    formed after 40 logged rotations (every quadratic matrix here outruns
    that): each within the FP64 bound of the oracle, and of one another at
    rounding level."""
    src = syn.uniform_points(6000, 90)
    tgt = syn.uniform_points(1500, 91)
    vals = syn.smooth_field(src)
    ref = cpu.mls_transfer(src, tgt, vals, 2, 2, k=32)
    base = run_gpu(src, tgt, vals, 2, 2, k=32)
    L = _capi.lib()
    assert L.dtk_set_rotation_log(log) == 0
    try:
        r = run_gpu(src, tgt, vals, 2, 2, k=32)
    finally:
        assert L.dtk_set_rotation_log(160) == 0
    for x in (base, r):
        assert np.array_equal(x["idx"], ref["idx"])
        assert_coeff_close(x["coeff"], ref["coeff"], ref["offset"], TOL)
        assert rel_l2(x["target"], ref["target"]) <= TOL
    assert_coeff_close(r["coeff"], base["coeff"], ref["offset"], 1e-13)
    assert not np.array_equal(r["coeff"], base["coeff"])  # the other product order ran


def test_radius_mode_against_oracle():
    src = syn.gaussian_mixture(8000, 80)
    tgt = syn.uniform_points(2000, 81)
    vals = syn.smooth_field(src)
    r = run_gpu(src, tgt, vals, 1, 2, radius=0.05)
    ref = cpu.mls_transfer(src, tgt, vals, 1, 2, r=0.05)
    assert np.array_equal(r["offset"], ref["offset"])
    tc, tt = tolerances(src, tgt, ref["offset"], ref["idx"], 1, 2, vals, ref["coeff"])
    # radius rows are sets; GPU order is the tree's traversal order
    for i in range(len(tgt)):
        a = slice(r["offset"][i], r["offset"][i + 1])
        oa, ob = np.argsort(r["idx"][a]), np.argsort(ref["idx"][a])
        assert np.array_equal(r["idx"][a][oa], ref["idx"][a][ob])
        if r["offset"][i + 1] > r["offset"][i]:
            ca, cb = r["coeff"][a][oa], ref["coeff"][a][ob]
            assert np.abs(ca - cb).max() <= tc * max(np.abs(cb).max(), 1e-300)
    assert rel_l2(r["target"], ref["target"]) <= tt


def test_layout_left_inputs():
    src = syn.uniform_points(3000, 90)
    tgt = syn.uniform_points(600, 91)
    vals = syn.smooth_field(src)
    s, t = dev(src).t().contiguous().t(), dev(tgt).t().contiguous().t()
    assert s.stride() == (1, len(src))
    op = dtk.MovingLeastSquaresOperator(None, s, t, dtk.Wendland(2), BASIS[2], k=20)
    out = torch.empty(len(tgt), dtype=torch.float64, device="cuda")
    op.apply(dev(vals), out)
    ref = cpu.mls_transfer(src, tgt, vals, 1, 2, k=20)
    assert rel_l2(out.cpu().numpy(), ref["target"]) <= TOL


def test_apply_preconditions():
    src = syn.uniform_points(100, 1)
    tgt = syn.uniform_points(10, 2)
    op = dtk.MovingLeastSquaresOperator(None, dev(src), dev(tgt))
    with pytest.raises(dtk.InvalidArgument):
        op.apply(torch.zeros(99, dtype=torch.float64, device="cuda"),
                 torch.zeros(10, dtype=torch.float64, device="cuda"))
    with pytest.raises(dtk.InvalidArgument):
        op.apply(torch.zeros(100, dtype=torch.float64, device="cuda"),
                 torch.zeros(11, dtype=torch.float64, device="cuda"))


def test_apply_is_repeatable_and_linear():
    src = syn.uniform_points(5000, 3)
    tgt = syn.uniform_points(2000, 4)
    op = dtk.MovingLeastSquaresOperator(None, dev(src), dev(tgt), dtk.Wendland(2), BASIS[2], k=32)
    a, b = dev(syn.smooth_field(src)), dev(src[:, 0] ** 3)
    ya, yb, yab = (torch.empty(len(tgt), dtype=torch.float64, device="cuda") for _ in range(3))
    op.apply(a, ya)
    op.apply(b, yb)
    op.apply(2.0 * a - 3.0 * b, yab)
    y2 = torch.empty_like(ya)
    op.apply(a, y2)
    assert torch.equal(ya, y2)
    assert torch.allclose(yab, 2.0 * ya - 3.0 * yb, rtol=0, atol=1e-12)
