"""GPU adjoint (dtk_mls_apply_adjoint) against the FP64 CPU oracle's adjoint and
against central finite differences (h = 1e-6) of an accurate FP64 forward with
frozen connectivity, on 64 random unit directions, for
L = 1/2 ||T f - g||^2, g = f + 0.05 cos(4 pi z) at the targets.

Tolerances: source-value gradients <= 1e-12 relative (FP64 form; the same
coefficients transposed); coordinate gradients <= 1e-8 relative to the oracle
(the oracle's pseudo-inverse is the reference's Jacobi, the GPU's an accurate
eigen-solve; they differ by the reference's ~1e-10 deviation) and
|FD - <grad, d>| <= 1e-6 ||grad|| against finite differences."""
import numpy as np
import pytest
import torch

import datatransferkit_gb300 as dtk
from datatransferkit_gb300 import synthetic as syn
from oracle import cpu
from tests.adjoint_reference import fd_coord_directional, forward

pytestmark = pytest.mark.gpu
RBF = {1: dtk.Wendland(2), 2: dtk.Wendland(4)}
BASIS = {1: dtk.MultivariatePolynomialBasis(dtk.Linear, 3),
         2: dtk.MultivariatePolynomialBasis(dtk.Quadratic, 3)}


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def setup_case(n_src, n_tgt, seed=8):
    src = syn.uniform_points(n_src, seed)
    tgt = syn.uniform_points(n_tgt, seed + 1)
    f = syn.smooth_field(src)
    g = syn.smooth_field(tgt) + 0.05 * np.cos(4 * np.pi * tgt[:, 2])
    return src, tgt, f, g


@pytest.mark.parametrize("rbf_id,basis_id,k", [(1, 2, 32), (2, 2, 32), (1, 1, 12)])
def test_adjoint_against_oracle_and_finite_differences(rbf_id, basis_id, k):
    src, tgt, f, g = setup_case(3000, 400)
    op = dtk.MovingLeastSquaresOperator(None, dev(src), dev(tgt), RBF[rbf_id], BASIS[basis_id],
                                        k=k, keep_points=True)
    off, idx, _ = cpu.knn(src, tgt, k)
    y = forward(src, tgt, idx, k, f, rbf_id, basis_id)
    cot = y - g
    gv, gc = op.apply_adjoint(dev(cot), dev(f), coords=True)
    gv, gc = gv.cpu().numpy(), gc.cpu().numpy()
    coeff, _, _, _ = cpu.mls_coefficients(src, tgt, off, idx, rbf_id, basis_id)
    gv_ref = cpu.apply_transpose(off, idx, coeff, cot, len(src))
    assert np.abs(gv - gv_ref).max() <= 1e-12 * np.abs(gv_ref).max()
    gc_ref = cpu.coord_grad(src, tgt, off, idx, rbf_id, basis_id, f, cot)
    assert np.abs(gc - gc_ref).max() <= 1e-8 * np.abs(gc_ref).max()
    rng = np.random.default_rng(10)
    scale = np.linalg.norm(gc)
    for _ in range(64):
        d = rng.standard_normal(src.shape)
        d /= np.linalg.norm(d)
        fd = fd_coord_directional(src, tgt, idx, k, f, g, rbf_id, basis_id, d)
        assert abs(fd - float((gc * d).sum())) <= 1e-6 * scale


def test_adjoint_is_deterministic_and_mixed_form_values():
    src, tgt, f, g = setup_case(20000, 5000, seed=20)
    cot = dev(np.random.default_rng(3).standard_normal(len(tgt)))
    for prec in ("fp64", "mixed"):
        op = dtk.MovingLeastSquaresOperator(None, dev(src), dev(tgt), RBF[2], BASIS[2], k=32,
                                            precision=prec, keep_points=True)
        a = op.apply_adjoint(cot, dev(f), coords=True)
        b = op.apply_adjoint(cot, dev(f), coords=True)
        assert torch.equal(a[0], b[0]) and torch.equal(a[1], b[1])  # bit-reproducible
        off, idx, coeff = op.csr()
        ref = cpu.apply_transpose(off.cpu().numpy(), idx.cpu().numpy(),
                                  coeff.double().cpu().numpy(), cot.cpu().numpy(), len(src))
        assert np.abs(a[0].cpu().numpy() - ref).max() <= 1e-12 * np.abs(ref).max()


def test_adjoint_radius_mode():
    src = syn.gaussian_mixture(8000, 30)
    tgt = syn.uniform_points(1500, 31)
    f = syn.smooth_field(src)
    cot = np.random.default_rng(4).standard_normal(len(tgt))
    op = dtk.MovingLeastSquaresOperator(None, dev(src), dev(tgt), RBF[1], BASIS[1], radius=0.05,
                                        keep_points=True)
    gv, gc = op.apply_adjoint(dev(cot), dev(f), coords=True)
    off, idx, _ = cpu.radius(src, tgt, 0.05)
    coeff, _, _, _ = cpu.mls_coefficients(src, tgt, off, idx, 1, 1)
    gv_ref = cpu.apply_transpose(off, idx, coeff, cot, len(src))
    gc_ref = cpu.coord_grad(src, tgt, off, idx, 1, 1, f, cot)
    rows = np.diff(off)
    # rows with fewer than 4 neighbours are rank-deficient for the linear basis;
    # compare the sources that only such rows do not touch
    bad = np.zeros(len(src), bool)
    for i in np.nonzero(rows < 8)[0]:
        bad[idx[off[i]:off[i + 1]]] = True
    ok = ~bad
    assert np.abs(gv.cpu().numpy()[ok] - gv_ref[ok]).max() <= 1e-10 * np.abs(gv_ref).max()
    assert np.abs(gc.cpu().numpy()[ok] - gc_ref[ok]).max() <= 1e-6 * np.abs(gc_ref).max()


def test_adjoint_preconditions():
    src, tgt, f, _ = setup_case(500, 50)
    op = dtk.MovingLeastSquaresOperator(None, dev(src), dev(tgt), RBF[1], BASIS[2], k=20)
    cot = dev(np.ones(len(tgt)))
    gv, _ = op.apply_adjoint(cot)  # values only: fine without kept points
    assert gv.shape == (len(src),)
    with pytest.raises(dtk.InvalidArgument):
        op.apply_adjoint(cot, dev(f), coords=True)  # needs keep_points
    with pytest.raises(dtk.InvalidArgument):
        op.apply_adjoint(dev(np.ones(len(tgt) + 1)))
