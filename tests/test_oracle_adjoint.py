"""The oracle's analytic adjoint (dtk_oracle_coord_grad, apply_transpose)
against central finite differences (h = 1e-6) of an accurate FP64 forward with
the connectivity frozen, on 64 random unit directions d (|FD - <grad, d>| <= 1e-6 ||grad||), for
L = 1/2 ||T f - g||^2 with g = f + 0.05 cos(4 pi z) at the targets."""
import numpy as np
import pytest

from oracle import cpu
from datatransferkit_gb300 import synthetic as syn
from tests.adjoint_reference import fd_coord_directional, forward


@pytest.mark.parametrize("rbf_id,basis_id,k", [(1, 2, 32), (2, 2, 32), (1, 1, 12)])
def test_oracle_adjoint_matches_finite_differences(rbf_id, basis_id, k):
    src = syn.uniform_points(3000, 8)
    tgt = syn.uniform_points(400, 9)
    f = syn.smooth_field(src)
    g = syn.smooth_field(tgt) + 0.05 * np.cos(4 * np.pi * tgt[:, 2])
    off, idx, _ = cpu.knn(src, tgt, k)
    y = forward(src, tgt, idx, k, f, rbf_id, basis_id)
    cot = y - g
    grad = cpu.coord_grad(src, tgt, off, idx, rbf_id, basis_id, f, cot)
    rng = np.random.default_rng(10)
    scale = np.linalg.norm(grad)
    for _ in range(64):
        d = rng.standard_normal(src.shape)
        d /= np.linalg.norm(d)  # unit direction: |<grad, d>| <= ||grad||
        fd = fd_coord_directional(src, tgt, idx, k, f, g, rbf_id, basis_id, d)
        an = float((grad * d).sum())
        assert abs(fd - an) <= 1e-6 * scale, (fd, an, scale)
    # source-value gradient: C^T cot (the loss is linear in the values)
    coeff, _, _, _ = cpu.mls_coefficients(src, tgt, off, idx, rbf_id, basis_id)
    gv = cpu.apply_transpose(off, idx, coeff, cot, len(src))
    d = rng.standard_normal(len(src))
    h = 1e-3
    lp = 0.5 * ((forward(src, tgt, idx, k, f + h * d, rbf_id, basis_id) - g) ** 2).sum()
    lm = 0.5 * ((forward(src, tgt, idx, k, f - h * d, rbf_id, basis_id) - g) ** 2).sum()
    assert abs((lp - lm) / (2 * h) - gv @ d) <= 1e-8 * abs(gv @ d)
