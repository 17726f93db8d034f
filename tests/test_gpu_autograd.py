"""torch.autograd binding of the adjoint: gradients equal the C-ABI adjoint's,
torch.autograd.gradcheck passes on the source values (the transfer is linear
in them), and the coordinate gradient of L = 1/2 ||T f - g||^2 matches
central finite differences (h = 1e-6) of an accurate FP64 forward with frozen
connectivity on 16 random unit directions: |FD - <grad, d>| <= 1e-6 ||grad||.
"""
import numpy as np
import pytest
import torch

import datatransferkit_gb300 as dtk
from datatransferkit_gb300 import synthetic as syn
from datatransferkit_gb300.autograd import mls_transfer
from oracle import cpu
from tests.adjoint_reference import fd_coord_directional

pytestmark = pytest.mark.gpu
QUAD = dtk.MultivariatePolynomialBasis(dtk.Quadratic, 3)


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def test_backward_matches_adjoint_and_finite_differences():
    src = syn.uniform_points(2000, 41)
    tgt = syn.uniform_points(300, 42)
    f = syn.smooth_field(src)
    g = syn.smooth_field(tgt) + 0.05 * np.cos(4 * np.pi * tgt[:, 2])
    fv = dev(f).requires_grad_(True)
    sp = dev(src).requires_grad_(True)
    y = mls_transfer(fv, sp, dev(tgt), dtk.Wendland(2), QUAD, k=32)
    loss = 0.5 * ((y - dev(g)) ** 2).sum()
    loss.backward()
    op = dtk.MovingLeastSquaresOperator(None, dev(src), dev(tgt), dtk.Wendland(2), QUAD, k=32,
                                        keep_points=True)
    gv, gc = op.apply_adjoint((y - dev(g)).detach(), dev(f), coords=True)
    assert torch.equal(fv.grad, gv) and torch.equal(sp.grad, gc)
    _, idx, _ = cpu.knn(src, tgt, 32)
    gcn = sp.grad.cpu().numpy()
    scale = np.linalg.norm(gcn)
    rng = np.random.default_rng(43)
    for _ in range(16):
        d = rng.standard_normal(src.shape)
        d /= np.linalg.norm(d)
        fd = fd_coord_directional(src, tgt, idx, 32, f, g, 1, 2, d)
        assert abs(fd - float((gcn * d).sum())) <= 1e-6 * scale


def test_gradcheck_source_values():
    src = dev(syn.uniform_points(120, 44))
    tgt = dev(syn.uniform_points(40, 45))
    fv = dev(syn.smooth_field(src.cpu().numpy())).requires_grad_(True)
    assert torch.autograd.gradcheck(
        lambda v: mls_transfer(v, src, tgt, dtk.Wendland(4), QUAD, k=20), (fv,), eps=1e-6, atol=1e-9)


def test_target_points_gradient_is_refused():
    src = dev(syn.uniform_points(100, 46))
    tgt = dev(syn.uniform_points(20, 47)).requires_grad_(True)
    fv = dev(syn.smooth_field(src.cpu().numpy()))
    y = mls_transfer(fv, src, tgt, k=8)
    with pytest.raises(NotImplementedError):
        y.sum().backward()
