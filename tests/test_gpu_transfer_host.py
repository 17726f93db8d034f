"""Setup and apply from host buffers (dtk_mls_transfer_host): the copies
overlap the work and the apply runs in row slices, so the results must equal
the device operator's bit for bit; kNN (uniform rows) and radius rows
(offset-addressed slices), both forms, pinned and pageable buffers."""
import pytest
import torch

import datatransferkit_gb300 as dtk
from datatransferkit_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu
QUAD = dtk.MultivariatePolynomialBasis(dtk.Quadratic, 3)


@pytest.mark.parametrize("mode", ["knn", "radius"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_host_transfer_matches_device_operator(mode, precision):
    src = syn.uniform_points(1_100_000, 71)
    tgt = syn.uniform_points(1_050_000, 72)  # over 1M targets: the apply runs in 8 slices
    vals = syn.smooth_field(src)
    opts = dict(k=32) if mode == "knn" else dict(radius=0.02)
    src_h, tgt_h, vals_h = (torch.from_numpy(a).pin_memory() for a in (src, tgt, vals))
    out_h = torch.empty(len(tgt), dtype=torch.float64).pin_memory()
    kept = dtk.MovingLeastSquaresOperator.transfer_host(None, src_h, tgt_h, vals_h, out_h, dtk.Wendland(2),
                                                        QUAD, precision=precision, keep=True, **opts)
    ref = dtk.MovingLeastSquaresOperator(None, src_h.cuda(), tgt_h.cuda(), dtk.Wendland(2), QUAD,
                                         precision=precision, **opts)
    y = torch.empty(len(tgt), dtype=torch.float64, device="cuda")
    ref.apply(vals_h.cuda(), y)
    assert torch.equal(out_h, y.cpu())
    for a, b in zip(kept.csr(), ref.csr()):
        assert torch.equal(a, b)
    out_p = torch.empty(len(tgt), dtype=torch.float64)  # pageable
    assert dtk.MovingLeastSquaresOperator.transfer_host(None, torch.from_numpy(src), torch.from_numpy(tgt),
                                                        torch.from_numpy(vals), out_p, dtk.Wendland(2), QUAD,
                                                        precision=precision, **opts) is None
    assert torch.equal(out_p, out_h)


def test_host_transfer_preconditions():
    src = torch.from_numpy(syn.uniform_points(100, 73))
    tgt = torch.from_numpy(syn.uniform_points(10, 74))
    with pytest.raises(dtk.InvalidArgument):  # device tensors are not host buffers
        dtk.MovingLeastSquaresOperator.transfer_host(None, src.cuda(), tgt, torch.zeros(100, dtype=torch.float64),
                                                     torch.zeros(10, dtype=torch.float64), k=8)
    with pytest.raises(dtk.InvalidArgument):
        dtk.MovingLeastSquaresOperator.transfer_host(None, src, tgt, torch.zeros(99, dtype=torch.float64),
                                                     torch.zeros(10, dtype=torch.float64), k=8)
    with pytest.raises(dtk.InvalidArgument):  # the empty source cloud
        dtk.MovingLeastSquaresOperator.transfer_host(None, src[:0], tgt, torch.zeros(0, dtype=torch.float64),
                                                     torch.zeros(10, dtype=torch.float64), k=8)
    out = torch.zeros(0, dtype=torch.float64)  # no targets
    dtk.MovingLeastSquaresOperator.transfer_host(None, src, tgt[:0], torch.zeros(100, dtype=torch.float64),
                                                 out, k=8)
