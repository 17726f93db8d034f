"""The operator product on disk and on the wire: an operator rebuilt from its
exported bytes applies bitwise like the original (FP64 and mixed forms, kNN and
radius rows), its values adjoint matches, and damaged or foreign byte strings are
rejected with InvalidArgument."""
import numpy as np
import pytest
import torch

import datatransferkit_gb300 as dtk
from datatransferkit_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu
Q = dtk.MultivariatePolynomialBasis(dtk.Quadratic, 3)


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("precision,k,radius", [("fp64", 32, None), ("mixed", 32, None),
                                                ("fp64", None, 0.05)])
def test_roundtrip_is_bitwise(precision, k, radius, tmp_path):
    src = syn.gaussian_mixture(20000, 41) if radius else syn.uniform_points(20000, 41)
    tgt = syn.uniform_points(5000, 42)
    op = dtk.MovingLeastSquaresOperator(None, dev(src), dev(tgt), dtk.Wendland(2), Q, k=k,
                                        radius=radius, precision=precision)
    vals = dev(syn.smooth_field(src))
    y0 = torch.empty(len(tgt), dtype=torch.float64, device="cuda")
    op.apply(vals, y0)
    op.save(tmp_path / "op.dtk")
    for op2 in (dtk.MovingLeastSquaresOperator.from_bytes(op.to_bytes()),
                dtk.MovingLeastSquaresOperator.load(tmp_path / "op.dtk")):
        y1 = torch.empty_like(y0)
        op2.apply(vals, y1)
        assert torch.equal(y0, y1)
        for a, b in zip(op.csr(), op2.csr()):
            assert torch.equal(a, b)
        cot = dev(np.random.default_rng(1).standard_normal(len(tgt)))
        assert torch.equal(op.apply_adjoint(cot)[0], op2.apply_adjoint(cot)[0])
        with pytest.raises(dtk.InvalidArgument):  # the points are not part of the product
            op2.apply_adjoint(cot, vals, coords=True)


def test_damaged_products_are_rejected():
    src = syn.uniform_points(2000, 43)
    tgt = syn.uniform_points(300, 44)
    data = dtk.MovingLeastSquaresOperator(None, dev(src), dev(tgt), k=8).to_bytes()
    flipped = bytearray(data)
    flipped[len(data) // 2] ^= 0x10
    for bad in (bytes(flipped), data[:-1], data + b"\0", b"XTKMLS01" + data[8:], data[:40]):
        with pytest.raises(dtk.InvalidArgument):
            dtk.MovingLeastSquaresOperator.from_bytes(bad)
