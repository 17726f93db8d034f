"""The C ABI's device-memory boundary: pointers the kernels dereference are
checked, and pageable host memory is refused with DTK_ERR_INVALID_ARG and a
message naming it (on a machine where the GPU cannot read pageable memory a
kernel would fault instead); pinned host memory, which CUDA maps, is used."""
import ctypes as C

import numpy as np
import pytest
import torch

import datatransferkit_gb300 as dtk
from datatransferkit_gb300 import _capi
from datatransferkit_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu
INVALID_ARG = 1


def test_pageable_host_pointers_are_refused():
    L = _capi.lib()
    src = np.ascontiguousarray(syn.uniform_points(100, 81))
    tgt = np.ascontiguousarray(syn.uniform_points(10, 82))
    o = _capi.Options()
    L.dtk_mls_default_options(C.byref(o))
    o.k = 8
    h = C.c_void_p()
    st = L.dtk_mls_create(C.byref(o), src.ctypes.data, 100, 3, 1, tgt.ctypes.data, 10, 3, 1, None, C.byref(h))
    assert st == INVALID_ARG and b"host memory" in L.dtk_last_error()
    assert not h.value
    op = dtk.MovingLeastSquaresOperator(None, torch.from_numpy(src).cuda(), torch.from_numpy(tgt).cuda(), k=8)
    vals, out = np.ones(100), np.zeros(10)
    assert L.dtk_mls_apply(op._h, vals.ctypes.data, 100, out.ctypes.data, 10, None) == INVALID_ARG
    assert b"source_values" in L.dtk_last_error()
    nn = dtk.NearestNeighborOperator(None, torch.from_numpy(src).cuda(), torch.from_numpy(tgt).cuda())
    assert L.dtk_nn_apply(nn._h, vals.ctypes.data, 100, out.ctypes.data, 10, None) == INVALID_ARG
    # pinned host memory is mapped for the device: accepted, and the result lands in it
    pin_v = torch.ones(100, dtype=torch.float64).pin_memory()
    pin_o = torch.zeros(10, dtype=torch.float64).pin_memory()
    assert L.dtk_mls_apply(op._h, pin_v.data_ptr(), 100, pin_o.data_ptr(), 10, None) == 0
    torch.cuda.synchronize()
    y = torch.empty(10, dtype=torch.float64, device="cuda")
    op.apply(torch.ones(100, dtype=torch.float64, device="cuda"), y)
    assert torch.equal(pin_o, y.cpu())


def test_svd_entry_points_refuse_pageable_host_matrices():
    L = _capi.lib()
    host = np.eye(4).reshape(1, 4, 4).copy()
    out = np.zeros_like(host)
    dev = torch.from_numpy(host).cuda()
    dev_out = torch.empty_like(dev)
    for fn in ("dtk_svd_pinv", "dtk_svd_pinv_noalloc"):
        f = getattr(L, fn)
        assert f(4, 1, host.ctypes.data, dev_out.data_ptr(), None, None) == INVALID_ARG, fn
        assert b"a is host memory" in L.dtk_last_error(), fn
        assert f(4, 1, dev.data_ptr(), out.ctypes.data, None, None) == INVALID_ARG, fn
        assert b"pinv is host memory" in L.dtk_last_error(), fn


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_create_from_neighbors_reproduces_create(precision):
    # the rows of a one-rank operator handed back to dtk_mls_create_from_neighbors:
    # in their order the coefficients are the create's bit for bit; with every
    # row reversed, the same coefficients up to the order of the moment sums
    from oracle import cpu
    src, tgt = syn.uniform_points(20_000, 83), syn.uniform_points(3_000, 84)
    s, t = torch.from_numpy(src).cuda(), torch.from_numpy(tgt).cuda()
    Q = dtk.MultivariatePolynomialBasis(dtk.Quadratic, 3)
    op = dtk.MovingLeastSquaresOperator(None, s, t, dtk.Wendland(4), Q, k=32, precision=precision)
    _, idx, coeff = op.csr()
    idx = idx.long()
    nb = s[idx].contiguous()
    local = torch.arange(idx.numel(), dtype=torch.int32, device="cuda")
    again = dtk.MovingLeastSquaresOperator.from_neighbors(t, 32, nb, local, idx.numel(), dtk.Wendland(4), Q,
                                                          precision=precision)
    assert torch.equal(again.csr()[2], coeff)
    rev = idx.view(-1, 32).flip(1).reshape(-1)
    other = dtk.MovingLeastSquaresOperator.from_neighbors(t, 32, s[rev].contiguous(), local, idx.numel(),
                                                          dtk.Wendland(4), Q, precision=precision)
    c2 = other.csr()[2].view(-1, 32).flip(1).reshape(-1)
    scale = coeff.abs().view(-1, 32).amax(1, keepdim=True)
    tol = 1e-12 if precision == "fp64" else 1e-6
    assert ((c2 - coeff).abs().view(-1, 32) <= tol * scale).all()
    # values through the fetched layout: this rank's values in entry order
    vals = syn.smooth_field(src)
    y = torch.empty(len(tgt), dtype=torch.float64, device="cuda")
    again.apply(torch.from_numpy(vals).cuda()[idx].contiguous(), y)
    ref = cpu.mls_transfer(src, tgt, vals, 2, 2, k=32)["target"]
    err = np.linalg.norm(y.cpu().numpy() - ref) / np.linalg.norm(ref)
    assert err <= (1e-13 if precision == "fp64" else 1e-6), err
    # rows must hold 1..32 entries; indices in range
    with pytest.raises(dtk.InvalidArgument):
        dtk.MovingLeastSquaresOperator.from_neighbors(t, 32, nb, local, idx.numel() - 1, dtk.Wendland(4), Q)
