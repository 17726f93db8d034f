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
