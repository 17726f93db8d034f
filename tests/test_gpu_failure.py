"""Failure detection without a GPU fault.

* The bounded device loops (the Jacobi rotations of the FP64 setup and of the
  batched pseudo-inverse, the tree traversal of the kNN and radius searches)
  stop at a cap and the call returns DTK_ERR_TIMEOUT with the context intact:
  dtk_set_loop_caps lowers the caps so that ordinary inputs exhaust them, and
  the next call with the built-in caps succeeds on the same device.
* A NaN or infinite coordinate in either cloud is DTK_ERR_INVALID_ARG before
  any search runs (the reference's operator would hand it to ArborX).
"""
import ctypes as C

import numpy as np
import pytest
import torch

import datatransferkit_gb300 as dtk
from datatransferkit_gb300 import _capi
from datatransferkit_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu
INVALID_ARG, TIMEOUT = 1, 5


def _create(src, tgt, k=20, precision=0, radius=0.0):
    L = _capi.lib()
    o = _capi.Options()
    L.dtk_mls_default_options(C.byref(o))
    o.k, o.basis, o.rbf, o.precision, o.radius = k, 2, 1, precision, radius
    h = C.c_void_p()
    st = L.dtk_mls_create(C.byref(o), src.data_ptr(), src.shape[0], 3, 1, tgt.data_ptr(), tgt.shape[0],
                          3, 1, None, C.byref(h))
    if h.value:
        L.dtk_mls_destroy(h)
    return st


@pytest.fixture
def clouds():
    src = torch.from_numpy(syn.uniform_points(3000, 91)).cuda()
    tgt = torch.from_numpy(syn.uniform_points(500, 92)).cuda()
    return src, tgt


@pytest.fixture
def restore_caps():
    yield
    assert _capi.lib().dtk_set_loop_caps(0, 0) == 0


def test_jacobi_cap_exhaustion_returns_timeout(clouds, restore_caps):
    L = _capi.lib()
    src, tgt = clouds
    assert L.dtk_set_loop_caps(3, 0) == 0  # 3 rotations: far below the ~110 a quadratic moment matrix takes
    assert _create(src, tgt) == TIMEOUT
    assert b"hit its cap" in L.dtk_last_error()
    mats = torch.from_numpy(np.stack([np.eye(8) + 0.1 * np.ones((8, 8))] * 4)).cuda()
    out = torch.empty_like(mats)
    for fn in ("dtk_svd_pinv", "dtk_svd_pinv_noalloc"):
        assert getattr(L, fn)(8, 4, mats.data_ptr(), out.data_ptr(), None, None) == TIMEOUT, fn
    # the same device and inputs work again with the built-in caps
    assert L.dtk_set_loop_caps(0, 0) == 0
    assert _create(src, tgt) == 0
    assert L.dtk_svd_pinv(8, 4, mats.data_ptr(), out.data_ptr(), None, None) == 0


def test_traversal_cap_exhaustion_returns_timeout(clouds, restore_caps):
    L = _capi.lib()
    src, tgt = clouds
    assert L.dtk_set_loop_caps(0, 1) == 0  # one traversal step: the root only
    assert _create(src, tgt, precision=1) == TIMEOUT
    assert _create(src, tgt, radius=0.1) == TIMEOUT
    offset = torch.empty(tgt.shape[0] + 1, dtype=torch.int32, device="cuda")
    idx = torch.empty(tgt.shape[0] * 8, dtype=torch.int32, device="cuda")
    assert L.dtk_knn_search(src.data_ptr(), src.shape[0], 3, 1, tgt.data_ptr(), tgt.shape[0], 3, 1, 8,
                            offset.data_ptr(), idx.data_ptr(), None) == TIMEOUT
    assert L.dtk_set_loop_caps(0, 0) == 0
    assert _create(src, tgt, precision=1) == 0
    assert _create(src, tgt, radius=0.1) == 0


def test_negative_caps_are_invalid():
    assert _capi.lib().dtk_set_loop_caps(-1, 0) == INVALID_ARG


@pytest.mark.parametrize("bad", [float("nan"), float("inf"), -float("inf")])
@pytest.mark.parametrize("cloud", ["source", "target"])
def test_nonfinite_coordinates_are_invalid(clouds, bad, cloud):
    L = _capi.lib()
    n0 = L.dtk_kernel_launch_count()
    assert _create(*clouds) == 0
    ok_launches = L.dtk_kernel_launch_count() - n0
    src, tgt = (c.clone() for c in clouds)
    (src if cloud == "source" else tgt)[17, 1] = bad
    n0 = L.dtk_kernel_launch_count()
    assert _create(src, tgt) == INVALID_ARG
    assert f"{cloud} point coordinates must be finite".encode() in L.dtk_last_error()
    # only the tree build's passes ran on the bad points: the offsets, query
    # record, kNN and setup launches of a good create are missing
    assert L.dtk_kernel_launch_count() - n0 <= ok_launches - 4
    with pytest.raises(dtk.InvalidArgument):
        dtk.NearestNeighborOperator(None, src, tgt)
    # and the context is intact
    assert _create(*clouds) == 0
