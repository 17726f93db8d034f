"""The C-ABI device steps of the distributed operators (dtk_knn_search_d2,
dtk_points_bounds, dtk_points_pack, dtk_gather_points, dtk_gather_values)
against the oracle and numpy, with their argument checks."""
import ctypes as C

import numpy as np
import pytest
import torch

from datatransferkit_gb300 import _capi
from datatransferkit_gb300 import synthetic as syn
from datatransferkit_gb300._capi import lib
from oracle import cpu

pytestmark = pytest.mark.gpu


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def test_knn_search_d2_matches_the_oracle():
    src, tgt = syn.uniform_points(5000, 3), syn.uniform_points(700, 4)
    for k in (1, 7, 32):
        idx = torch.empty((len(tgt), k), dtype=torch.int32, device="cuda")
        d2 = torch.empty((len(tgt), k), dtype=torch.float64, device="cuda")
        s, t = dev(src), dev(tgt)
        assert lib().dtk_knn_search_d2(s.data_ptr(), len(src), 3, 1, t.data_ptr(), len(tgt), 3, 1, k,
                                       idx.data_ptr(), d2.data_ptr(), None) == 0
        torch.cuda.synchronize()
        _, ri, rd = cpu.knn(src, tgt, k)
        assert np.array_equal(idx.cpu().numpy().reshape(-1), ri)
        assert np.array_equal(d2.cpu().numpy().reshape(-1), rd)  # the same formula, bit for bit
    # LayoutLeft sources, fewer sources than k: rows of n_src
    few = np.ascontiguousarray(src[:5].T)
    idx = torch.empty((len(tgt), 5), dtype=torch.int32, device="cuda")
    d2 = torch.empty((len(tgt), 5), dtype=torch.float64, device="cuda")
    f = dev(few)
    t = dev(tgt)
    assert lib().dtk_knn_search_d2(f.data_ptr(), 5, 1, 5, t.data_ptr(), len(tgt), 3, 1, 32, idx.data_ptr(),
                                   d2.data_ptr(), None) == 0
    _, ri, rd = cpu.knn(src[:5], tgt, 32)
    assert np.array_equal(idx.cpu().numpy().reshape(-1), ri) and np.array_equal(d2.cpu().numpy().reshape(-1), rd)
    assert lib().dtk_knn_search_d2(f.data_ptr(), 5, 1, 5, t.data_ptr(), len(tgt), 3, 1, 33, idx.data_ptr(),
                                   d2.data_ptr(), None) == 2  # k <= 32


def test_bounds_and_pack():
    pts = syn.uniform_points(10_001, 5) * np.array([2.0, -1.0, 0.5]) + np.array([-3.0, 0.25, 7.0])
    for layout in ("right", "left"):
        a = pts if layout == "right" else np.ascontiguousarray(pts.T)
        d = dev(a)
        ps, ds = (3, 1) if layout == "right" else (1, len(pts))
        box = (C.c_double * 6)()
        assert lib().dtk_points_bounds(d.data_ptr(), len(pts), ps, ds, box, None) == 0
        assert list(box) == list(pts.min(0)) + list(pts.max(0))
        out = torch.empty((len(pts), 3), dtype=torch.float64, device="cuda")
        assert lib().dtk_points_pack(d.data_ptr(), len(pts), ps, ds, out.data_ptr(), None) == 0
        assert np.array_equal(out.cpu().numpy(), pts)
    box = (C.c_double * 6)()
    assert lib().dtk_points_bounds(None, 0, 3, 1, box, None) == 0
    assert list(box) == [np.inf] * 3 + [-np.inf] * 3


def test_gathers_and_their_index_checks():
    src = syn.uniform_points(100, 6)
    extra = syn.uniform_points(7, 7)
    idx = np.array([0, 99, 100, 106, 5], dtype=np.int32)
    s, e, i = dev(src), dev(extra), dev(idx)
    out = torch.empty((len(idx), 3), dtype=torch.float64, device="cuda")
    assert lib().dtk_gather_points(s.data_ptr(), 100, 3, 1, e.data_ptr(), 7, i.data_ptr(), len(idx),
                                   out.data_ptr(), None) == 0
    want = np.concatenate([src, extra])[idx]
    assert np.array_equal(out.cpu().numpy(), want)
    bad = dev(np.array([107], dtype=np.int32))
    assert lib().dtk_gather_points(s.data_ptr(), 100, 3, 1, e.data_ptr(), 7, bad.data_ptr(), 1, out.data_ptr(),
                                   None) == 1
    vals = dev(np.arange(10.0))
    vi = dev(np.array([9, 0, 3], dtype=np.int32))
    vo = torch.empty(3, dtype=torch.float64, device="cuda")
    assert lib().dtk_gather_values(vals.data_ptr(), 10, vi.data_ptr(), 3, vo.data_ptr(), None) == 0
    assert vo.cpu().tolist() == [9.0, 0.0, 3.0]
    vb = dev(np.array([10], dtype=np.int32))
    assert lib().dtk_gather_values(vals.data_ptr(), 10, vb.data_ptr(), 1, vo.data_ptr(), None) == 1
    assert b"DTK_REQUIRE" in lib().dtk_last_error()
    # host memory is refused before any kernel
    host = np.zeros(3)
    assert lib().dtk_gather_values(host.ctypes.data, 3, vi.data_ptr(), 3, vo.data_ptr(), None) == 1
