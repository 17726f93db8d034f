"""dtk_svd_pinv_noalloc: the batched pseudo-inverse for callers that cannot
allocate device memory (fixed device-memory budgets, frameworks whose
allocator owns the device, code that cannot take an allocation's implicit
synchronisation).  It runs the same kernel as dtk_svd_pinv on a static device
work area, so both entry points must agree, within the SVD tests' tolerance
(1e-12 relative), on two calls in a row through the C ABI -- the second call
also shows that the shared work area and its counters carry nothing over.
This file is collected last on purpose."""
import ctypes as C
from pathlib import Path

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"
TOL = 1e-12


def _call(lib, fn, mats: torch.Tensor):
    out = torch.full_like(mats, np.nan)
    under = C.c_int64(-1)
    status = getattr(lib, fn)(mats.shape[1], mats.shape[0], mats.data_ptr(), out.data_ptr(),
                             C.byref(under), torch.cuda.current_stream().cuda_stream)
    assert status == 0, lib.dtk_last_error()
    torch.cuda.synchronize()
    return out.cpu().numpy(), under.value


def test_noalloc_matches_allocating_entry_point_twice(dtk_lib):
    g = dict(np.load(GOLDEN / "svd.npz"))
    # first call: 10 rank-deficient 40x40 matrices; second: 10 full-rank 32x32
    for name, expect_under in (("deficient", 10), ("full", 0)):
        mats = torch.from_numpy(g[name]).cuda()
        p_ref, u_ref = _call(dtk_lib, "dtk_svd_pinv", mats)
        p_new, u_new = _call(dtk_lib, "dtk_svd_pinv_noalloc", mats)
        assert u_ref == u_new == expect_under
        scale = np.abs(p_ref).max()
        assert np.abs(p_new - p_ref).max() <= TOL * scale
        assert np.abs(p_new - g[f"{name}_pinv"]).max() <= TOL * np.abs(g[f"{name}_pinv"]).max()


def test_noalloc_rejects_requests_beyond_its_work_area(dtk_lib):
    n, count = 64, (1 << 20) // (3 * 64 * 64) + 1  # one matrix too many
    status = dtk_lib.dtk_svd_pinv_noalloc(n, count, 1, 1, None, None)
    assert status == 1  # DTK_ERR_INVALID_ARG, before any device work
    assert b"static work area" in dtk_lib.dtk_last_error()
