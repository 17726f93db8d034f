"""The library's device memory pool: blocks freed by a destroyed operator stay
cached (so the next setup maps no memory), and release_cached_memory returns
them to the driver; memory of live operators is not touched."""
import numpy as np
import pytest
import torch

import datatransferkit_gb300 as dtk
from datatransferkit_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu
MB = 1 << 20


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def free_bytes():
    torch.cuda.synchronize()
    return torch.cuda.mem_get_info()[0]


def test_pool_caches_then_releases():
    src = dev(syn.uniform_points(1_000_000, 61))
    tgt = dev(syn.uniform_points(1_000_000, 62))
    vals = dev(syn.smooth_field(src.cpu().numpy()))
    out = torch.empty(1_000_000, dtype=torch.float64, device="cuda")
    dtk.release_cached_memory()
    free0 = free_bytes()
    op = dtk.MovingLeastSquaresOperator(None, src, tgt, k=32)
    op.apply(vals, out)
    keep = dtk.MovingLeastSquaresOperator(None, src[:1000], tgt[:1000], k=8)  # stays alive
    op.close()
    free1 = free_bytes()
    assert free1 < free0 - 100 * MB  # the CSR (32M entries) and the scratch stay cached
    dtk.release_cached_memory()
    free2 = free_bytes()
    assert free2 > free1 + 100 * MB
    # only the live operator's buffers remain: its small allocations may sit
    # in (and keep mapped) one block the pool carved for a larger transient
    # buffer of the first setup (the 64 MB of query records at 1M targets);
    # the first operator's CSR alone is 384 MB
    assert free2 > free0 - 128 * MB
    y = torch.empty(1000, dtype=torch.float64, device="cuda")
    keep.apply(vals[:1000], y)  # still usable after the release
    assert torch.isfinite(y).all()
