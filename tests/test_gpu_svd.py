"""The batched Jacobi pseudo-inverse kernel on the reference's SVD tests
(tstSVD.cpp:67-150) and the golden pseudo-inverses of the reference code."""
from pathlib import Path

import numpy as np
import pytest
import torch

import datatransferkit_gb300 as dtk

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"


def check_identity(mats, pinv, deficient=()):
    prod = np.einsum("bik,bkj->bij", pinv, mats)
    n = mats.shape[1]
    for i in range(n):
        for j in range(n):
            if i == j and i not in deficient:
                np.testing.assert_allclose(prod[:, i, i], 1.0, rtol=1e-12)
            else:
                np.testing.assert_allclose(prod[:, i, j] + 1, 1.0, rtol=1e-12)


def test_svd_full_rank_and_rank_deficient():
    g = dict(np.load(GOLDEN / "svd.npz"))
    p, u = dtk.svd_pinv(torch.from_numpy(g["full"]).cuda())
    p = p.cpu().numpy()
    assert u == 0
    check_identity(g["full"], p)
    assert np.abs(p - g["full_pinv"]).max() <= 1e-12 * np.abs(g["full_pinv"]).max()
    p, u = dtk.svd_pinv(torch.from_numpy(g["deficient"]).cuda())
    p = p.cpu().numpy()
    assert u == 10
    check_identity(g["deficient"], p, deficient={3})
    assert np.abs(p - g["deficient_pinv"]).max() <= 1e-12 * np.abs(g["deficient_pinv"]).max()


def test_svd_zero_and_identity():
    a = np.zeros((3, 5, 5))
    a[1] = np.eye(5)
    a[2] = np.diag([1.0, 2.0, 0.0, 4.0, 1e-20])
    p, u = dtk.svd_pinv(torch.from_numpy(a).cuda())
    p = p.cpu().numpy()
    assert u == 2  # the zero matrix and the one with tiny/zero singular values
    assert np.array_equal(p[0], np.zeros((5, 5)))
    np.testing.assert_allclose(p[1], np.eye(5), rtol=0, atol=1e-15)
    np.testing.assert_allclose(np.diag(p[2]), [1.0, 0.5, 0.0, 0.25, 0.0], rtol=1e-15)
