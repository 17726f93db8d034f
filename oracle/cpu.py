"""ctypes binding of the FP64 CPU oracle (dtk_oracle.cpp) -- test infrastructure.

Every function takes/returns numpy arrays.  Point arrays are (n, 3) float64
C-contiguous.  RBF ids: 0..3 = Wendland<0,2,4,6>, 4..5 = Wu<2,4>,
6..8 = Buhmann<2,3,4>.  Basis ids: 0 = Constant3, 1 = Linear3, 2 = Quadratic3.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import build as _build

_lib = None
_lib_contract = None

RBF_IDS = {"wendland0": 0, "wendland2": 1, "wendland4": 2, "wendland6": 3,
           "wu2": 4, "wu4": 5, "buhmann2": 6, "buhmann3": 7, "buhmann4": 8}
BASIS_SIZE = {0: 1, 1: 4, 2: 10}

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)


def lib(contract: bool = False):
    """The oracle library; contract=True gives its multiply-add-contracted build."""
    global _lib, _lib_contract
    if contract:
        if _lib_contract is None:
            _lib_contract = _declare(C.CDLL(str(_build.build_oracle(contract=True))))
        return _lib_contract
    if _lib is None:
        _lib = _declare(C.CDLL(str(_build.build_oracle())))
    return _lib


def _declare(L):
    L.dtk_oracle_knn.argtypes = [_dp, C.c_int64, _dp, C.c_int64, C.c_int, _ip, _ip, _dp]
    L.dtk_oracle_knn_brute.argtypes = L.dtk_oracle_knn.argtypes
    L.dtk_oracle_radius_count.argtypes = [_dp, C.c_int64, _dp, C.c_int64, C.c_double, _ip]
    L.dtk_oracle_radius_count.restype = C.c_int64
    L.dtk_oracle_radius_fill.argtypes = [_dp, C.c_int64, _dp, C.c_int64, C.c_double, _ip, _ip, _dp]
    L.dtk_oracle_mls_coefficients.argtypes = [_dp, _dp, C.c_int64, _ip, _ip, C.c_int, C.c_int, _dp, _dp, _dp]
    L.dtk_oracle_mls_coefficients.restype = C.c_int64
    L.dtk_oracle_apply.argtypes = [C.c_int64, _ip, _ip, _dp, _dp, _dp]
    L.dtk_oracle_apply_transpose.argtypes = [C.c_int64, C.c_int64, _ip, _ip, _dp, _dp, _dp]
    L.dtk_oracle_coord_grad.argtypes = [_dp, C.c_int64, _dp, C.c_int64, _ip, _ip, C.c_int, C.c_int, _dp, _dp, _dp]
    L.dtk_oracle_svd_pinv.argtypes = [C.c_int, C.c_int64, _dp, _dp]
    L.dtk_oracle_svd_pinv.restype = C.c_int64
    L.dtk_oracle_rbf.argtypes = [C.c_int, _dp, C.c_int64, _dp]
    L.dtk_oracle_basis.argtypes = [C.c_int, _dp, C.c_int64, _dp]
    L.dtk_oracle_max_threads.restype = C.c_int
    L.dtk_oracle_set_threads.argtypes = [C.c_int]
    return L


def _d(a):
    return a.ctypes.data_as(_dp) if a is not None else None


def _i(a):
    return a.ctypes.data_as(_ip) if a is not None else None


def _pts(p):
    p = np.ascontiguousarray(p, dtype=np.float64)
    if p.size == 0:
        p = p.reshape(0, 3)
    assert p.ndim == 2 and p.shape[1] == 3
    return p


def max_threads() -> int:
    return lib().dtk_oracle_max_threads()


def set_threads(n: int) -> None:
    lib().dtk_oracle_set_threads(int(n))


def knn(src, tgt, k, brute=False):
    """Exact kNN (offset, idx, d2) under the (d2, index) contract."""
    src, tgt = _pts(src), _pts(tgt)
    row = min(int(k), len(src))
    offset = np.zeros(len(tgt) + 1, np.int32)
    idx = np.zeros(len(tgt) * row, np.int32)
    d2 = np.zeros(len(tgt) * row, np.float64)
    f = lib().dtk_oracle_knn_brute if brute else lib().dtk_oracle_knn
    rc = f(_d(src), len(src), _d(tgt), len(tgt), int(k), _i(offset), _i(idx), _d(d2))
    if rc != 0:
        raise ValueError("oracle knn rejected its arguments")
    return offset, idx, d2


def radius(src, tgt, r):
    """All sources with sqrt(d2) <= r, rows ascending by (d2, index)."""
    src, tgt = _pts(src), _pts(tgt)
    offset = np.zeros(len(tgt) + 1, np.int32)
    nnz = lib().dtk_oracle_radius_count(_d(src), len(src), _d(tgt), len(tgt), float(r), _i(offset))
    if nnz < 0:
        raise ValueError("oracle radius search rejected its arguments")
    idx = np.zeros(nnz, np.int32)
    d2 = np.zeros(nnz, np.float64)
    lib().dtk_oracle_radius_fill(_d(src), len(src), _d(tgt), len(tgt), float(r), _i(offset), _i(idx), _d(d2))
    return offset, idx, d2


def mls_coefficients(src, tgt, offset, idx, rbf, basis, want_row0=False, contract=False):
    """(coeff, radius, row0|None, n_underdetermined) for given connectivity."""
    src, tgt = _pts(src), _pts(tgt)
    offset = np.ascontiguousarray(offset, np.int32)
    idx = np.ascontiguousarray(idx, np.int32)
    m = BASIS_SIZE[basis]
    coeff = np.zeros(int(offset[-1]), np.float64)
    rad = np.zeros(len(tgt), np.float64)
    row0 = np.zeros(len(tgt) * m, np.float64) if want_row0 else None
    under = lib(contract).dtk_oracle_mls_coefficients(_d(src), _d(tgt), len(tgt), _i(offset), _i(idx),
                                              int(rbf), int(basis), _d(coeff), _d(rad), _d(row0))
    if under < 0:
        raise ValueError("oracle setup rejected its arguments")
    return coeff, rad, (row0.reshape(len(tgt), m) if want_row0 else None), int(under)


def apply(offset, idx, coeff, values):
    offset = np.ascontiguousarray(offset, np.int32)
    idx = np.ascontiguousarray(idx, np.int32)
    coeff = np.ascontiguousarray(coeff, np.float64)
    values = np.ascontiguousarray(values, np.float64)
    out = np.zeros(len(offset) - 1, np.float64)
    lib().dtk_oracle_apply(len(out), _i(offset), _i(idx), _d(coeff), _d(values), _d(out))
    return out


def apply_transpose(offset, idx, coeff, cot, n_src):
    offset = np.ascontiguousarray(offset, np.int32)
    idx = np.ascontiguousarray(idx, np.int32)
    coeff = np.ascontiguousarray(coeff, np.float64)
    cot = np.ascontiguousarray(cot, np.float64)
    g = np.zeros(n_src, np.float64)
    lib().dtk_oracle_apply_transpose(len(offset) - 1, n_src, _i(offset), _i(idx), _d(coeff), _d(cot), _d(g))
    return g


def coord_grad(src, tgt, offset, idx, rbf, basis, values, cot):
    src, tgt = _pts(src), _pts(tgt)
    offset = np.ascontiguousarray(offset, np.int32)
    idx = np.ascontiguousarray(idx, np.int32)
    values = np.ascontiguousarray(values, np.float64)
    cot = np.ascontiguousarray(cot, np.float64)
    g = np.zeros((len(src), 3), np.float64)
    rc = lib().dtk_oracle_coord_grad(_d(src), len(src), _d(tgt), len(tgt), _i(offset), _i(idx),
                                     int(rbf), int(basis), _d(values), _d(cot), _d(g))
    if rc != 0:
        raise ValueError("oracle coord_grad rejected its arguments")
    return g


def svd_pinv(mats):
    """Batched DTK Jacobi pseudo-inverse; returns (pinv, n_underdetermined)."""
    mats = np.ascontiguousarray(mats, np.float64)
    count, n, _ = mats.shape
    out = np.zeros_like(mats)
    under = lib().dtk_oracle_svd_pinv(n, count, _d(mats), _d(out))
    return out, int(under)


def rbf(rbf_id, x):
    x = np.ascontiguousarray(x, np.float64)
    out = np.zeros_like(x)
    lib().dtk_oracle_rbf(int(rbf_id), _d(x), x.size, _d(out))
    return out


def basis(basis_id, pts):
    pts = _pts(pts)
    out = np.zeros((len(pts), BASIS_SIZE[basis_id]), np.float64)
    lib().dtk_oracle_basis(int(basis_id), _d(pts), len(pts), _d(out))
    return out


def mls_transfer(src, tgt, values, rbf_id, basis_id, k=None, r=None):
    """Whole reference pipeline: search, setup, apply.  Returns a dict."""
    if r is not None:
        offset, idx, d2 = radius(src, tgt, r)
    else:
        offset, idx, d2 = knn(src, tgt, BASIS_SIZE[basis_id] if k is None else k)
    coeff, rad, _, under = mls_coefficients(src, tgt, offset, idx, rbf_id, basis_id)
    out = apply(offset, idx, coeff, values)
    return dict(offset=offset, idx=idx, d2=d2, coeff=coeff, radius=rad,
                underdetermined=under, target=out)


def rounding_spread(src, tgt, offset, idx, rbf, basis, values, coeff=None):
    """How far the reference algorithm moves under another valid rounding.

    Returns (coefficient spread, target spread): the largest per-row
    max|c - c'| / max|c| and the relative L2 distance of the transferred
    values between the oracle and its multiply-add-contracted build.
    """
    if coeff is None:
        coeff = mls_coefficients(src, tgt, offset, idx, rbf, basis)[0]
    c2 = mls_coefficients(src, tgt, offset, idx, rbf, basis, contract=True)[0]
    worst = 0.0
    offset = np.asarray(offset)
    for i in range(len(offset) - 1):
        a, b = c2[offset[i]:offset[i + 1]], coeff[offset[i]:offset[i + 1]]
        if len(b):
            worst = max(worst, float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)))
    y = apply(offset, idx, coeff, values)
    y2 = apply(offset, idx, c2, values)
    ny = np.linalg.norm(y)
    return worst, float(np.linalg.norm(y2 - y) / (ny if ny > 0 else 1.0))
