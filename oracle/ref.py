"""ctypes binding of the reference's own MLS numerics (test infrastructure).

Loads ``oracle/_ref/libdtk_ref.so``: the DataTransferKit headers
DTK_DetailsMovingLeastSquaresOperatorImpl.hpp, DTK_DetailsSVDImpl.hpp,
DTK_CompactlySupportedRadialBasisFunctions.hpp and
DTK_MultivariatePolynomialBasis.hpp compiled unchanged, where they lie,
against the project-written Kokkos/ArborX API shim.  Available only where
the reference sources exist; ``available()`` says whether it is.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import build as _build

_lib = None
_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)


def available() -> bool:
    try:
        return lib() is not None
    except Exception:
        return False


def lib():
    global _lib
    if _lib is None:
        so = _build.build_ref()
        if so is None:
            return None
        L = C.CDLL(str(so))
        L.dtk_ref_mls_coefficients.argtypes = [_dp, _dp, C.c_int64, _ip, _ip, C.c_int, C.c_int, _dp]
        L.dtk_ref_mls_coefficients.restype = C.c_int64
        L.dtk_ref_apply.argtypes = [C.c_int64, _ip, _ip, _dp, _dp, _dp]
        L.dtk_ref_svd_pinv.argtypes = [C.c_int, C.c_int64, _dp, _dp]
        L.dtk_ref_svd_pinv.restype = C.c_int64
        L.dtk_ref_rbf.argtypes = [C.c_int, _dp, C.c_int64, _dp]
        L.dtk_ref_basis.argtypes = [C.c_int, _dp, C.c_int64, _dp]
        _lib = L
    return _lib


def mls_coefficients(src, tgt, offset, idx, rbf, basis):
    src = np.ascontiguousarray(src, np.float64).reshape(-1, 3)
    tgt = np.ascontiguousarray(tgt, np.float64).reshape(-1, 3)
    offset = np.ascontiguousarray(offset, np.int32)
    idx = np.ascontiguousarray(idx, np.int32)
    coeff = np.zeros(int(offset[-1]), np.float64)
    under = lib().dtk_ref_mls_coefficients(src.ctypes.data_as(_dp), tgt.ctypes.data_as(_dp), len(tgt),
                                           offset.ctypes.data_as(_ip), idx.ctypes.data_as(_ip),
                                           int(rbf), int(basis), coeff.ctypes.data_as(_dp))
    if under < 0:
        raise RuntimeError(f"reference setup failed ({under})")
    return coeff, int(under)


def apply(offset, idx, coeff, values):
    offset = np.ascontiguousarray(offset, np.int32)
    idx = np.ascontiguousarray(idx, np.int32)
    coeff = np.ascontiguousarray(coeff, np.float64)
    values = np.ascontiguousarray(values, np.float64)
    out = np.zeros(len(offset) - 1, np.float64)
    lib().dtk_ref_apply(len(out), offset.ctypes.data_as(_ip), idx.ctypes.data_as(_ip),
                        coeff.ctypes.data_as(_dp), values.ctypes.data_as(_dp), out.ctypes.data_as(_dp))
    return out


def svd_pinv(mats):
    mats = np.ascontiguousarray(mats, np.float64)
    count, n, _ = mats.shape
    out = np.zeros_like(mats)
    under = lib().dtk_ref_svd_pinv(n, count, mats.ctypes.data_as(_dp), out.ctypes.data_as(_dp))
    return out, int(under)


def rbf(rbf_id, x):
    x = np.ascontiguousarray(x, np.float64)
    out = np.zeros_like(x)
    lib().dtk_ref_rbf(int(rbf_id), x.ctypes.data_as(_dp), x.size, out.ctypes.data_as(_dp))
    return out


def basis(basis_id, pts):
    pts = np.ascontiguousarray(pts, np.float64).reshape(-1, 3)
    m = {0: 1, 1: 4, 2: 10}[basis_id]
    out = np.zeros((len(pts), m), np.float64)
    lib().dtk_ref_basis(int(basis_id), pts.ctypes.data_as(_dp), len(pts), out.ctypes.data_as(_dp))
    return out
