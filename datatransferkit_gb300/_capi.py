"""ctypes binding of ``libdtk_gb300.so`` (the C ABI in ``include/dtk_gb300.h``).

The library is built in-tree by ``datatransferkit_gb300.build`` (or
``__graft_entry__.build()``).  There is no fallback: if the library is
missing, loading raises, and every operator call fails loudly.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

_HERE = Path(__file__).resolve().parent
LIB_PATH = _HERE / "libdtk_gb300.so"

# dtk_status
DTK_OK = 0
STATUS_NAMES = {0: "DTK_OK", 1: "DTK_ERR_INVALID_ARG", 2: "DTK_ERR_UNSUPPORTED",
                3: "DTK_ERR_CUDA", 4: "DTK_ERR_OOM", 5: "DTK_ERR_TIMEOUT", 6: "DTK_ERR_INTERNAL"}

# Every function declared in include/dtk_gb300.h.
EXPORTED = [
    "dtk_mls_default_options", "dtk_mls_create", "dtk_mls_apply", "dtk_mls_apply_adjoint",
    "dtk_mls_get_csr", "dtk_mls_get_sizes", "dtk_mls_underdetermined_count",
    "dtk_mls_get_stage_times", "dtk_mls_get_search_times", "dtk_mls_get_rotation_count", "dtk_mls_destroy",
    "dtk_knn_search", "dtk_svd_pinv", "dtk_mls_batch_create", "dtk_mls_batch_apply",
    "dtk_mls_batch_get_csr", "dtk_mls_batch_destroy", "dtk_mls_batch_get_stage_times", "dtk_last_error", "dtk_status_string",
    "dtk_kernel_launch_count", "dtk_svd_pinv_noalloc", "dtk_mls_apply_multi", "dtk_nn_create",
    "dtk_nn_apply", "dtk_nn_apply_multi", "dtk_nn_get_indices", "dtk_nn_destroy",
    "dtk_mls_export_size", "dtk_mls_export", "dtk_mls_import", "dtk_release_cached_memory",
    "dtk_mls_transfer_host", "dtk_set_loop_caps", "dtk_stream_synchronize", "dtk_mls_create_from_neighbors",
    "dtk_mls_batch_resetup", "dtk_mls_batch_get_config", "dtk_set_setup_lanes", "dtk_set_rotation_log",
    "dtk_knn_search_d2", "dtk_points_bounds", "dtk_points_pack", "dtk_gather_points", "dtk_gather_values",
]


class Options(C.Structure):
    _fields_ = [("rbf", C.c_int32), ("basis", C.c_int32), ("k", C.c_int32),
                ("precision", C.c_int32), ("radius", C.c_double), ("comm_size", C.c_int32),
                ("keep_points", C.c_int32)]


class DTKError(RuntimeError):
    """A dtk_status other than DTK_OK (mirrors DataTransferKitException)."""

    def __init__(self, status: int, message: str):
        self.status = status
        self.status_name = STATUS_NAMES.get(status, str(status))
        super().__init__(f"{self.status_name}: {message}")


class InvalidArgument(DTKError, ValueError):
    pass


class Unsupported(DTKError, NotImplementedError):
    pass


_lib = None
_vp = C.c_void_p
_i64 = C.c_int64


def _declare(L):
    L.dtk_mls_default_options.argtypes = [C.POINTER(Options)]
    L.dtk_mls_default_options.restype = None
    L.dtk_mls_create.argtypes = [C.POINTER(Options), _vp, _i64, _i64, _i64, _vp, _i64, _i64, _i64,
                                 _vp, C.POINTER(_vp)]
    L.dtk_mls_apply.argtypes = [_vp, _vp, _i64, _vp, _i64, _vp]
    L.dtk_mls_apply_adjoint.argtypes = [_vp, _vp, _i64, _vp, _vp, _vp, _vp]
    L.dtk_mls_get_csr.argtypes = [_vp, C.POINTER(_vp), C.POINTER(_vp), C.POINTER(_vp),
                                  C.POINTER(_i64), C.POINTER(C.c_int32)]
    L.dtk_mls_get_sizes.argtypes = [_vp, C.POINTER(_i64), C.POINTER(_i64), C.POINTER(_i64)]
    L.dtk_mls_underdetermined_count.argtypes = [_vp, C.POINTER(_i64)]
    L.dtk_mls_get_stage_times.argtypes = [_vp, C.POINTER(C.c_float), C.POINTER(C.c_float)]
    L.dtk_mls_get_search_times.argtypes = [_vp, C.POINTER(C.c_float), C.POINTER(C.c_float)]
    L.dtk_mls_get_rotation_count.argtypes = [_vp, C.POINTER(_i64), C.POINTER(_i64)]
    L.dtk_kernel_launch_count.argtypes = []
    L.dtk_release_cached_memory.argtypes = []
    L.dtk_mls_transfer_host.argtypes = [C.POINTER(Options), _vp, _i64, _vp, _i64, _vp, _vp, _vp,
                                        C.POINTER(_vp)]
    L.dtk_mls_destroy.argtypes = [_vp]
    L.dtk_knn_search.argtypes = [_vp, _i64, _i64, _i64, _vp, _i64, _i64, _i64, C.c_int32, _vp, _vp, _vp]
    L.dtk_svd_pinv.argtypes = [C.c_int32, _i64, _vp, _vp, C.POINTER(_i64), _vp]
    L.dtk_svd_pinv_noalloc.argtypes = L.dtk_svd_pinv.argtypes
    L.dtk_mls_batch_create.argtypes = [C.c_int32, C.POINTER(Options), C.POINTER(_i64), _vp,
                                       C.POINTER(_i64), _vp, _vp, C.POINTER(_vp)]
    L.dtk_mls_batch_apply.argtypes = [_vp, _vp, _vp, C.c_int32, _vp]
    L.dtk_mls_batch_get_csr.argtypes = L.dtk_mls_get_csr.argtypes
    L.dtk_mls_batch_destroy.argtypes = [_vp]
    L.dtk_mls_apply_multi.argtypes = [_vp, _vp, _i64, _i64, _i64, _i64, _vp, _i64, _i64, _i64, _vp]
    L.dtk_nn_create.argtypes = [_vp, _i64, _i64, _i64, _vp, _i64, _i64, _i64, C.c_int32, _vp, C.POINTER(_vp)]
    L.dtk_nn_apply.argtypes = [_vp, _vp, _i64, _vp, _i64, _vp]
    L.dtk_nn_apply_multi.argtypes = L.dtk_mls_apply_multi.argtypes
    L.dtk_nn_get_indices.argtypes = [_vp, C.POINTER(_vp), C.POINTER(_i64)]
    L.dtk_nn_destroy.argtypes = [_vp]
    L.dtk_mls_export_size.argtypes = [_vp, C.POINTER(_i64)]
    L.dtk_mls_export.argtypes = [_vp, _vp, _i64, _vp]
    L.dtk_mls_import.argtypes = [_vp, _i64, _vp, C.POINTER(_vp)]
    L.dtk_mls_batch_get_stage_times.argtypes = [_vp, C.POINTER(C.c_float), C.POINTER(C.c_float),
                                                C.POINTER(C.c_float)]
    L.dtk_set_loop_caps.argtypes = [_i64, _i64]
    L.dtk_stream_synchronize.argtypes = [_vp]
    L.dtk_mls_batch_resetup.argtypes = [_vp, _vp, _vp, _vp]
    L.dtk_knn_search_d2.argtypes = [_vp, _i64, _i64, _i64, _vp, _i64, _i64, _i64, C.c_int32, _vp, _vp, _vp]
    L.dtk_points_bounds.argtypes = [_vp, _i64, _i64, _i64, _vp, _vp]
    L.dtk_points_pack.argtypes = [_vp, _i64, _i64, _i64, _vp, _vp]
    L.dtk_gather_points.argtypes = [_vp, _i64, _i64, _i64, _vp, _i64, _vp, _i64, _vp, _vp]
    L.dtk_gather_values.argtypes = [_vp, _i64, _vp, _i64, _vp, _vp]
    L.dtk_mls_batch_get_config.argtypes = [_vp, _vp, _vp, _vp]
    L.dtk_set_setup_lanes.argtypes = [C.c_int32, C.c_int32]
    L.dtk_set_rotation_log.argtypes = [C.c_int32]
    L.dtk_mls_create_from_neighbors.argtypes = [C.POINTER(Options), _vp, _i64, _i64, _i64, C.c_int32, _vp, _vp,
                                                _i64, _vp, C.POINTER(_vp)]
    L.dtk_last_error.restype = C.c_char_p
    L.dtk_last_error.argtypes = []
    L.dtk_status_string.restype = C.c_char_p
    L.dtk_status_string.argtypes = [C.c_int]
    for name in EXPORTED:
        if name not in ("dtk_last_error", "dtk_status_string", "dtk_mls_default_options"):
            getattr(L, name).restype = C.c_int
    L.dtk_kernel_launch_count.restype = _i64


def lib():
    """The loaded library; raises if it was not built."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise ImportError(
                f"{LIB_PATH} is missing: build the CUDA library first "
                "(python -c 'import __graft_entry__ as g; g.build()'); there is no CPU fallback")
        L = C.CDLL(str(LIB_PATH))
        _declare(L)
        _lib = L
    return _lib


def check(status: int) -> None:
    if status != DTK_OK:
        msg = lib().dtk_last_error().decode(errors="replace")
        if status == 1:
            raise InvalidArgument(status, msg)
        if status == 2:
            raise Unsupported(status, msg)
        raise DTKError(status, msg)
