"""C ABI checks that need no GPU: the library loads, exports every function
that include/dtk_gb300.h declares, and rejects bad arguments with the
reference's error convention (DTK_REQUIRE -> DTK_ERR_INVALID_ARG) before it
touches the device."""
import ctypes as C
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_functions():
    text = (ROOT / "include" / "dtk_gb300.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"\b(dtk_[a-z0-9_]+)\s*\(", text)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("dtk_mls_create", "dtk_mls_apply", "dtk_mls_destroy", "dtk_mls_apply_adjoint",
                 "dtk_knn_search", "dtk_svd_pinv", "dtk_mls_batch_create"):
        assert must in names


def test_library_exports_every_declared_symbol(dtk_lib):
    missing = [n for n in declared_functions() if not hasattr(dtk_lib, n)]
    assert not missing, missing
    from datatransferkit_gb300 import _capi
    assert sorted(_capi.EXPORTED) == declared_functions()


def test_default_options_mirror_template_defaults(dtk_lib):
    from datatransferkit_gb300._capi import Options
    o = Options()
    dtk_lib.dtk_mls_default_options(C.byref(o))
    # MovingLeastSquaresOperator<Device, Wendland<0>, MultivariatePolynomialBasis<Linear, 3>>
    assert (o.rbf, o.basis, o.k, o.precision, o.radius, o.comm_size) == (0, 1, 0, 0, 0.0, 1)


def _create(dtk_lib, o, n_src=4, n_tgt=2, src=1, tgt=1):
    h = C.c_void_p()
    st = dtk_lib.dtk_mls_create(C.byref(o), src, n_src, 3, 1, tgt, n_tgt, 3, 1, None, C.byref(h))
    return st, h


def test_create_rejects_bad_arguments_before_device_work(dtk_lib):
    from datatransferkit_gb300._capi import Options
    o = Options()
    dtk_lib.dtk_mls_default_options(C.byref(o))
    o.comm_size = 2
    st, h = _create(dtk_lib, o)
    assert st == 2 and not h.value  # DTK_ERR_UNSUPPORTED: one rank only
    assert b"single-rank" in dtk_lib.dtk_last_error()
    dtk_lib.dtk_mls_default_options(C.byref(o))
    o.rbf = 42
    assert _create(dtk_lib, o)[0] == 1
    dtk_lib.dtk_mls_default_options(C.byref(o))
    o.k = 33
    assert _create(dtk_lib, o)[0] == 2  # kNN limited to k <= 32
    dtk_lib.dtk_mls_default_options(C.byref(o))
    o.radius = float("nan")
    assert _create(dtk_lib, o)[0] == 1
    dtk_lib.dtk_mls_default_options(C.byref(o))
    # empty source cloud: DTK_CHECK(!search_tree.empty())
    assert _create(dtk_lib, o, n_src=0)[0] == 1
    assert b"empty" in dtk_lib.dtk_last_error()
    # null pointers with non-zero counts
    assert _create(dtk_lib, o, src=None)[0] == 1
    assert _create(dtk_lib, o, tgt=None)[0] == 1
    assert dtk_lib.dtk_mls_create(None, 1, 4, 3, 1, 1, 2, 3, 1, None, C.byref(C.c_void_p())) == 1


def test_apply_and_queries_reject_null_handle(dtk_lib):
    assert dtk_lib.dtk_mls_apply(None, None, 0, None, 0, None) == 1
    n = C.c_int64()
    assert dtk_lib.dtk_mls_underdetermined_count(None, C.byref(n)) == 1
    assert dtk_lib.dtk_mls_destroy(None) == 0


HANDLE_ENTRIES = ("dtk_mls_apply", "dtk_mls_apply_adjoint", "dtk_mls_apply_multi", "dtk_mls_get_csr",
                  "dtk_mls_get_sizes", "dtk_mls_underdetermined_count", "dtk_mls_get_stage_times",
                  "dtk_mls_get_search_times", "dtk_mls_get_rotation_count", "dtk_mls_export_size",
                  "dtk_mls_export", "dtk_nn_apply", "dtk_nn_apply_multi", "dtk_nn_get_indices",
                  "dtk_mls_batch_apply", "dtk_mls_batch_get_csr", "dtk_mls_batch_get_stage_times",
                  "dtk_mls_batch_resetup", "dtk_mls_batch_get_config")
CREATE_ENTRIES = ("dtk_mls_import", "dtk_mls_transfer_host", "dtk_nn_create", "dtk_knn_search",
                  "dtk_mls_batch_create", "dtk_svd_pinv_noalloc", "dtk_mls_create_from_neighbors",
                  "dtk_knn_search_d2", "dtk_points_bounds")


def _null_args(fn):
    return [0 if t in (C.c_int64, C.c_int32, C.c_int) else None for t in fn.argtypes]


def test_every_entry_rejects_null_arguments(dtk_lib):
    # a null handle (or null inputs) is DTK_ERR_INVALID_ARG with a message,
    # decided before any device call; destroying a null handle is a no-op
    for name in HANDLE_ENTRIES + CREATE_ENTRIES:
        fn = getattr(dtk_lib, name)
        assert fn(*_null_args(fn)) == 1, name
        assert dtk_lib.dtk_last_error().startswith(b"DTK_REQUIRE"), name
    for name in ("dtk_mls_destroy", "dtk_nn_destroy", "dtk_mls_batch_destroy"):
        assert getattr(dtk_lib, name)(None) == 0, name


def test_create_from_neighbors_rejects_bad_arguments_before_device_work(dtk_lib):
    from datatransferkit_gb300._capi import Options
    o = Options()

    def create(row=4, n_src=10, nb=1, idx=1, n_tgt=2):
        h = C.c_void_p()
        st = dtk_lib.dtk_mls_create_from_neighbors(C.byref(o), 1, n_tgt, 3, 1, row, nb, idx, n_src, None,
                                                   C.byref(h))
        assert not h.value
        return st

    dtk_lib.dtk_mls_default_options(C.byref(o))
    o.radius = 0.5
    assert create() == 2  # kNN rows only
    dtk_lib.dtk_mls_default_options(C.byref(o))
    o.keep_points = 1
    assert create() == 2  # no points are kept for the coordinate adjoint
    dtk_lib.dtk_mls_default_options(C.byref(o))
    o.comm_size = 2
    assert create() == 2  # the handle is one rank's part
    dtk_lib.dtk_mls_default_options(C.byref(o))
    assert create(row=0) == 1 and create(row=33) == 1
    assert create(n_src=0) == 1 and create(n_src=1 << 31) == 1
    assert create(nb=None) == 1 and create(idx=None) == 1
    assert create(n_tgt=(1 << 31) // 4) == 1  # n_targets * row beyond int32 offsets
    assert b"DTK_REQUIRE" in dtk_lib.dtk_last_error()


def test_setup_lanes_accept_powers_of_two_only(dtk_lib):
    for bad in ((3, 8), (8, 64), (-1, 0), (0, 48)):
        assert dtk_lib.dtk_set_setup_lanes(*bad) == 1
    assert dtk_lib.dtk_set_setup_lanes(4, 16) == 0
    assert dtk_lib.dtk_set_setup_lanes(0, 0) == 0  # back to tuning


def test_rotation_log_range(dtk_lib):
    for bad in (-1, 161):
        assert dtk_lib.dtk_set_rotation_log(bad) == 1
    assert dtk_lib.dtk_set_rotation_log(0) == 0
    assert dtk_lib.dtk_set_rotation_log(160) == 0  # the default


def test_svd_rejects_bad_sizes(dtk_lib):
    assert dtk_lib.dtk_svd_pinv(0, 1, 1, 1, None, None) == 1
    assert dtk_lib.dtk_svd_pinv(65, 1, 1, 1, None, None) == 1


def test_noalloc_rejects_counts_whose_work_size_would_overflow(dtk_lib):
    # 3 n^2 count overflows int64 for these counts: the bound on count comes
    # first, so they are refused before any device call
    for n, count in ((64, (1 << 63) // 8), (64, (1 << 63) - 1), (1, (1 << 62))):
        assert dtk_lib.dtk_svd_pinv_noalloc(n, count, 1, 1, None, None) == 1
        assert b"static work area" in dtk_lib.dtk_last_error()


def test_status_strings(dtk_lib):
    for s, name in [(0, b"DTK_OK"), (1, b"DTK_ERR_INVALID_ARG"), (5, b"DTK_ERR_TIMEOUT")]:
        assert dtk_lib.dtk_status_string(s) == name


def test_python_operator_rejects_host_tensors():
    torch = pytest.importorskip("torch")
    import datatransferkit_gb300 as dtk
    with pytest.raises(dtk.InvalidArgument):
        dtk.MovingLeastSquaresOperator(None, torch.zeros(4, 3, dtype=torch.float64),
                                       torch.zeros(2, 3, dtype=torch.float64))
