"""C-ABI checks that need no GPU: the library builds for sm_103a, loads, and
exports every function include/msl_gb300.h declares; calls before msl_init
fail with a status code instead of crashing or exiting."""
import ctypes

import pytest

from muesli4_gb300 import abi, build


@pytest.fixture(scope="module")
def lib():
    build.build()
    return abi.load()


def test_header_declares_the_hot_path(lib):
    names = abi.declared_functions()
    for required in ("msl_init", "msl_map", "msl_zip", "msl_zip3", "msl_map_index", "msl_zip_index", "msl_fold",
                     "msl_fold_absdiff_max", "msl_copy", "msl_download", "msl_stencil2d", "msl_stencil2d_iterate",
                     "msl_stencil3d", "msl_stencil3d_iterate"):
        assert required in names


def test_every_declared_symbol_is_exported(lib):
    missing = [n for n in abi.declared_functions() if not hasattr(lib, n)]
    assert not missing


def test_every_declared_function_has_ctypes_signature(lib):
    """ctypes passes the arguments of a function without argtypes as C ints,
    which truncates 64-bit pointers and sizes: the binding must type every
    entry point the header declares."""
    untyped = [n for n in abi.declared_functions() if getattr(lib, n).argtypes is None]
    assert not untyped
    assert all(getattr(lib, n).restype is not None for n in abi.declared_functions())


def test_calls_before_init_report_not_initialized(lib):
    p = ctypes.c_void_p()
    assert lib.msl_alloc(ctypes.byref(p), 16) == abi.MSL_ERR_NOT_INITIALIZED
    assert b"msl_init" in lib.msl_last_error_string()
    assert lib.msl_map(abi.MSL_F32, abi.MSL_MAP_AFFINE, None, None, 4, None) == abi.MSL_ERR_NOT_INITIALIZED
    assert lib.msl_fold(abi.MSL_F32, abi.MSL_FOLD_SUM, None, 4, None) == abi.MSL_ERR_NOT_INITIALIZED
    assert lib.msl_terminate() == abi.MSL_OK  # terminating an idle library is a no-op
    c = ctypes.c_ulonglong()
    assert lib.msl_launch_count(ctypes.byref(c)) == abi.MSL_OK


def test_init_without_a_device_fails_cleanly(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    rc = lib.msl_init(0)
    assert rc in (abi.MSL_ERR_CUDA, abi.MSL_ERR_INVALID_ARGUMENT)
    assert lib.msl_last_error_string()


def test_status_codes_are_distinct():
    codes = [v for k, v in vars(abi).items() if k.startswith("MSL_ERR_")]
    assert len(codes) == len(set(codes)) and all(c < 0 for c in codes)


def test_setters_validate_their_arguments(lib):
    """Process-wide settings need no device; out-of-range values are refused
    with INVALID_ARGUMENT and leave the setting unchanged."""
    bad = abi.MSL_ERR_INVALID_ARGUMENT
    assert lib.msl_set_temporal_depth(33) == bad and lib.msl_set_temporal_depth(-1) == bad
    assert lib.msl_set_temporal_depth(32) == abi.MSL_OK and lib.msl_set_temporal_depth(0) == abi.MSL_OK
    assert lib.msl_set_stencil3d_depth(0) == bad and lib.msl_set_stencil3d_depth(3) == bad
    assert lib.msl_set_stencil3d_depth(1) == abi.MSL_OK and lib.msl_set_stencil3d_depth(2) == abi.MSL_OK
    assert lib.msl_set_stencil3d_zchunk(-1) == bad and lib.msl_set_stencil3d_zchunk(1025) == bad
    assert lib.msl_set_stencil3d_zchunk(1) == abi.MSL_OK and lib.msl_set_stencil3d_zchunk(0) == abi.MSL_OK
    assert lib.msl_set_stencil3d_persistent(2) == bad and lib.msl_set_stencil3d_persistent(-2) == bad
    assert lib.msl_set_stencil3d_persistent(-1) == abi.MSL_OK
    assert lib.msl_set_tma(0) == abi.MSL_OK and lib.msl_set_tma(1) == abi.MSL_OK


def test_injected_allocation_failures_need_no_device(lib):
    """The host-side allocation fault hook: after `after` allowed allocations,
    msl_alloc and msl_batch_create fail with OUT_OF_MEMORY (checked before the
    device is needed, so it runs here); -1 turns it off again."""
    p = ctypes.c_void_p()
    rows = (ctypes.c_int * 1)(64)
    h = ctypes.c_void_p()
    try:
        assert lib.msl_debug_fail_allocs(0) == abi.MSL_OK
        assert lib.msl_alloc(ctypes.byref(p), 16) == abi.MSL_ERR_OUT_OF_MEMORY
        assert b"injected" in lib.msl_last_error_string()
        assert lib.msl_batch_create(abi.MSL_F32, 1, rows, rows, 0, ctypes.byref(h)) == abi.MSL_ERR_OUT_OF_MEMORY
        assert not h.value
        assert lib.msl_debug_fail_allocs(2) == abi.MSL_OK
        # two allocations pass the hook (and then need the device), the third fails
        assert lib.msl_alloc(ctypes.byref(p), 16) == abi.MSL_ERR_NOT_INITIALIZED
        assert lib.msl_batch_create(abi.MSL_F32, 1, rows, rows, 0, ctypes.byref(h)) == abi.MSL_ERR_NOT_INITIALIZED
        assert lib.msl_alloc(ctypes.byref(p), 16) == abi.MSL_ERR_OUT_OF_MEMORY
        assert lib.msl_alloc(ctypes.byref(p), 0) == abi.MSL_ERR_NOT_INITIALIZED  # zero bytes allocate nothing
    finally:
        lib.msl_debug_fail_allocs(-1)
    assert lib.msl_alloc(ctypes.byref(p), 16) == abi.MSL_ERR_NOT_INITIALIZED


def test_failure_detection_calls_before_init(lib):
    assert lib.msl_set_wait_limit(4) == abi.MSL_ERR_NOT_INITIALIZED
    assert lib.msl_wait_selftest(4, 0) == abi.MSL_ERR_NOT_INITIALIZED
    assert lib.msl_server_cancel(None, 1) == abi.MSL_ERR_INVALID_ARGUMENT


def test_tile_rows_setter_needs_no_device(lib):
    bad = abi.MSL_ERR_INVALID_ARGUMENT
    assert lib.msl_set_tile_rows(24) == bad and lib.msl_set_tile_rows(-1) == bad and lib.msl_set_tile_rows(128) == bad
    for ok in (16, 32, 64, 0):
        assert lib.msl_set_tile_rows(ok) == abi.MSL_OK


def _server_checkpoint(records):
    """A server checkpoint in the library's layout: magic, header (tol,
    max_iters, check_every, depth2d, budget, next_id, count), one record per
    request (id, kind, state, depth, rows, cols, pad, iters, residual), then
    every request's FP32 cells in record order."""
    import struct
    out = b"MSLSRV01" + struct.pack("<dqiiQqq", 1e-4, 1000, 10, 2, 0, 10, len(records))
    for rid, state in records:
        out += struct.pack("<qiiiiiiqd", rid, 0, state, 1, 3, 4, 0, 20, 0.5)
    for _ in records:
        out += struct.pack("<12f", *range(12))
    return out


def test_server_restore_rejects_repeated_request_ids(lib, tmp_path):
    """The restore parses and checks the whole file before it touches the
    device: a well-formed checkpoint gets as far as starting a server (which
    needs msl_init), one that names a request id twice is rejected."""
    import ctypes
    h = ctypes.c_void_p()
    good = tmp_path / "good.ckpt"
    good.write_bytes(_server_checkpoint([(1, 0), (2, 1), (3, 2)]))
    assert lib.msl_server_restore(str(good).encode(), ctypes.byref(h)) == abi.MSL_ERR_NOT_INITIALIZED
    bad = tmp_path / "repeated.ckpt"
    bad.write_bytes(_server_checkpoint([(1, 0), (2, 1), (1, 1)]))
    assert lib.msl_server_restore(str(bad).encode(), ctypes.byref(h)) == abi.MSL_ERR_INVALID_ARGUMENT
    assert b"not a complete server checkpoint" in lib.msl_last_error_string()
    assert not h.value
