"""msl_fold_noalloc: the fold entry point that allocates nothing.

It serves callers that cannot allocate device memory -- loops that must not
pay the implicit synchronisation of cudaMalloc/cudaFree, plugins inside a host
whose device memory belongs to that host's own allocator. Its scratch is a static device array, so its results are
checked against the allocating msl_fold on the same input, twice in a row
(the second call reuses the array the first one left behind). The test itself
allocates the input and the one-element result; the entry point does not.

This file is collected last so that a run stopping at its first failure has
run every other test before it.
"""
import ctypes
import math

import numpy as np
import pytest

from muesli4_gb300 import workloads as W

pytestmark = pytest.mark.gpu

U = 2.0 ** -24


def gamma(k):
    return k * U / (1 - k * U)


def noalloc_fold(A, code, op, x_dev, n, dtype):
    res = A.DeviceArray((1,), dtype)
    rc = A.load().msl_fold_noalloc(code, op, x_dev.ptr, n, res.ptr, ctypes.c_void_p(A.stream_handle()))
    A.check(rc, "msl_fold_noalloc")
    A.sync()
    return res.download()[0]


CASES = [
    ("f32 sum", np.float32, "MSL_FOLD_SUM", 1),
    ("f32 sum", np.float32, "MSL_FOLD_SUM", 4099),
    ("f32 sum", np.float32, "MSL_FOLD_SUM", (1 << 24) + 3),
    ("f32 max", np.float32, "MSL_FOLD_MAX", 1000003),
    ("f64 min", np.float64, "MSL_FOLD_MIN", 777777),
    ("i32 sum", np.int32, "MSL_FOLD_SUM", (1 << 22) + 1),
    ("i32 max", np.int32, "MSL_FOLD_MAX", 12345),
]


@pytest.mark.parametrize("name,dtype,op,n", CASES, ids=[f"{c[0]}-{c[3]}" for c in CASES])
def test_noalloc_fold_matches_fold_twice(gpu, name, dtype, op, n):
    rng = np.random.default_rng(n)
    if dtype == np.int32:
        x = rng.integers(-(1 << 30), 1 << 30, n, dtype=np.int32)
    else:
        x = rng.uniform(-1, 1, n).astype(dtype)
    d = gpu.DeviceArray.from_host(x)
    code, opc = gpu.DTYPE_OF[np.dtype(dtype)], getattr(gpu, op)
    want = gpu.fold(opc, d)  # the allocating entry point
    sm, _, _ = gpu.device_info()
    for _ in range(2):
        got = noalloc_fold(gpu, code, opc, d, n, dtype)
        if op == "MSL_FOLD_SUM" and dtype != np.int32:
            # two different summation trees: each within gamma_d * sum|x| of the exact sum
            s_abs = float(np.abs(x.astype(np.float64)).sum())
            d_fold = math.ceil(n / (sm * 4 * 512)) + 64
            d_noalloc = 1024 + 64
            assert abs(float(got) - float(want)) <= (gamma(d_fold) + gamma(d_noalloc)) * s_abs + 1e-30
        else:
            assert got == want


def test_noalloc_fold_two_calls_in_a_row_int_exact(gpu):
    x = W.uniform_i32((1 << 20) + 7, 0, 1000, 44)
    d = gpu.DeviceArray.from_host(x)
    want = gpu.fold(gpu.MSL_FOLD_SUM, d)
    first = noalloc_fold(gpu, gpu.MSL_I32, gpu.MSL_FOLD_SUM, d, x.size, np.int32)
    second = noalloc_fold(gpu, gpu.MSL_I32, gpu.MSL_FOLD_SUM, d, x.size, np.int32)
    assert first == want and second == want


def test_noalloc_fold_rejects_sizes_beyond_its_scratch(gpu):
    d = gpu.DeviceArray((4,), np.float32)
    res = gpu.DeviceArray((1,), np.float32)
    rc = gpu.load().msl_fold_noalloc(gpu.MSL_F32, gpu.MSL_FOLD_SUM, d.ptr, (1 << 30) + 1, res.ptr, None)
    assert rc == gpu.MSL_ERR_SIZE_MISMATCH
    assert b"capacity" in gpu.load().msl_last_error_string()
