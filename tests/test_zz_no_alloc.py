"""msl_fold_noalloc: the fold entry point that allocates nothing.

It serves callers that cannot allocate device memory -- loops that must not
pay the implicit synchronisation of cudaMalloc/cudaFree, plugins inside a host
whose device memory belongs to that host's own allocator. Its scratch is a
static device array. Each case calls it twice in a row (the second call reuses
the array the first one left behind) and checks both results against numpy:
exactly for integer sums and for max / min, and within the reordering bound
for float sums. The results are also compared with the allocating msl_fold.
The tests allocate the input and the one-element result; the entry point does
not.

This file is collected last so that a run stopping at its first failure has
run every other test before it.
"""
import ctypes
import math
import os
import subprocess
import sys
import textwrap

import numpy as np
import pytest

from muesli4_gb300 import workloads as W

pytestmark = pytest.mark.gpu

U = 2.0 ** -24
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def gamma(k):
    return k * U / (1 - k * U)


def noalloc_fold(A, code, op, x_dev, n, dtype):
    res = A.DeviceArray((1,), dtype)
    rc = A.load().msl_fold_noalloc(code, op, x_dev.ptr, n, res.ptr, ctypes.c_void_p(A.stream_handle()))
    A.check(rc, "msl_fold_noalloc")
    A.sync()
    return res.download()[0]


def numpy_fold(op, x):
    if op == "MSL_FOLD_MAX":
        return x.max()
    if op == "MSL_FOLD_MIN":
        return x.min()
    if x.dtype == np.int32:  # two's-complement wrap-around, as the kernels add
        return wrap32(int(x.astype(np.int64).sum()))
    return float(np.sum(x.astype(np.float64)))


def wrap32(s):
    return np.int32((s + (1 << 31)) % (1 << 32) - (1 << 31))


def sum_bound(n, x, sm):
    """|S_gpu - S_exact| <= gamma_d * sum|x|; d = the longest serial chain of
    any thread (at most 1024 elements per thread, or n spread over at least
    one 512-thread CTA per SM) plus the tree depth."""
    d = min(1024, math.ceil(n / (sm * 512))) + 64
    return gamma(d) * float(np.abs(x.astype(np.float64)).sum()) + 1e-30


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
def test_noalloc_fold_matches_numpy_twice(gpu, name, dtype, op, n):
    rng = np.random.default_rng(n)
    if dtype == np.int32:
        x = rng.integers(-(1 << 30), 1 << 30, n, dtype=np.int32)
    else:
        x = rng.uniform(-1, 1, n).astype(dtype)
    d = gpu.DeviceArray.from_host(x)
    code, opc = gpu.DTYPE_OF[np.dtype(dtype)], getattr(gpu, op)
    want = numpy_fold(op, x)
    allocating = gpu.fold(opc, d)
    sm, _, _ = gpu.device_info()
    for _ in range(2):
        got = noalloc_fold(gpu, code, opc, d, n, dtype)
        if op == "MSL_FOLD_SUM" and dtype != np.int32:
            assert abs(float(got) - want) <= sum_bound(n, x, sm)
            assert abs(float(got) - float(allocating)) <= 2 * sum_bound(n, x, sm)
        else:
            assert got == want and got == allocating


def test_noalloc_fold_two_calls_in_a_row_int_exact(gpu):
    x = W.uniform_i32((1 << 20) + 7, 0, 1000, 44)
    d = gpu.DeviceArray.from_host(x)
    want = numpy_fold("MSL_FOLD_SUM", x)
    first = noalloc_fold(gpu, gpu.MSL_I32, gpu.MSL_FOLD_SUM, d, x.size, np.int32)
    second = noalloc_fold(gpu, gpu.MSL_I32, gpu.MSL_FOLD_SUM, d, x.size, np.int32)
    assert first == want and second == want


def masked_index_sum(n, mask=1023):
    """sum of (i & mask) for i < n, wrapped to int32."""
    period = mask + 1
    full, rest = divmod(n, period)
    return wrap32(full * (mask * period // 2) + rest * (rest - 1) // 2)


@pytest.mark.parametrize("n", [(1 << 29) + 5, 1 << 30], ids=["2^29+5", "2^30"])
def test_noalloc_fold_capacity_edge(gpu, n):
    """Inputs large enough that the grid is raised above one wave (to keep
    every thread at <= 1024 elements), up to the largest accepted size. The
    input x[i] = i & 1023 is made on the device (map_index of zeros), so the
    exact int32 sum has a closed form."""
    z = gpu.DeviceArray((n,), np.int32)
    gpu.fill(z, 0)
    gpu.map_index(gpu.MSL_IDX_XOR_MASK, z, z, (1023,))
    want = masked_index_sum(n)
    for _ in range(2):
        assert noalloc_fold(gpu, gpu.MSL_I32, gpu.MSL_FOLD_SUM, z, n, np.int32) == want
    assert noalloc_fold(gpu, gpu.MSL_I32, gpu.MSL_FOLD_MAX, z, n, np.int32) == 1023
    del z


def test_noalloc_fold_rejects_sizes_beyond_its_scratch(gpu):
    d = gpu.DeviceArray((4,), np.float32)
    res = gpu.DeviceArray((1,), np.float32)
    rc = gpu.load().msl_fold_noalloc(gpu.MSL_F32, gpu.MSL_FOLD_SUM, d.ptr, (1 << 30) + 1, res.ptr, None)
    assert rc == gpu.MSL_ERR_SIZE_MISMATCH
    assert b"capacity" in gpu.load().msl_last_error_string()


# A caller of its own: it loads the library, never calls msl_init, allocates
# its input with the CUDA runtime on a stream it creates, and calls the entry
# point before and after cudaDeviceReset (which rebuilds the primary context,
# so the static array then lives at a new address).
FRESH_PROCESS = textwrap.dedent(r"""
    import ctypes, sys
    import numpy as np
    sys.path.insert(0, sys.argv[1])
    from muesli4_gb300 import abi
    L = abi.load()
    rt = ctypes.CDLL("libcudart.so.13")  # the runtime the library already loaded
    vp = ctypes.c_void_p
    for f, a in (("cudaSetDevice", [ctypes.c_int]), ("cudaStreamCreate", [ctypes.POINTER(vp)]),
                 ("cudaStreamDestroy", [vp]), ("cudaMalloc", [ctypes.POINTER(vp), ctypes.c_size_t]),
                 ("cudaFree", [vp]), ("cudaMemcpy", [vp, vp, ctypes.c_size_t, ctypes.c_int]),
                 ("cudaStreamSynchronize", [vp]), ("cudaDeviceReset", [])):
        getattr(rt, f).argtypes = a
        getattr(rt, f).restype = ctypes.c_int

    def ok(rc, what):
        assert rc == 0, (what, rc)

    x = np.random.default_rng(5).integers(-1000, 1000, 3_000_001, dtype=np.int32)
    want = int(x.astype(np.int64).sum())
    for rnd in range(2):
        ok(rt.cudaSetDevice(0), "cudaSetDevice")
        s, d_x, d_r = vp(), vp(), vp()
        ok(rt.cudaStreamCreate(ctypes.byref(s)), "cudaStreamCreate")
        ok(rt.cudaMalloc(ctypes.byref(d_x), x.nbytes), "cudaMalloc")
        ok(rt.cudaMalloc(ctypes.byref(d_r), 4), "cudaMalloc")
        ok(rt.cudaMemcpy(d_x, x.ctypes.data, x.nbytes, 1), "H2D")
        for call in range(2):
            rc = L.msl_fold_noalloc(abi.MSL_I32, abi.MSL_FOLD_SUM, d_x, x.size, d_r, s)
            assert rc == 0, L.msl_last_error_string()
            ok(rt.cudaStreamSynchronize(s), "sync")
            r = np.zeros(1, np.int32)
            ok(rt.cudaMemcpy(r.ctypes.data, d_r, 4, 2), "D2H")
            assert int(r[0]) == want, (rnd, call, int(r[0]), want)
        ok(rt.cudaFree(d_x), "cudaFree")
        ok(rt.cudaFree(d_r), "cudaFree")
        ok(rt.cudaStreamDestroy(s), "cudaStreamDestroy")
        if rnd == 0:
            ok(rt.cudaDeviceReset(), "cudaDeviceReset")
    print("fresh-process noalloc fold ok")
""")


def test_noalloc_fold_without_init_in_a_fresh_process_across_device_reset(gpu):
    r = subprocess.run([sys.executable, "-c", FRESH_PROCESS, ROOT], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "fresh-process noalloc fold ok" in r.stdout
