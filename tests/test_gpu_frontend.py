"""The drop-in C++ front end (DA/DM/DC with user functors) on the GPU.

tests/frontend/frontend_checks.cu is written the way reference programs are
written (Functor subclasses with MSL_USERFUNC operators, MSL_USERFUNC lambdas,
stencil functions as template arguments, the legacy PLMatrix stencil). It is
compiled with nvcc for sm_103a against muesli4_gb300/include and
libmsl_gb300.so, loaded in-process, and checked against the reference tests'
known answers and against the CPU oracle (bit-exact).
"""
import ctypes
import glob
import os
import subprocess

import numpy as np
import pytest

from muesli4_gb300 import workloads as W
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = os.path.join(HERE, "frontend", "frontend_checks.cu")
OUT = os.path.join(HERE, "_build", "libfrontend_checks.so")


def build_checks() -> str:
    deps = [SRC] + glob.glob(os.path.join(ROOT, "muesli4_gb300", "include", "**", "*"), recursive=True)
    deps.append(os.path.join(ROOT, "muesli4_gb300", "libmsl_gb300.so"))
    if os.path.exists(OUT) and os.path.getmtime(OUT) >= max(os.path.getmtime(d) for d in deps if os.path.isfile(d)):
        return OUT
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    cmd = ["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "--extended-lambda",
           "--expt-relaxed-constexpr", "-fmad=false", "-diag-suppress", "177", "-Xcompiler", "-fPIC", "-shared",
           "-I", os.path.join(ROOT, "muesli4_gb300", "include"), "-I", os.path.join(ROOT, "include"),
           "-o", OUT, SRC, "-L", os.path.join(ROOT, "muesli4_gb300"), "-lmsl_gb300",
           "-Xlinker", "-rpath," + os.path.join(ROOT, "muesli4_gb300")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return OUT


@pytest.fixture(scope="module")
def fe(gpu):
    L = ctypes.CDLL(build_checks())
    assert L.fe_init() == 0
    return L


def ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


@pytest.mark.parametrize("dim", [1, 7, 1000, 100003])
def test_da_known_answers(fe, dim):
    assert fe.fe_da_kat(dim) == 0


@pytest.mark.parametrize("shape", [(1, 1), (3, 5), (64, 64), (300, 257)])
def test_dm_known_answers(fe, shape):
    assert fe.fe_dm_kat(*shape) == 0


@pytest.mark.parametrize("shape", [(4, 5, 6), (100, 100, 16), (33, 70, 9)])
def test_dc_known_answers_and_27_point_stencil(fe, shape):
    rows, cols, depth = shape
    assert fe.fe_dc_kat(rows, cols, depth) == 0


@pytest.mark.parametrize("shape,iters", [((48, 64), 10), ((130, 97), 7), ((1024, 1024), 100)])
def test_jacobi_through_mapstencil(fe, shape, iters):
    g = W.jacobi_grid(*shape, seed=42)
    out = np.empty_like(g)
    res = ctypes.c_float()
    assert fe.fe_jacobi(ptr(g), shape[0], shape[1], iters, ptr(out), ctypes.byref(res)) == 0
    want, prev, _ = O.stencil2d_iterate(0, g, 1, 0.0, iters)
    assert np.array_equal(out, want)
    assert res.value == np.max(np.abs(want - prev))


def test_jacobi_matches_reference_golden(fe):
    f = np.load(os.path.join(HERE, "golden", "dm_jacobi_residual.npz"))
    g = f["in0"]
    out = np.empty_like(g)
    res = ctypes.c_float()
    assert fe.fe_jacobi(ptr(g), g.shape[0], g.shape[1], int(f["ints"][2]), ptr(out), ctypes.byref(res)) == 0
    assert np.array_equal(out.ravel(), f["out"])
    assert np.float32(res.value) == f["residual"][0]


@pytest.mark.parametrize("shape", [(12, 10, 14), (64, 64, 64), (19, 33, 70)])
def test_heat3d_through_dc_mapstencil(fe, shape):
    c = W.heat_cube(*shape, seed=3)
    out = np.empty_like(c)
    assert fe.fe_heat3d(ptr(c), *shape, 4, ptr(out)) == 0
    assert np.array_equal(out, O.stencil3d_iterate(0, c, 1, 0.0, 4)[0])


def test_boxsum3d_template_radius(fe):
    c = W.heat_cube(9, 10, 11, seed=57)
    out = np.empty_like(c)
    assert fe.fe_boxsum3d_r2(ptr(c), 9, 10, 11, ptr(out)) == 0
    assert np.array_equal(out, O.stencil3d(1, c, 2, 0.0))


@pytest.mark.parametrize("shape,iters", [((64, 80), 20), ((257, 129), 9)])
def test_life_through_legacy_mapstencilmm(fe, shape, iters):
    b = W.life_board(*shape, seed=5)
    out = np.empty_like(b)
    assert fe.fe_life_mm(ptr(b), shape[0], shape[1], iters, ptr(out)) == 0
    assert np.array_equal(out, O.stencil2d_iterate(4, b, 1, 0, iters)[0])


def nvf_cross_restated(g, r, iters):
    """The WeightedCross stencil of frontend_checks.cu over a matrix whose
    outside cells (row, col) read 3*row - 7*col + 0.25, in float32 with the
    functor's order of operations (power-of-two weights and divisor: exact)."""
    rows, cols = g.shape
    rr, cc = np.meshgrid(np.arange(-r, rows + r), np.arange(-r, cols + r), indexing="ij")
    halo = (np.float32(3) * rr.astype(np.float32) - np.float32(7) * cc.astype(np.float32)
            + np.float32(0.25)).astype(np.float32)
    a = g.astype(np.float32)
    for _ in range(iters):
        p = halo.copy()
        p[r:r + rows, r:r + cols] = a
        s = np.zeros_like(a)
        s = s + p[0:rows, r:r + cols]
        s = s + np.float32(2) * p[2 * r:2 * r + rows, r:r + cols]
        s = s + np.float32(4) * p[r:r + rows, 0:cols]
        s = s + np.float32(8) * p[r:r + rows, 2 * r:2 * r + cols]
        a = (s / np.float32(4 * r)).astype(np.float32)
    return a


@pytest.mark.parametrize("shape,r,iters", [((40, 72), 1, 5), ((97, 33), 2, 4), ((64, 64), 1, 1), ((5, 3), 3, 2)])
def test_mapstencilmm_with_neutral_value_functor(fe, shape, r, iters):
    g = W.uniform_f32(shape[0] * shape[1], 0, 100, 21).reshape(shape)
    out = np.empty_like(g)
    assert fe.fe_stencil_mm_nvf(ptr(g), shape[0], shape[1], r, iters, ptr(out)) == 0
    assert np.array_equal(out, nvf_cross_restated(g, r, iters))


def test_mapzipfold_lambdas(fe):
    n = (1 << 20) + 3
    x = W.uniform_f32(n, -1, 1, 42)
    y = W.uniform_f32(n, -1, 1, 43)
    m, z = np.empty_like(x), np.empty_like(x)
    s = ctypes.c_float()
    assert fe.fe_mapzipfold(ptr(x), ptr(y), n, ptr(m), ptr(z), ctypes.byref(s)) == 0
    want_m = O.map(0, x, (2.5, 1.0))
    want_z = O.zip(3, want_m, y)
    assert np.array_equal(m, want_m)
    assert np.array_equal(z, want_z)
    exact = float(np.sum(want_z, dtype=np.float64))
    u = 2.0 ** -24
    assert abs(s.value - exact) <= 200 * u * float(np.abs(want_z).sum())


def test_dm_and_dc_index_functors_pin_argument_order(fe):
    rng = np.random.default_rng(8)
    a = rng.integers(-500, 500, (37, 53)).astype(np.int32)
    b = rng.integers(-500, 500, (37, 53)).astype(np.int32)
    m, z = np.empty_like(a), np.empty_like(a)
    assert fe.fe_dm_index(ptr(a), ptr(b), 37, 53, ptr(m), ptr(z)) == 0
    assert np.array_equal(m, O.map_index(0, a, (1000, 7, -1)))
    assert np.array_equal(z, O.zip_index(0, a, b, (1000, 7, 2, -3)))
    a3 = rng.integers(-500, 500, (5, 7, 11)).astype(np.int32)
    b3 = rng.integers(-500, 500, (5, 7, 11)).astype(np.int32)
    m3, z3 = np.empty_like(a3), np.empty_like(a3)
    assert fe.fe_dc_index(ptr(a3), ptr(b3), 5, 7, 11, ptr(m3), ptr(z3)) == 0
    assert np.array_equal(m3, O.map_index(0, a3, (7, 1000, 100000, -1)))
    assert np.array_equal(z3, O.zip_index(0, a3, b3, (7, 1000, 100000, 2, -3)))


# ---- row / column skeletons and the DM x DA zips ------------------------------------
GOLDEN = os.path.join(HERE, "golden")


@pytest.mark.parametrize("shape", [(1, 1), (5, 3), (41, 77), (9, 129), (3, 4097), (1000, 7)],
                         ids=lambda s: f"{s[0]}x{s[1]}")
@pytest.mark.parametrize("tpb", [1024, 256, 32, 4])
def test_reduce_rows(fe, shape, tpb):
    rows, cols = shape
    g = np.random.default_rng(rows + cols)
    xi = g.integers(-2**31, 2**31, shape, dtype=np.int64).astype(np.int32)
    out = np.empty(rows, np.int32)
    assert fe.fe_reduce_rows_i32(ptr(xi), rows, cols, tpb, ptr(out)) == 0
    assert np.array_equal(out, O.fold_rows(0, xi, tpb))
    xf = g.uniform(-1, 1, shape).astype(np.float32)
    outf = np.empty(rows, np.float32)
    for op in (0, 1):  # lambda sum, Functor2 max
        assert fe.fe_reduce_rows_f32(ptr(xf), rows, cols, tpb, op, ptr(outf)) == 0
        assert np.array_equal(outf.view(np.uint32), O.fold_rows(op, xf, tpb).view(np.uint32))


def test_reduce_rows_golden(fe):
    for name, fn, dt in (("dm_reduce_rows_sum_i32", fe.fe_reduce_rows_i32, np.int32),
                         ("dm_reduce_rows_sum_i32_wide", fe.fe_reduce_rows_i32, np.int32)):
        f = np.load(os.path.join(GOLDEN, name + ".npz"))
        x = np.ascontiguousarray(f["in0"])
        out = np.empty(x.shape[0], dt)
        assert fn(ptr(x), x.shape[0], x.shape[1], 1024, ptr(out)) == 0
        assert np.array_equal(out, f["out"])
    f = np.load(os.path.join(GOLDEN, "dm_reduce_rows_max_f32.npz"))
    x = np.ascontiguousarray(f["in0"])
    out = np.empty(x.shape[0], np.float32)
    assert fe.fe_reduce_rows_f32(ptr(x), x.shape[0], x.shape[1], 1024, 1, ptr(out)) == 0
    assert np.array_equal(out, f["out"])


def test_reduce_two_columns_golden_and_oracle(fe):
    f = np.load(os.path.join(GOLDEN, "dm_reduce_two_columns.npz"))
    x = np.ascontiguousarray(f["in0"])
    out = np.empty(x.shape[0], np.float32)
    assert fe.fe_reduce_two_columns(ptr(x), x.shape[0], x.shape[1], ptr(out)) == 0
    assert np.array_equal(out.view(np.uint32), f["out"].view(np.uint32))
    big = np.random.default_rng(3).uniform(-1, 1, (5000, 37)).astype(np.float32)
    out = np.empty(5000, np.float32)
    assert fe.fe_reduce_two_columns(ptr(big), 5000, 37, ptr(out)) == 0
    assert np.array_equal(out.view(np.uint32), O.reduce_two_columns_dot(big).view(np.uint32))


@pytest.mark.parametrize("name", ["dm_rotate_rows_p2", "dm_rotate_rows_m3", "dm_rotate_rows_p11", "dm_rotate_rows_p12",
                                  "dm_rotate_cols_p3", "dm_rotate_cols_m5", "dm_rotate_cols_m30", "dm_rotate_cols_p13"])
def test_rotate_golden(fe, name):
    f = np.load(os.path.join(GOLDEN, name + ".npz"))
    x = np.ascontiguousarray(f["in0"])
    rows, cols, a = (int(v) for v in f["ints"])
    out = np.empty_like(x)
    assert fe.fe_rotate(ptr(x), rows, cols, a, 0 if "rows" in name else 1, ptr(out)) == 0
    assert np.array_equal(out, f["out"].reshape(x.shape))


def test_set_column_golden(fe):
    f = np.load(os.path.join(GOLDEN, "dm_set_column.npz"))
    x, v = np.ascontiguousarray(f["in0"]), np.ascontiguousarray(f["in1"])
    rows, cols, col = (int(k) for k in f["ints"])
    out = np.empty_like(x)
    assert fe.fe_set_column(ptr(x), ptr(v), rows, cols, col, ptr(out)) == 0
    assert np.array_equal(out, f["out"].reshape(x.shape))


def _wrap(a):
    return (np.asarray(a, np.int64) & 0xFFFFFFFF).astype(np.uint32).view(np.int32)


BROADCAST_FIXTURES = sorted(os.path.basename(p)[:-4] for pat in ("dm_zipindex_ma_", "dm_zipindex_a_", "dm_zipindex_aaa_",
                                                                   "dm_crosszip_", "da_mapindex_dmrows_",
                                                                   "da_zipindex_dmrows_")
                            for p in glob.glob(os.path.join(HERE, "golden", pat + "*.npz")))
BROADCAST_KIND = {"dm_zipindex_ma": 0, "dm_zipindex_a": 1, "dm_zipindex_aaa": 2, "dm_crosszip": 3,
                  "da_mapindex_dmrows": 4, "da_zipindex_dmrows": 5}


@pytest.mark.parametrize("name", BROADCAST_FIXTURES)
def test_dm_da_broadcast_zips_match_reference_fixtures(fe, name):
    """The front end's broadcast zips against the reference's own outputs
    (same functors as oracle/ref_harness.cpp; crossZipIndexInPlace in the
    GPU build's form, which writes through the matrices' pointers)."""
    f = np.load(os.path.join(HERE, "golden", name + ".npz"))
    rows, cols = (int(v) for v in f["ints"])
    kind = BROADCAST_KIND[name.rsplit("_", 1)[0]]
    a = np.ascontiguousarray(f["in0"].reshape(rows, cols))
    if kind >= 4:
        b = np.zeros_like(a)
        u, v, w = f["in1"].copy(), f["in2"].copy(), np.zeros(rows, np.int32)
        out = np.empty(rows, np.int32)
    else:
        b = np.ascontiguousarray(f["in1"].reshape(rows, cols))
        u, v, w = f["in2"].copy(), f["in3"].copy(), f["in4"].copy()
        out = np.empty((rows, cols), np.int32)
    assert fe.fe_dm_da(kind, ptr(a), ptr(b), ptr(u), ptr(v), ptr(w), rows, cols, ptr(out)) == 0
    assert np.array_equal(out.ravel(), f["out"]), name


@pytest.mark.parametrize("shape", [(1, 1), (7, 5), (64, 64), (33, 1000), (1000, 3)], ids=lambda s: f"{s[0]}x{s[1]}")
def test_dm_da_broadcast_zips(fe, shape):
    rows, cols = shape
    g = np.random.default_rng(rows * 3 + cols)
    a = g.integers(-1000, 1000, shape, dtype=np.int32)
    b = g.integers(-1000, 1000, shape, dtype=np.int32)
    u, v, w = (g.integers(-1000, 1000, rows, dtype=np.int32) for _ in range(3))
    r = np.arange(rows, dtype=np.int64)[:, None]
    c = np.arange(cols, dtype=np.int64)[None, :]
    A, B = a.astype(np.int64), b.astype(np.int64)
    U, V, Wv = (z.astype(np.int64)[:, None] for z in (u, v, w))
    want = {
        0: 1000 * r + 7 * c + 2 * A - 3 * B + 5 * U,
        1: 1000 * r + 7 * c - A + 11 * U,
        2: 1000 * r + 7 * c + A - 2 * U + 3 * V - 5 * Wv,
    }
    out = np.empty(shape, np.int32)
    for kind, exp in want.items():
        assert fe.fe_dm_da(kind, ptr(a), ptr(b), ptr(u), ptr(v), ptr(w), rows, cols, ptr(out)) == 0
        assert np.array_equal(out, _wrap(exp)), kind
    if rows == cols:  # crossZipIndexInPlace: a[r][c] = b[c][r] + a[r][c]
        assert fe.fe_dm_da(3, ptr(a), ptr(b), ptr(u), ptr(v), ptr(w), rows, cols, ptr(out)) == 0
        assert np.array_equal(out, _wrap(B.T + A))
    out1 = np.empty(rows, np.int32)
    assert fe.fe_dm_da(4, ptr(a), ptr(b), ptr(u), ptr(v), ptr(w), rows, cols, ptr(out1)) == 0
    i = np.arange(rows, dtype=np.int64)
    assert np.array_equal(out1, _wrap(i + A.sum(axis=1) - u))
    assert fe.fe_dm_da(5, ptr(a), ptr(b), ptr(u), ptr(v), ptr(w), rows, cols, ptr(out1)) == 0
    assert np.array_equal(out1, _wrap(A[i, i % cols] * v + u + i))
