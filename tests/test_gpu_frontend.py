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
