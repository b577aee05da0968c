"""Python access to the CPU oracle (liboracle.so) -- TEST INFRASTRUCTURE.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
module, always as the checker or the timed CPU baseline, never as the product
path. The functions mirror the C ABI of include/msl_gb300.h but take and
return numpy arrays.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_HARNESS = os.path.join(HERE, "_ref", "ref_harness")

F32, F64, I32, BF16 = 0, 1, 2, 3
_NP = {F32: np.float32, F64: np.float64, I32: np.int32, BF16: np.uint16}

_lib = None


def build(force: bool = False) -> str:
    """Compile liboracle.so with make (g++ -fopenmp -ffp-contract=off)."""
    if force or not os.path.exists(LIB_PATH):
        subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        vp, sz, i, d = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_double
        dp, llp, ip = ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_int)
        L.oracle_set_threads.argtypes = [i]
        L.oracle_map.argtypes = [i, i, vp, vp, sz, dp]
        L.oracle_zip.argtypes = [i, i, vp, vp, vp, sz]
        L.oracle_zip3.argtypes = [i, i, vp, vp, vp, vp, sz]
        L.oracle_map_index.argtypes = [i, i, vp, vp, i, llp, dp]
        L.oracle_zip_index.argtypes = [i, i, vp, vp, vp, i, llp, dp]
        L.oracle_fold.argtypes = [i, i, vp, sz, vp]
        L.oracle_fold_absdiff_max.argtypes = [i, vp, vp, sz, dp]
        L.oracle_stencil2d.argtypes = [i, i, vp, vp, i, i, i, d]
        L.oracle_stencil2d_iterate.argtypes = [i, i, vp, vp, i, i, i, d, i, dp, ip]
        L.oracle_stencil3d.argtypes = [i, i, vp, vp, i, i, i, i, d]
        L.oracle_stencil3d_iterate.argtypes = [i, i, vp, vp, i, i, i, i, d, i, dp, ip]
        ll = ctypes.c_longlong
        L.oracle_fold_rows.argtypes = [i, i, vp, ll, ll, i, vp]
        L.oracle_fold_cols.argtypes = [i, i, vp, ll, ll, vp]
        L.oracle_zip_rows.argtypes = [i, i, vp, vp, vp, ll, ll]
        L.oracle_rotate_rows.argtypes = [i, vp, vp, ll, ll, ll]
        L.oracle_rotate_cols.argtypes = [i, vp, vp, ll, ll, ll]
        L.oracle_set_column.argtypes = [i, vp, vp, ll, ll, ll]
        L.oracle_dump_text.argtypes = [ctypes.c_char_p, i, vp, i, i, i]
        L.oracle_jacobi_defect_bf16.argtypes = [vp, i, i, d, ll, i, llp, dp]
        _lib = L
    return _lib


def _ptr(a: np.ndarray):
    assert a.flags.c_contiguous
    return a.ctypes.data_as(ctypes.c_void_p)


def _params(p):
    if p is None:
        return None
    arr = (ctypes.c_double * 8)(*([float(v) for v in p] + [0.0] * (8 - len(p))))
    return arr


def _check(rc: int, what: str):
    if rc != 0:
        raise RuntimeError(f"oracle {what} failed with status {rc}")


def dtype_code(a: np.ndarray) -> int:
    return {np.dtype(np.float32): F32, np.dtype(np.float64): F64, np.dtype(np.int32): I32,
            np.dtype(np.uint16): BF16}[a.dtype]


def set_threads(n: int) -> int:
    return lib().oracle_set_threads(n)


def map(op: int, x: np.ndarray, params=None) -> np.ndarray:
    out = np.empty_like(x)
    _check(lib().oracle_map(dtype_code(x), op, _ptr(x), _ptr(out), x.size, _params(params)), "map")
    return out


def zip(op: int, a: np.ndarray, b: np.ndarray) -> np.ndarray:
    out = np.empty_like(a)
    _check(lib().oracle_zip(dtype_code(a), op, _ptr(a), _ptr(b), _ptr(out), a.size), "zip")
    return out


def zip3(op: int, a, b, c) -> np.ndarray:
    out = np.empty_like(a)
    _check(lib().oracle_zip3(dtype_code(a), op, _ptr(a), _ptr(b), _ptr(c), _ptr(out), a.size), "zip3")
    return out


def map_index(op: int, x: np.ndarray, params=None) -> np.ndarray:
    """x.ndim selects DA (1), DM (2: rows, cols) or DC (3: depth, rows, cols)."""
    out = np.empty_like(x)
    dims = (ctypes.c_longlong * 3)(*x.shape, *([0] * (3 - x.ndim)))
    _check(lib().oracle_map_index(dtype_code(x), op, _ptr(x), _ptr(out), x.ndim, dims, _params(params)),
           "map_index")
    return out


def zip_index(op: int, a: np.ndarray, b: np.ndarray, params=None) -> np.ndarray:
    out = np.empty_like(a)
    dims = (ctypes.c_longlong * 3)(*a.shape, *([0] * (3 - a.ndim)))
    _check(lib().oracle_zip_index(dtype_code(a), op, _ptr(a), _ptr(b), _ptr(out), a.ndim, dims,
                                  _params(params)), "zip_index")
    return out


def fold(op: int, x: np.ndarray):
    res = np.zeros(1, dtype=x.dtype)
    _check(lib().oracle_fold(dtype_code(x), op, _ptr(x), x.size, _ptr(res)), "fold")
    return res[0]


def fold_absdiff_max(a: np.ndarray, b: np.ndarray) -> float:
    r = ctypes.c_double()
    _check(lib().oracle_fold_absdiff_max(dtype_code(a), _ptr(a), _ptr(b), a.size, ctypes.byref(r)),
           "fold_absdiff_max")
    return r.value


def stencil2d(kind: int, x: np.ndarray, radius: int, neutral: float) -> np.ndarray:
    out = np.empty_like(x)
    rows, cols = x.shape
    _check(lib().oracle_stencil2d(dtype_code(x), kind, _ptr(x), _ptr(out), rows, cols, radius,
                                  float(neutral)), "stencil2d")
    return out


def stencil2d_iterate(kind: int, x: np.ndarray, radius: int, neutral: float, iters: int):
    """Returns (last sweep, previous sweep, FP64 residual max|last - previous|)."""
    a = x.copy()
    b = np.empty_like(x)
    rows, cols = x.shape
    res = ctypes.c_double()
    inb = ctypes.c_int()
    _check(lib().oracle_stencil2d_iterate(dtype_code(x), kind, _ptr(a), _ptr(b), rows, cols, radius,
                                          float(neutral), iters, ctypes.byref(res), ctypes.byref(inb)),
           "stencil2d_iterate")
    return (b, a, res.value) if inb.value else (a, b, res.value)


def stencil3d(kind: int, x: np.ndarray, radius: int, neutral: float) -> np.ndarray:
    out = np.empty_like(x)
    d, r, c = x.shape
    _check(lib().oracle_stencil3d(dtype_code(x), kind, _ptr(x), _ptr(out), d, r, c, radius, float(neutral)),
           "stencil3d")
    return out


def stencil3d_iterate(kind: int, x: np.ndarray, radius: int, neutral: float, iters: int):
    a = x.copy()
    b = np.empty_like(x)
    d, r, c = x.shape
    res = ctypes.c_double()
    inb = ctypes.c_int()
    _check(lib().oracle_stencil3d_iterate(dtype_code(x), kind, _ptr(a), _ptr(b), d, r, c, radius,
                                          float(neutral), iters, ctypes.byref(res), ctypes.byref(inb)),
           "stencil3d_iterate")
    return (b, a, res.value) if inb.value else (a, b, res.value)


def jacobi_defect_bf16(x: np.ndarray, tol: float, max_iters: int, cycle: int):
    """Plain Jacobi by defect correction with bfloat16 corrections: returns
    (FP32 solution, sweeps, FP64 residual max |J(u) - u|)."""
    u = np.ascontiguousarray(x, dtype=np.float32).copy()
    it, res = ctypes.c_longlong(), ctypes.c_double()
    _check(lib().oracle_jacobi_defect_bf16(_ptr(u), u.shape[0], u.shape[1], float(tol), int(max_iters), int(cycle),
                                           ctypes.byref(it), ctypes.byref(res)), "jacobi_defect_bf16")
    return u, it.value, res.value


# ---- bfloat16 helpers (storage as uint16) -----------------------------------
def to_bf16(x: np.ndarray) -> np.ndarray:
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    nan = (u & 0x7FFFFFFF) > 0x7F800000
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)
    r[nan] = ((u[nan] >> 16) | 0x40).astype(np.uint16)
    return r


def from_bf16(h: np.ndarray) -> np.ndarray:
    return (h.astype(np.uint32) << 16).view(np.float32)


# ---- DM row / column skeletons ------------------------------------------------
def fold_rows(op: int, m: np.ndarray, threads_per_block: int = 1024) -> np.ndarray:
    m = np.ascontiguousarray(m)
    out = np.empty(m.shape[0], m.dtype)
    _check(lib().oracle_fold_rows(dtype_code(m), op, _ptr(m), m.shape[0], m.shape[1], threads_per_block, _ptr(out)),
           "fold_rows")
    return out


def fold_cols(op: int, m: np.ndarray) -> np.ndarray:
    m = np.ascontiguousarray(m)
    out = np.empty(m.shape[1], m.dtype)
    _check(lib().oracle_fold_cols(dtype_code(m), op, _ptr(m), m.shape[0], m.shape[1], _ptr(out)), "fold_cols")
    return out


def zip_rows(op: int, m: np.ndarray, v: np.ndarray) -> np.ndarray:
    m, v = np.ascontiguousarray(m), np.ascontiguousarray(v, dtype=m.dtype)
    out = np.empty_like(m)
    _check(lib().oracle_zip_rows(dtype_code(m), op, _ptr(m), _ptr(v), _ptr(out), m.shape[0], m.shape[1]), "zip_rows")
    return out


def rotate_rows(m: np.ndarray, a: int) -> np.ndarray:
    """Returns the rotated copy; raises on |a| > rows like the reference's exception."""
    m = np.ascontiguousarray(m)
    out = np.empty_like(m)
    _check(lib().oracle_rotate_rows(dtype_code(m), _ptr(m), _ptr(out), m.shape[0], m.shape[1], int(a)), "rotate_rows")
    return out


def rotate_cols(m: np.ndarray, a: int) -> np.ndarray:
    m = np.ascontiguousarray(m)
    out = np.empty_like(m)
    _check(lib().oracle_rotate_cols(dtype_code(m), _ptr(m), _ptr(out), m.shape[0], m.shape[1], int(a)), "rotate_cols")
    return out


def set_column(m: np.ndarray, v: np.ndarray, col: int) -> np.ndarray:
    out = np.array(m, copy=True, order="C")
    v = np.ascontiguousarray(v, dtype=m.dtype)
    _check(lib().oracle_set_column(dtype_code(out), _ptr(out), _ptr(v), out.shape[0], out.shape[1], int(col)),
           "set_column")
    return out


def reduce_two_columns_dot(m: np.ndarray) -> np.ndarray:
    """DM::reducetwoColumns (src/dm.cpp:1729-1752) with f(x, y, s) = s + x*y:
    per row, s = 0, then s = f(row[j], row[(j + 1) % cols], s) for j = 0 ... cols-1,
    one float32 rounding per operation."""
    m = np.ascontiguousarray(m, dtype=np.float32)
    s = np.zeros(m.shape[0], np.float32)
    cols = m.shape[1]
    for j in range(cols):
        s = s + m[:, j] * m[:, (j + 1) % cols]
    return s


def dump_text(path: str, grid: np.ndarray) -> None:
    """Append `grid` (2-D rows x cols or 3-D depth x rows x cols) to `path` in the
    reference examples' `;`-separated text format."""
    g = np.ascontiguousarray(grid)
    d, r, c = (1, *g.shape) if g.ndim == 2 else g.shape
    _check(lib().oracle_dump_text(os.fsencode(path), dtype_code(g), _ptr(g), d, r, c), "dump_text")
