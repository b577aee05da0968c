"""ctypes binding of libmsl_gb300.so (the C ABI declared in include/msl_gb300.h).

This is how Python callers -- the tests and the benchmark -- reach the GPU
skeletons. It loads the in-tree library and raises if it is missing: there is
no CPU fallback anywhere in the product path.
"""
from __future__ import annotations

import ctypes
import os
import re

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LIB_PATH = os.path.join(HERE, "libmsl_gb300.so")
HEADER = os.path.join(ROOT, "include", "msl_gb300.h")

# Constants of msl_gb300.h (parsed from the header so they cannot drift).
_CONST = {}
with open(HEADER) as _f:
    for _m in re.finditer(r"#define\s+(MSL_[A-Z0-9_]+)\s+\(?(-?\d+)\)?", _f.read()):
        _CONST[_m.group(1)] = int(_m.group(2))
globals().update(_CONST)

NP_DTYPE = {MSL_F32: np.float32, MSL_F64: np.float64, MSL_I32: np.int32, MSL_BF16: np.uint16}  # noqa: F821
DTYPE_OF = {np.dtype(np.float32): MSL_F32, np.dtype(np.float64): MSL_F64,  # noqa: F821
            np.dtype(np.int32): MSL_I32, np.dtype(np.uint16): MSL_BF16}  # noqa: F821


class MslError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"[{code}] {message}")
        self.code = code


def declared_functions() -> list[str]:
    """Names of the functions msl_gb300.h declares."""
    with open(HEADER) as f:
        text = f.read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(msl_\w+)\s*\(", text, flags=re.M)))


_lib = None


def load() -> ctypes.CDLL:
    """Load the in-tree libmsl_gb300.so (raises ImportError if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
    L = ctypes.CDLL(LIB_PATH)
    i, sz, d, vp = ctypes.c_int, ctypes.c_size_t, ctypes.c_double, ctypes.c_void_p
    dp, ip, llp = ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_longlong)
    ll = ctypes.c_longlong
    sig = {
        "msl_init": [i], "msl_terminate": [], "msl_sync": [], "msl_get_stream": [ctypes.POINTER(vp)],
        "msl_set_stream": [vp], "msl_device_info": [ip, ctypes.POINTER(sz), ctypes.POINTER(sz)],
        "msl_launch_count": [ctypes.POINTER(ctypes.c_ulonglong)], "msl_set_tma": [i],
        "msl_set_stencil3d_persistent": [i], "msl_set_stencil3d_depth": [i], "msl_set_stencil3d_zchunk": [i],
        "msl_alloc": [ctypes.POINTER(vp), sz], "msl_free": [vp], "msl_upload": [vp, vp, sz],
        "msl_download": [vp, vp, sz], "msl_copy": [vp, vp, sz], "msl_fill": [i, vp, sz, d],
        "msl_upload_async": [vp, vp, sz, vp], "msl_download_async": [vp, vp, sz, vp],
        "msl_map": [i, i, vp, vp, sz, dp], "msl_zip": [i, i, vp, vp, vp, sz], "msl_zip3": [i, i, vp, vp, vp, vp, sz],
        "msl_map_index": [i, i, vp, vp, i, llp, dp], "msl_zip_index": [i, i, vp, vp, vp, i, llp, dp],
        "msl_fold": [i, i, vp, sz, vp], "msl_fold_absdiff_max": [i, vp, vp, sz, dp],
        "msl_stencil2d": [i, i, vp, vp, i, i, i, d], "msl_stencil2d_iterate": [i, i, vp, vp, i, i, i, d, i, dp, ip],
        "msl_stencil3d": [i, i, vp, vp, i, i, i, i, d],
        "msl_stencil3d_iterate": [i, i, vp, vp, i, i, i, i, d, i, dp, ip],
        "msl_set_temporal_depth": [i], "msl_autotune_stencil2d": [i, i, i, i, i, i, ip, dp],
        "msl_set_tile_rows": [i], "msl_autotune_stencil2d_shape": [i, i, i, i, i, i, ip, ip, dp],
        "msl_autotune_save": [ctypes.c_char_p], "msl_autotune_load": [ctypes.c_char_p],
        "msl_fold_noalloc": [i, i, vp, sz, vp, vp],
        "msl_fold_rows": [i, i, vp, ll, ll, i, vp], "msl_fold_cols": [i, i, vp, ll, ll, vp],
        "msl_zip_rows": [i, i, vp, vp, vp, ll, ll], "msl_rotate_rows": [i, vp, vp, ll, ll, ll],
        "msl_rotate_cols": [i, vp, vp, ll, ll, ll], "msl_set_column": [i, vp, vp, ll, ll, ll],
        "msl_batch_create": [i, i, ip, ip, sz, ctypes.POINTER(vp)], "msl_batch_set_grid": [vp, i, vp],
        "msl_batch_solve": [vp, d, ctypes.c_longlong, i, i],
        "msl_batch_get_grid": [vp, i, vp, ctypes.POINTER(ctypes.c_longlong), dp],
        "msl_batch_info": [vp, ip, ip, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(sz)],
        "msl_batch_destroy": [vp], "msl_batch_reset": [vp],
        "msl_grid_dump_text": [ctypes.c_char_p, i, vp, i, i, i], "msl_grid_load_text": [ctypes.c_char_p, i, vp, i, i, i],
        "msl_batch_checkpoint": [vp, ctypes.c_char_p], "msl_batch_restore": [ctypes.c_char_p, sz, ctypes.POINTER(vp)],
        "msl_server_start": [sz, d, ctypes.c_longlong, i, i, ctypes.POINTER(vp)],
        "msl_server_submit": [vp, i, i, i, i, vp, ctypes.POINTER(ctypes.c_longlong)],
        "msl_server_wait": [vp, ctypes.c_longlong, d],
        "msl_server_result": [vp, ctypes.c_longlong, vp, ctypes.POINTER(ctypes.c_longlong), dp, dp, dp],
        "msl_server_release": [vp, ctypes.c_longlong],
        "msl_server_stats": [vp, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong),
                             ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(sz), ctypes.POINTER(ctypes.c_longlong)],
        "msl_server_stop": [vp], "msl_server_checkpoint": [vp, ctypes.c_char_p, i],
        "msl_server_cancel": [vp, ctypes.c_longlong],
        "msl_set_wait_limit": [ctypes.c_uint], "msl_wait_selftest": [ctypes.c_uint, i],
        "msl_debug_fail_allocs": [ctypes.c_longlong],
        "msl_server_restore": [ctypes.c_char_p, ctypes.POINTER(vp)],
    }
    for name, args in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = ctypes.c_int
    L.msl_last_error_string.argtypes = []
    L.msl_last_error_string.restype = ctypes.c_char_p
    _lib = L
    return L


def check(rc: int, what: str = "") -> None:
    if rc != 0:
        msg = load().msl_last_error_string().decode(errors="replace")
        raise MslError(rc, f"{what}: {msg}" if what else msg)


def init(device: int = 0) -> None:
    check(load().msl_init(device), "msl_init")


def terminate() -> None:
    check(load().msl_terminate(), "msl_terminate")


def sync() -> None:
    check(load().msl_sync(), "msl_sync")


def stream_handle() -> int:
    s = ctypes.c_void_p()
    check(load().msl_get_stream(ctypes.byref(s)), "msl_get_stream")
    return s.value or 0


def launch_count() -> int:
    c = ctypes.c_ulonglong()
    check(load().msl_launch_count(ctypes.byref(c)))
    return c.value


def set_tma(enabled: bool) -> None:
    check(load().msl_set_tma(1 if enabled else 0))


def set_stencil3d_persistent(mode: int) -> None:
    """3-D stencil kernel: 1 persistent, 0 one CTA per block, -1 default."""
    check(load().msl_set_stencil3d_persistent(int(mode)), "msl_set_stencil3d_persistent")


def set_stencil3d_depth(sweeps: int) -> None:
    """heat3D sweeps per launch: 2 the z-marching kernel (default), 1 one sweep."""
    check(load().msl_set_stencil3d_depth(int(sweeps)), "msl_set_stencil3d_depth")


def set_stencil3d_zchunk(planes: int) -> None:
    """z planes per CTA of the z-marching heat3D kernel (0 = chosen per grid)."""
    check(load().msl_set_stencil3d_zchunk(int(planes)), "msl_set_stencil3d_zchunk")


def set_temporal_depth(depth: int) -> None:
    """Sweeps fused per launch by stencil2d_iterate (0 = autotuner's choice)."""
    check(load().msl_set_temporal_depth(int(depth)), "msl_set_temporal_depth")


def autotune_stencil2d(kind: int, dtype: int, rows: int, cols: int, radius: int, iters: int):
    """Returns (best temporal depth, cell updates per second)."""
    d, r = ctypes.c_int(), ctypes.c_double()
    check(load().msl_autotune_stencil2d(dtype, kind, rows, cols, radius, iters, ctypes.byref(d), ctypes.byref(r)),
          "msl_autotune_stencil2d")
    return d.value, r.value


def autotune_stencil2d_shape(kind: int, dtype: int, rows: int, cols: int, radius: int, iters: int):
    """Returns (best temporal depth, best tile rows, cell updates per second)."""
    d, t, r = ctypes.c_int(), ctypes.c_int(), ctypes.c_double()
    check(load().msl_autotune_stencil2d_shape(dtype, kind, rows, cols, radius, iters, ctypes.byref(d), ctypes.byref(t),
                                              ctypes.byref(r)), "msl_autotune_stencil2d_shape")
    return d.value, t.value, r.value


def set_tile_rows(rows: int) -> None:
    """Tile height of the temporal-blocking kernel (16, 32, 64; 0 = autotuned)."""
    check(load().msl_set_tile_rows(int(rows)), "msl_set_tile_rows")


def autotune_save(path: str) -> None:
    check(load().msl_autotune_save(path.encode()), "msl_autotune_save")


def autotune_load(path: str) -> None:
    check(load().msl_autotune_load(path.encode()), "msl_autotune_load")


class Batch:
    """Batched plain-Jacobi solves (msl_batch_*)."""

    def __init__(self, shapes, storage=None, hbm_budget: int = 0):
        self.shapes = [(int(r), int(c)) for r, c in shapes]
        self.storage = MSL_F32 if storage is None else storage  # noqa: F821
        rows = (ctypes.c_int * len(shapes))(*[r for r, _ in self.shapes])
        cols = (ctypes.c_int * len(shapes))(*[c for _, c in self.shapes])
        h = ctypes.c_void_p()
        self.handle = None
        check(load().msl_batch_create(self.storage, len(shapes), rows, cols, hbm_budget, ctypes.byref(h)),
              "msl_batch_create")
        self.handle = h

    def set_grid(self, i: int, grid: np.ndarray) -> None:
        g = np.ascontiguousarray(grid, dtype=np.float32)
        assert g.shape == self.shapes[i]
        check(load().msl_batch_set_grid(self.handle, i, g.ctypes.data), "msl_batch_set_grid")

    def reset(self) -> None:
        check(load().msl_batch_reset(self.handle), "msl_batch_reset")

    def solve(self, tol: float, max_iters: int, check_every: int, depth: int = 0) -> None:
        check(load().msl_batch_solve(self.handle, tol, max_iters, check_every, depth), "msl_batch_solve")

    def get_grid(self, i: int):
        out = np.empty(self.shapes[i], np.float32)
        it, res = ctypes.c_longlong(), ctypes.c_double()
        check(load().msl_batch_get_grid(self.handle, i, out.ctypes.data, ctypes.byref(it), ctypes.byref(res)),
              "msl_batch_get_grid")
        return out, it.value, res.value

    def checkpoint(self, path: str) -> None:
        check(load().msl_batch_checkpoint(self.handle, os.fsencode(path)), "msl_batch_checkpoint")

    @classmethod
    def restore(cls, path: str, hbm_budget: int = 0) -> "Batch":
        """A batch from a checkpoint file; solve() resumes every grid."""
        h = ctypes.c_void_p()
        check(load().msl_batch_restore(os.fsencode(path), hbm_budget, ctypes.byref(h)), "msl_batch_restore")
        with open(path, "rb") as f:
            head = np.frombuffer(f.read(16)[8:], np.int32)
            recs = np.frombuffer(f.read(32 * int(head[1])), np.int32).reshape(-1, 8)
        b = cls.__new__(cls)
        b.shapes = [(int(r), int(c)) for r, c in recs[:, :2]]
        b.storage = int(head[0])
        b.handle = h
        return b

    def info(self):
        n, res, tiles, b = ctypes.c_int(), ctypes.c_int(), ctypes.c_longlong(), ctypes.c_size_t()
        check(load().msl_batch_info(self.handle, ctypes.byref(n), ctypes.byref(res), ctypes.byref(tiles),
                                    ctypes.byref(b)), "msl_batch_info")
        return {"count": n.value, "resident": res.value, "tiles": tiles.value, "device_bytes": b.value}

    def close(self) -> None:
        if self.handle:
            load().msl_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def solve_plain(kind: int, grid: DeviceArray, other: DeviceArray, tol: float, max_iters: int, check_every: int):
    """One grid at a time: msl_stencil2d_iterate (2-D arrays) or
    msl_stencil3d_iterate (3-D arrays, neutral 0) in chunks of check_every
    sweeps until the residual is <= tol. Returns (array holding the result,
    sweeps, residual)."""
    a, b = grid, other
    it, res = 0, float("inf")
    step = stencil3d_iterate if len(grid.shape) == 3 else stencil2d_iterate
    while it < max_iters:
        last, res = step(kind, a, b, 1, 0.0, check_every)
        it += check_every
        if last is b:
            a, b = b, a
        if not res > tol:
            break
    return a, it, res


class Server:
    """Stencil-solve server (msl_server_*): continuous batching of 2-D Jacobi
    and 3-D heat solves."""

    def __init__(self, hbm_budget: int = 0, tol: float = 1e-4, max_iters: int = 5000, check_every: int = 100,
                 depth: int = 0):
        h = ctypes.c_void_p()
        self.handle = None
        check(load().msl_server_start(hbm_budget, tol, max_iters, check_every, depth, ctypes.byref(h)),
              "msl_server_start")
        self.handle = h
        self.shapes = {}

    def submit(self, init: np.ndarray) -> int:
        """A 2-D array is a plain-Jacobi request, a 3-D array a heat3D request."""
        a = np.ascontiguousarray(init, dtype=np.float32)
        rid = ctypes.c_longlong()
        if a.ndim == 2:
            kind, dims = MSL_SERVE_JACOBI2D, (1, a.shape[0], a.shape[1])  # noqa: F821
        else:
            kind, dims = MSL_SERVE_HEAT3D, a.shape  # noqa: F821
        check(load().msl_server_submit(self.handle, kind, dims[0], dims[1], dims[2], a.ctypes.data, ctypes.byref(rid)),
              "msl_server_submit")
        self.shapes[rid.value] = a.shape
        return rid.value

    def wait(self, rid: int, timeout: float = -1.0) -> None:
        check(load().msl_server_wait(self.handle, rid, timeout), "msl_server_wait")

    def result(self, rid: int):
        """(values, sweeps, residual, latency_s, queue_s) of a finished request."""
        out = np.empty(self.shapes[rid], np.float32)
        it, res, lat, q = ctypes.c_longlong(), ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        check(load().msl_server_result(self.handle, rid, out.ctypes.data, ctypes.byref(it), ctypes.byref(res),
                                       ctypes.byref(lat), ctypes.byref(q)), "msl_server_result")
        return out, it.value, res.value, lat.value, q.value

    def cancel(self, rid: int) -> None:
        check(load().msl_server_cancel(self.handle, rid), "msl_server_cancel")

    def release(self, rid: int) -> None:
        check(load().msl_server_release(self.handle, rid), "msl_server_release")
        self.shapes.pop(rid, None)

    def stats(self):
        c, a, q, i = (ctypes.c_longlong() for _ in range(4))
        b = ctypes.c_size_t()
        check(load().msl_server_stats(self.handle, ctypes.byref(c), ctypes.byref(a), ctypes.byref(q), ctypes.byref(b),
                                      ctypes.byref(i)), "msl_server_stats")
        return {"completed": c.value, "active": a.value, "queued": q.value, "device_bytes": b.value,
                "intervals": i.value}

    def checkpoint(self, path: str, halt: bool = False) -> None:
        check(load().msl_server_checkpoint(self.handle, os.fsencode(path), 1 if halt else 0), "msl_server_checkpoint")

    @staticmethod
    def read_checkpoint_records(path: str):
        """(id, kind, state, depth, rows, cols, sweeps, residual) of every request in a checkpoint file."""
        with open(path, "rb") as f:
            head = f.read(56)
            count = int(np.frombuffer(head[48:56], np.int64)[0])
            raw = f.read(48 * count)
        out = []
        for k in range(count):
            rec = raw[48 * k:48 * (k + 1)]
            rid = int(np.frombuffer(rec[:8], np.int64)[0])
            kind, state, depth, rows, cols, _ = (int(v) for v in np.frombuffer(rec[8:32], np.int32))
            it = int(np.frombuffer(rec[32:40], np.int64)[0])
            res = float(np.frombuffer(rec[40:48], np.float64)[0])
            out.append((rid, kind, state, depth, rows, cols, it, res))
        return out

    @classmethod
    def restore(cls, path: str) -> "Server":
        h = ctypes.c_void_p()
        check(load().msl_server_restore(os.fsencode(path), ctypes.byref(h)), "msl_server_restore")
        srv = cls.__new__(cls)
        srv.handle = h
        srv.shapes = {}
        for rid, kind, _, depth, rows, cols, _, _ in cls.read_checkpoint_records(path):
            srv.shapes[rid] = (rows, cols) if kind == MSL_SERVE_JACOBI2D else (depth, rows, cols)  # noqa: F821
        return srv

    def stop(self) -> None:
        if self.handle:
            h, self.handle = self.handle, None
            check(load().msl_server_stop(h), "msl_server_stop")

    def __del__(self):
        try:
            self.stop()
        except Exception:
            pass


def device_info():
    sm, fr, to = ctypes.c_int(), ctypes.c_size_t(), ctypes.c_size_t()
    check(load().msl_device_info(ctypes.byref(sm), ctypes.byref(fr), ctypes.byref(to)))
    return sm.value, fr.value, to.value


class DeviceArray:
    """A device buffer owned through msl_alloc/msl_free, with a numpy shape/dtype."""

    def __init__(self, shape, dtype, ptr: int | None = None):
        self.shape = tuple(int(s) for s in (shape if isinstance(shape, (tuple, list)) else (shape,)))
        self.dtype = np.dtype(dtype)
        self.size = int(np.prod(self.shape)) if self.shape else 1
        self.nbytes = self.size * self.dtype.itemsize
        self._owned = ptr is None
        if ptr is None:
            p = ctypes.c_void_p()
            check(load().msl_alloc(ctypes.byref(p), self.nbytes), "msl_alloc")
            ptr = p.value or 0
        self.ptr = ptr

    @classmethod
    def from_host(cls, a: np.ndarray) -> "DeviceArray":
        a = np.ascontiguousarray(a)
        d = cls(a.shape, a.dtype)
        d.upload(a)
        return d

    def upload(self, a: np.ndarray) -> None:
        a = np.ascontiguousarray(a, dtype=self.dtype)
        assert a.size == self.size
        check(load().msl_upload(self.ptr, a.ctypes.data, self.nbytes), "msl_upload")

    def download(self) -> np.ndarray:
        out = np.empty(self.shape, self.dtype)
        check(load().msl_download(out.ctypes.data, self.ptr, self.nbytes), "msl_download")
        return out

    @property
    def code(self) -> int:
        return DTYPE_OF[self.dtype]

    def free(self) -> None:
        if self._owned and self.ptr:
            L = _lib
            if L is not None:
                L.msl_free(self.ptr)
            self.ptr = 0

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def _params(p):
    if p is None:
        return None
    vals = [float(v) for v in p] + [0.0] * (8 - len(p))
    return (ctypes.c_double * 8)(*vals)


def _dims(shape):
    return (ctypes.c_longlong * 3)(*shape, *([0] * (3 - len(shape))))


# ---- skeleton calls on DeviceArrays -------------------------------------------------
def fill(x: DeviceArray, value: float) -> None:
    check(load().msl_fill(x.code, x.ptr, x.size, float(value)), "msl_fill")


def copy(dst: DeviceArray, src: DeviceArray) -> None:
    check(load().msl_copy(dst.ptr, src.ptr, src.nbytes), "msl_copy")


def map(op: int, x: DeviceArray, out: DeviceArray, params=None) -> None:
    check(load().msl_map(x.code, op, x.ptr, out.ptr, x.size, _params(params)), "msl_map")


def zip(op: int, a: DeviceArray, b: DeviceArray, out: DeviceArray) -> None:
    check(load().msl_zip(a.code, op, a.ptr, b.ptr, out.ptr, a.size), "msl_zip")


def zip3(op: int, a: DeviceArray, b: DeviceArray, c: DeviceArray, out: DeviceArray) -> None:
    check(load().msl_zip3(a.code, op, a.ptr, b.ptr, c.ptr, out.ptr, a.size), "msl_zip3")


def map_index(op: int, x: DeviceArray, out: DeviceArray, params=None) -> None:
    check(load().msl_map_index(x.code, op, x.ptr, out.ptr, len(x.shape), _dims(x.shape), _params(params)),
          "msl_map_index")


def zip_index(op: int, a: DeviceArray, b: DeviceArray, out: DeviceArray, params=None) -> None:
    check(load().msl_zip_index(a.code, op, a.ptr, b.ptr, out.ptr, len(a.shape), _dims(a.shape), _params(params)),
          "msl_zip_index")


def fold(op: int, x: DeviceArray):
    res = np.zeros(1, x.dtype)
    check(load().msl_fold(x.code, op, x.ptr, x.size, res.ctypes.data), "msl_fold")
    return res[0]


def fold_absdiff_max(a: DeviceArray, b: DeviceArray) -> float:
    r = ctypes.c_double()
    check(load().msl_fold_absdiff_max(a.code, a.ptr, b.ptr, a.size, ctypes.byref(r)), "msl_fold_absdiff_max")
    return r.value


def fold_rows(op: int, m: DeviceArray, threads_per_block: int = 1024) -> DeviceArray:
    """Per-row fold of a 2-D array (DM::reduceRows); returns a device vector."""
    rows, cols = m.shape
    out = DeviceArray((rows,), m.dtype)
    check(load().msl_fold_rows(m.code, op, m.ptr, rows, cols, threads_per_block, out.ptr), "msl_fold_rows")
    return out


def fold_cols(op: int, m: DeviceArray) -> DeviceArray:
    rows, cols = m.shape
    out = DeviceArray((cols,), m.dtype)
    check(load().msl_fold_cols(m.code, op, m.ptr, rows, cols, out.ptr), "msl_fold_cols")
    return out


def zip_rows(op: int, m: DeviceArray, v: DeviceArray, out: DeviceArray) -> None:
    rows, cols = m.shape
    check(load().msl_zip_rows(m.code, op, m.ptr, v.ptr, out.ptr, rows, cols), "msl_zip_rows")


def rotate_rows(m: DeviceArray, out: DeviceArray, a: int) -> None:
    rows, cols = m.shape
    check(load().msl_rotate_rows(m.code, m.ptr, out.ptr, rows, cols, int(a)), "msl_rotate_rows")


def rotate_cols(m: DeviceArray, out: DeviceArray, a: int) -> None:
    rows, cols = m.shape
    check(load().msl_rotate_cols(m.code, m.ptr, out.ptr, rows, cols, int(a)), "msl_rotate_cols")


def set_column(m: DeviceArray, v: DeviceArray, col: int) -> None:
    rows, cols = m.shape
    check(load().msl_set_column(m.code, m.ptr, v.ptr, rows, cols, int(col)), "msl_set_column")


def _grid_dims(shape):
    return (1, *shape) if len(shape) == 2 else tuple(shape)


def grid_dump_text(path: str, x: DeviceArray) -> None:
    """Append a 2-D or 3-D device grid to `path` in the `;`-separated text format."""
    d, r, c = _grid_dims(x.shape)
    check(load().msl_grid_dump_text(os.fsencode(path), x.code, x.ptr, d, r, c), "msl_grid_dump_text")


def grid_load_text(path: str, x: DeviceArray) -> None:
    d, r, c = _grid_dims(x.shape)
    check(load().msl_grid_load_text(os.fsencode(path), x.code, x.ptr, d, r, c), "msl_grid_load_text")


def stencil2d(kind: int, x: DeviceArray, out: DeviceArray, radius: int, neutral: float) -> None:
    rows, cols = x.shape
    check(load().msl_stencil2d(x.code, kind, x.ptr, out.ptr, rows, cols, radius, float(neutral)), "msl_stencil2d")


def stencil2d_iterate(kind: int, a: DeviceArray, b: DeviceArray, radius: int, neutral: float, iters: int,
                      residual: bool = True):
    """Ping-pong sweeps; returns (array holding the last sweep, residual or None)."""
    rows, cols = a.shape
    r = ctypes.c_double()
    inb = ctypes.c_int()
    check(load().msl_stencil2d_iterate(a.code, kind, a.ptr, b.ptr, rows, cols, radius, float(neutral), iters,
                                       ctypes.byref(r) if residual else None, ctypes.byref(inb)),
          "msl_stencil2d_iterate")
    return (b if inb.value else a), (r.value if residual else None)


def stencil3d(kind: int, x: DeviceArray, out: DeviceArray, radius: int, neutral: float) -> None:
    d, rows, cols = x.shape
    check(load().msl_stencil3d(x.code, kind, x.ptr, out.ptr, d, rows, cols, radius, float(neutral)), "msl_stencil3d")


def stencil3d_iterate(kind: int, a: DeviceArray, b: DeviceArray, radius: int, neutral: float, iters: int,
                      residual: bool = True):
    d, rows, cols = a.shape
    r = ctypes.c_double()
    inb = ctypes.c_int()
    check(load().msl_stencil3d_iterate(a.code, kind, a.ptr, b.ptr, d, rows, cols, radius, float(neutral), iters,
                                       ctypes.byref(r) if residual else None, ctypes.byref(inb)),
          "msl_stencil3d_iterate")
    return (b if inb.value else a), (r.value if residual else None)
