"""GPU skeletons (through the C ABI) against the CPU oracle on seeded inputs.

Integer, index and stencil results must be bit-exact; FP32 map/zip/stencil
results too (the kernels evaluate the functors one IEEE operation at a time in
the reference's order, as the oracle does). FP32 folds are compared against
an exact sum within the stated reordering bound (see test_fold_f32_sum_bound).
Shapes cover the reference tests' edge cases: empty and one-element inputs,
ragged sizes, odd grid widths that TMA cannot address, radii larger than half
the grid, non-zero neutral values and misaligned buffers.
"""
import math

import numpy as np
import pytest

from muesli4_gb300 import workloads as W
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu

SIZES = [1, 3, 4, 5, 17, 1023, 4099, (1 << 20) + 7]


def dev(A, x):
    return A.DeviceArray.from_host(x)


def bits_equal(a, b):
    a, b = np.ascontiguousarray(a), np.ascontiguousarray(b)
    return a.shape == b.shape and a.dtype == b.dtype and np.array_equal(a.view(np.uint8), b.view(np.uint8))


# ---- map / zip -------------------------------------------------------------------------
@pytest.mark.parametrize("n", SIZES)
@pytest.mark.parametrize("dtype", [np.float32, np.float64, np.int32])
def test_map_affine(gpu, n, dtype):
    rng = np.random.default_rng(n)
    x = (rng.uniform(-1, 1, n) * (1000 if dtype == np.int32 else 1)).astype(dtype)
    p = (2.5, 1.0) if dtype != np.int32 else (3, -7)
    d, o = dev(gpu, x), gpu.DeviceArray(x.shape, x.dtype)
    gpu.map(gpu.MSL_MAP_AFFINE, d, o, p)
    assert bits_equal(o.download(), O.map(gpu.MSL_MAP_AFFINE, x, p))
    gpu.map(gpu.MSL_MAP_AFFINE, d, d, p)  # mapInPlace
    assert bits_equal(d.download(), O.map(gpu.MSL_MAP_AFFINE, x, p))


@pytest.mark.parametrize("op", ["MSL_MAP_ABS", "MSL_MAP_SQUARE"])
def test_map_other_ops(gpu, op):
    x = np.random.default_rng(3).uniform(-5, 5, 10007).astype(np.float32)
    d, o = dev(gpu, x), gpu.DeviceArray(x.shape, x.dtype)
    gpu.map(getattr(gpu, op), d, o)
    assert bits_equal(o.download(), O.map(getattr(gpu, op), x))


@pytest.mark.parametrize("op", ["MSL_ZIP_ADD", "MSL_ZIP_SUB", "MSL_ZIP_MUL", "MSL_ZIP_MULADD", "MSL_ZIP_ABSDIFF",
                                "MSL_ZIP_MAX", "MSL_ZIP_MIN"])
@pytest.mark.parametrize("dtype", [np.float32, np.float64, np.int32])
def test_zip_ops(gpu, op, dtype):
    rng = np.random.default_rng(11)
    n = 70001
    a = (rng.uniform(-1, 1, n) * (1 << 20 if dtype == np.int32 else 1)).astype(dtype)
    b = (rng.uniform(-1, 1, n) * (1 << 20 if dtype == np.int32 else 1)).astype(dtype)
    da, db, o = dev(gpu, a), dev(gpu, b), gpu.DeviceArray(a.shape, a.dtype)
    code = getattr(gpu, op)
    gpu.zip(code, da, db, o)
    assert bits_equal(o.download(), O.zip(code, a, b))


def test_zip_argument_order_is_pinned(gpu):
    """zip(b, c, f) computes f(b[i], c[i]) (the reference GPU build's order);
    a - b is not symmetric, so a swapped order would fail."""
    a = np.arange(1, 101, dtype=np.int32)
    b = np.full(100, 1000, np.int32)
    da, db, o = dev(gpu, a), dev(gpu, b), gpu.DeviceArray(a.shape, a.dtype)
    gpu.zip(gpu.MSL_ZIP_SUB, da, db, o)
    assert np.array_equal(o.download(), a - b)


def test_zip_inplace_and_zip3(gpu):
    rng = np.random.default_rng(5)
    a, b, c = (rng.uniform(-1, 1, 50003).astype(np.float32) for _ in range(3))
    da, db, dc = dev(gpu, a), dev(gpu, b), dev(gpu, c)
    o = gpu.DeviceArray(a.shape, a.dtype)
    for op in (gpu.MSL_ZIP3_MULADD, gpu.MSL_ZIP3_SUM):
        gpu.zip3(op, da, db, dc, o)
        assert bits_equal(o.download(), O.zip3(op, a, b, c))
    gpu.zip(gpu.MSL_ZIP_MULADD, da, db, da)  # zipInPlace
    assert bits_equal(da.download(), O.zip(gpu.MSL_ZIP_MULADD, a, b))


def test_misaligned_buffers_take_the_scalar_path(gpu):
    """Views that start one element into an allocation are not 16-byte aligned."""
    n = 4099
    x = np.random.default_rng(9).uniform(-1, 1, n + 1).astype(np.float32)
    d = dev(gpu, x)
    o = gpu.DeviceArray((n + 1,), np.float32)
    dv = gpu.DeviceArray((n,), np.float32, ptr=d.ptr + 4)
    ov = gpu.DeviceArray((n,), np.float32, ptr=o.ptr + 4)
    gpu.map(gpu.MSL_MAP_AFFINE, dv, ov, (2.5, 1.0))
    assert bits_equal(o.download()[1:], O.map(gpu.MSL_MAP_AFFINE, x[1:].copy(), (2.5, 1.0)))
    assert gpu.fold(gpu.MSL_FOLD_MAX, dv) == O.fold(gpu.MSL_FOLD_MAX, x[1:].copy())


def test_empty_inputs(gpu):
    d = gpu.DeviceArray((0,), np.float32)
    gpu.map(gpu.MSL_MAP_AFFINE, d, d, (1, 1))  # no-op
    with pytest.raises(gpu.MslError) as e:
        gpu.fold(gpu.MSL_FOLD_SUM, d)
    assert e.value.code == gpu.MSL_ERR_INVALID_ARGUMENT


# ---- index skeletons -----------------------------------------------------------------
SHAPES_IDX = [(1,), (7,), (4099,), (1, 1), (1, 9), (9, 1), (37, 53), (300, 257), (1, 1, 1), (5, 7, 11), (17, 3, 129)]


def coeffs(nd, zip_):
    base = {1: (3,), 2: (1000, 7), 3: (7, 1000, 100000)}[nd]
    return base + ((2, -3) if zip_ else (-1,))


@pytest.mark.parametrize("shape", SHAPES_IDX, ids=str)
@pytest.mark.parametrize("dtype", [np.int32, np.float32])
def test_map_index_linear(gpu, shape, dtype):
    x = np.random.default_rng(len(shape)).integers(-500, 500, shape).astype(dtype)
    p = coeffs(len(shape), False)
    d, o = dev(gpu, x), gpu.DeviceArray(x.shape, x.dtype)
    gpu.map_index(gpu.MSL_IDX_LINEAR, d, o, p)
    assert bits_equal(o.download(), O.map_index(gpu.MSL_IDX_LINEAR, x, p))
    gpu.map_index(gpu.MSL_IDX_PRODUCT, d, o)
    assert bits_equal(o.download(), O.map_index(gpu.MSL_IDX_PRODUCT, x))


@pytest.mark.parametrize("shape", SHAPES_IDX, ids=str)
def test_zip_index(gpu, shape):
    rng = np.random.default_rng(77)
    a = rng.integers(-500, 500, shape).astype(np.int32)
    b = rng.integers(-500, 500, shape).astype(np.int32)
    p = coeffs(len(shape), True)
    da, db, o = dev(gpu, a), dev(gpu, b), gpu.DeviceArray(a.shape, a.dtype)
    gpu.zip_index(gpu.MSL_IDX_LINEAR, da, db, o, p)
    assert bits_equal(o.download(), O.zip_index(gpu.MSL_IDX_LINEAR, a, b, p))
    gpu.zip_index(gpu.MSL_IDX_PRODUCT, da, db, da)  # zipIndexInPlace
    assert bits_equal(da.download(), O.zip_index(gpu.MSL_IDX_PRODUCT, a, b))


@pytest.mark.parametrize("shape", [(5,), (6, 9), (4, 5, 6), (64, 48)], ids=str)
def test_map_index_border_init(gpu, shape):
    x = np.random.default_rng(1).random(shape, dtype=np.float32)
    d, o = dev(gpu, x), gpu.DeviceArray(x.shape, x.dtype)
    gpu.map_index(gpu.MSL_IDX_BORDER, d, o, (100.0, 0.0))
    assert bits_equal(o.download(), O.map_index(gpu.MSL_IDX_BORDER, x, (100.0, 0.0)))


def test_map_index_xor(gpu):
    x = W.uniform_i32(1 << 20 | 5, 0, 1000, 44)
    d, o = dev(gpu, x), gpu.DeviceArray(x.shape, x.dtype)
    gpu.map_index(gpu.MSL_IDX_XOR_MASK, d, o, (1023,))
    assert bits_equal(o.download(), O.map_index(gpu.MSL_IDX_XOR_MASK, x, (1023,)))


# ---- folds -------------------------------------------------------------------------------
@pytest.mark.parametrize("n", SIZES + [12345678])
def test_fold_i32_exact(gpu, n):
    x = np.random.default_rng(n).integers(-(1 << 30), 1 << 30, n, dtype=np.int32)
    d = dev(gpu, x)
    assert gpu.fold(gpu.MSL_FOLD_SUM, d) == O.fold(gpu.MSL_FOLD_SUM, x)  # wrap-around sum
    assert gpu.fold(gpu.MSL_FOLD_MAX, d) == x.max()
    assert gpu.fold(gpu.MSL_FOLD_MIN, d) == x.min()


def gamma(k):
    u = 2.0 ** -24
    return k * u / (1 - k * u)


@pytest.mark.parametrize("n", SIZES + [12345678])
def test_fold_f32_sum_bound(gpu, n):
    """|S_gpu - S_exact| <= gamma_d * sum|x|, d = the deepest chain of the
    kernel's summation tree: per-thread serial length (at most n / threads
    plus 20 for the vector, unrolled chains and tail) + the warp, CTA and
    last-CTA trees (< 44 levels), so d = ceil(n / threads) + 64.
    The reference's own sequential fold only meets gamma_{n-1}; both are
    reported against the exact (FP64/fsum) value."""
    x = np.random.default_rng(n).uniform(-1, 1, n).astype(np.float32)
    d = dev(gpu, x)
    got = float(gpu.fold(gpu.MSL_FOLD_SUM, d))
    exact = math.fsum(x.astype(np.float64))
    sm, _, _ = gpu.device_info()
    threads = sm * 512  # the fold runs at least one 512-thread CTA per SM
    depth = math.ceil(n / threads) + 64
    s_abs = float(np.abs(x.astype(np.float64)).sum())
    assert abs(got - exact) <= gamma(depth) * s_abs + 1e-30
    ref_seq = float(O.fold(gpu.MSL_FOLD_SUM, x))
    assert abs(got - ref_seq) <= (gamma(depth) + gamma(n - 1)) * s_abs + 1e-30


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_fold_max_min_exact(gpu, dtype):
    x = np.random.default_rng(4).uniform(-10, -1, 300007).astype(dtype)  # all negative
    d = dev(gpu, x)
    assert gpu.fold(gpu.MSL_FOLD_MAX, d) == x.max()
    assert gpu.fold(gpu.MSL_FOLD_MIN, d) == x.min()


def test_fold_scratch_is_reusable(gpu):
    """Back-to-back folds share the context scratch; the ticket resets itself."""
    for k in range(5):
        x = np.full(100000 + k, k + 1, np.int32)
        assert gpu.fold(gpu.MSL_FOLD_SUM, dev(gpu, x)) == (k + 1) * (100000 + k)


@pytest.mark.parametrize("n", [1, 5, 4099, 1 << 20])
def test_fold_absdiff_max_fp64(gpu, n):
    rng = np.random.default_rng(n)
    a = rng.random(n, dtype=np.float32)
    b = rng.random(n, dtype=np.float32)
    assert gpu.fold_absdiff_max(dev(gpu, a), dev(gpu, b)) == O.fold_absdiff_max(a, b)


def test_copy_is_exact(gpu):
    for nbytes in (1, 15, 16, 4096 + 3, 1 << 22):
        x = np.random.default_rng(nbytes).integers(0, 256, nbytes, dtype=np.uint8)
        src = gpu.DeviceArray((nbytes,), np.uint8)
        dst = gpu.DeviceArray((nbytes,), np.uint8)
        src.upload(x)
        gpu.copy(dst, src)
        assert np.array_equal(dst.download(), x)


def test_fill(gpu):
    for dtype, v in ((np.float32, 2.5), (np.int32, -3), (np.float64, 1e300)):
        d = gpu.DeviceArray((1003,), dtype)
        gpu.fill(d, v)
        assert np.all(d.download() == dtype(v))


# ---- 2-D stencils -------------------------------------------------------------------
SHAPES_2D = [(1, 1), (1, 7), (7, 1), (3, 5), (33, 47), (64, 64), (65, 129), (100, 100), (97, 256), (256, 520)]


@pytest.mark.parametrize("tma", [True, False], ids=["tma", "plain"])
@pytest.mark.parametrize("shape", SHAPES_2D, ids=str)
@pytest.mark.parametrize("kind,neutral", [("MSL_ST2_JACOBI5", 0.0), ("MSL_ST2_HEAT5", 0.75)])
def test_stencil2d_float(gpu, shape, kind, neutral, tma):
    x = np.random.default_rng(shape[0] * 1000 + shape[1]).random(shape, dtype=np.float32)
    gpu.set_tma(tma)
    try:
        d, o = dev(gpu, x), gpu.DeviceArray(x.shape, x.dtype)
        code = getattr(gpu, kind)
        gpu.stencil2d(code, d, o, 1, neutral)
        assert bits_equal(o.download(), O.stencil2d(code, x, 1, neutral))
    finally:
        gpu.set_tma(True)


@pytest.mark.parametrize("tma", [True, False], ids=["tma", "plain"])
@pytest.mark.parametrize("r", [1, 2, 3, 4, 5, 6, 7, 8, 10, 12])
@pytest.mark.parametrize("shape", [(13, 17), (64, 96), (130, 260), (33, 130)], ids=str)
def test_stencil2d_box(gpu, r, shape, tma):
    """Radii 1-4, 6, 8, 10 with neutral +0 run the two-columns-per-thread
    kernel with packed additions; odd widths store column by column."""
    x = W.blur_image(*shape, seed=r)
    d, o = dev(gpu, x), gpu.DeviceArray(x.shape, x.dtype)
    gpu.set_tma(tma)
    try:
        for kind in (gpu.MSL_ST2_BOXMEAN, gpu.MSL_ST2_BOXSUM):
            gpu.stencil2d(kind, d, o, r, 0.0)
            assert bits_equal(o.download(), O.stencil2d(kind, x, r, 0.0)), (kind, r)
    finally:
        gpu.set_tma(True)


@pytest.mark.parametrize("r", [1, 4, 10])
def test_stencil2d_box_special_values(gpu, r):
    """Packed additions round each lane like a scalar addition: infinities,
    subnormals, negative values and a -0 neutral value (which takes the
    one-column kernel) all match the oracle bit for bit."""
    rng = np.random.default_rng(r)
    x = W.blur_image(70, 200, seed=r)
    u = rng.random(x.shape)
    x[u < 0.01] = np.float32(np.inf)
    x[(u >= 0.01) & (u < 0.03)] = np.float32(3e-41)
    x[(u >= 0.03) & (u < 0.2)] *= np.float32(-1.0)
    d, o = dev(gpu, x), gpu.DeviceArray(x.shape, x.dtype)
    for neutral in (0.0, -0.0):
        for kind in (gpu.MSL_ST2_BOXMEAN, gpu.MSL_ST2_BOXSUM):
            gpu.stencil2d(kind, d, o, r, neutral)
            assert bits_equal(o.download(), O.stencil2d(kind, x, r, neutral)), (kind, neutral)


def test_stencil2d_box_neutral_and_f64(gpu):
    x = W.blur_image(70, 90, seed=3)
    d, o = dev(gpu, x), gpu.DeviceArray(x.shape, x.dtype)
    gpu.stencil2d(gpu.MSL_ST2_BOXMEAN, d, o, 4, 255.0)
    assert bits_equal(o.download(), O.stencil2d(gpu.MSL_ST2_BOXMEAN, x, 4, 255.0))
    x64 = x.astype(np.float64)
    d, o = dev(gpu, x64), gpu.DeviceArray(x64.shape, x64.dtype)
    gpu.stencil2d(gpu.MSL_ST2_BOXMEAN, d, o, 3, 0.0)
    assert bits_equal(o.download(), O.stencil2d(gpu.MSL_ST2_BOXMEAN, x64, 3, 0.0))


@pytest.mark.parametrize("shape", [(1, 1), (3, 3), (64, 80), (127, 255), (512, 512)], ids=str)
def test_stencil2d_life(gpu, shape):
    x = W.life_board(*shape, seed=shape[1])
    a, b = dev(gpu, x), gpu.DeviceArray(x.shape, x.dtype)
    last, _ = gpu.stencil2d_iterate(gpu.MSL_ST2_LIFE, a, b, 1, 0, 25, residual=False)
    assert bits_equal(last.download(), O.stencil2d_iterate(gpu.MSL_ST2_LIFE, x, 1, 0, 25)[0])


@pytest.mark.parametrize("iters", [1, 2, 7])
def test_stencil2d_iterate_residual(gpu, iters):
    g = W.jacobi_grid(130, 200, 42)
    a, b = dev(gpu, g), gpu.DeviceArray(g.shape, g.dtype)
    last, res = gpu.stencil2d_iterate(gpu.MSL_ST2_JACOBI5, a, b, 1, 0.0, iters)
    want, _, want_res = O.stencil2d_iterate(gpu.MSL_ST2_JACOBI5, g, 1, 0.0, iters)
    assert bits_equal(last.download(), want)
    assert res == want_res


def test_stencil2d_bf16_storage(gpu):
    g = W.jacobi_grid(96, 128, 42)
    h = O.to_bf16(g)
    a, b = dev(gpu, h), gpu.DeviceArray(h.shape, np.uint16)
    last, res = gpu.stencil2d_iterate(gpu.MSL_ST2_JACOBI5, a, b, 1, 0.0, 5)
    want, _, want_res = O.stencil2d_iterate(gpu.MSL_ST2_JACOBI5, h, 1, 0.0, 5)
    assert bits_equal(last.download(), want)
    assert res == want_res


def test_stencil_argument_errors(gpu):
    x = gpu.DeviceArray((8, 8), np.float32)
    with pytest.raises(gpu.MslError) as e:
        gpu.stencil2d(gpu.MSL_ST2_LIFE, x, gpu.DeviceArray((8, 8), np.float32), 1, 0.0)
    assert e.value.code == gpu.MSL_ERR_INVALID_ARGUMENT
    with pytest.raises(gpu.MslError):
        gpu.stencil2d(gpu.MSL_ST2_HEAT5, x, x, 1, 0.0)  # in == out
    with pytest.raises(gpu.MslError):
        gpu.stencil2d(gpu.MSL_ST2_BOXMEAN, x, gpu.DeviceArray((8, 8), np.float32), 200, 0.0)


# ---- 3-D stencils --------------------------------------------------------------------
SHAPES_3D = [(1, 1, 1), (5, 7, 11), (12, 10, 14), (33, 17, 70), (40, 64, 64), (20, 33, 200)]


@pytest.mark.parametrize("kernel", ["tma", "plain", "persistent"])
@pytest.mark.parametrize("shape", SHAPES_3D, ids=str)
def test_stencil3d_heat(gpu, shape, kernel):
    """heat3D (7-point register path) on the one-CTA-per-block kernel with TMA
    or plain staging loads, and on the persistent double-buffered kernel; a
    non-zero neutral value takes the bounds-tested view on boundary blocks."""
    x = W.heat_cube(*shape, seed=sum(shape))
    gpu.set_tma(kernel != "plain")
    gpu.set_stencil3d_persistent(1 if kernel == "persistent" else 0)
    try:
        for neutral in (0.0, 0.75):
            a, b = dev(gpu, x), gpu.DeviceArray(x.shape, x.dtype)
            last, res = gpu.stencil3d_iterate(gpu.MSL_ST3_HEAT7, a, b, 1, neutral, 3)
            want, _, want_res = O.stencil3d_iterate(gpu.MSL_ST3_HEAT7, x, 1, neutral, 3)
            assert bits_equal(last.download(), want), neutral
            assert res == want_res
    finally:
        gpu.set_tma(True)
        gpu.set_stencil3d_persistent(-1)


@pytest.mark.parametrize("sweeps_per_launch", [2, 1])
@pytest.mark.parametrize("shape", [(1, 1, 4), (5, 7, 11), (33, 17, 70), (40, 64, 64), (70, 20, 36), (65, 33, 200)],
                         ids=str)
def test_stencil3d_heat_z_marching(gpu, shape, sweeps_per_launch):
    """heat3D two sweeps per launch (z-marching kernel) against the oracle for
    1..5 sweeps (odd counts end with a one-sweep launch), with the residual of
    the last sweep; chunk, block and grid edges fall inside the shapes."""
    x = W.heat_cube(*shape, seed=sum(shape) + 1)
    gpu.set_stencil3d_depth(sweeps_per_launch)
    try:
        for iters in range(1, 6):
            a, b = dev(gpu, x), gpu.DeviceArray(x.shape, x.dtype)
            last, res = gpu.stencil3d_iterate(gpu.MSL_ST3_HEAT7, a, b, 1, 0.0, iters)
            want, _, want_res = O.stencil3d_iterate(gpu.MSL_ST3_HEAT7, x, 1, 0.0, iters)
            assert bits_equal(last.download(), want), iters
            assert res == want_res, iters
    finally:
        gpu.set_stencil3d_depth(2)


@pytest.mark.parametrize("depth", [1, 2, 4, 8])
def test_jacobi_negative_zero_block(gpu, depth):
    """A block of -0 cells: a cell whose four neighbours are all -0 sums to +0
    in the reference's order (((0 + W) + E) + N) + S, and its value stays +0
    after the multiplication by 0.25 -- on the one-sweep, temporal-blocking and
    batch paths alike, against the oracle."""
    g = W.jacobi_grid(200, 300, 21)  # too large for a CTA-resident solve: the batch's work-list rounds
    g[40:160, 60:240] = np.float32(-0.0)
    gpu.set_temporal_depth(depth)
    try:
        a, b = dev(gpu, g), gpu.DeviceArray(g.shape, g.dtype)
        last, res = gpu.stencil2d_iterate(gpu.MSL_ST2_JACOBI5, a, b, 1, 0.0, 8)
    finally:
        gpu.set_temporal_depth(0)
    want, _, want_res = O.stencil2d_iterate(gpu.MSL_ST2_JACOBI5, g, 1, 0.0, 8)
    assert bits_equal(last.download(), want)
    assert res == want_res
    batch = gpu.Batch([g.shape])
    try:
        batch.set_grid(0, g)
        batch.solve(tol=0.0, max_iters=8, check_every=8, depth=depth)
        assert bits_equal(batch.get_grid(0)[0], want)
    finally:
        batch.close()


@pytest.mark.parametrize("zchunk", [1, 2, 3, 7, 24, 0])
def test_stencil3d_heat_z_chunks(gpu, zchunk):
    """The z-marching kernel's result does not depend on how the depth is cut
    into per-CTA chunks (1 plane per CTA up to the whole depth; 0 = chosen per
    grid): 4 sweeps with the residual against the oracle."""
    x = W.heat_cube(40, 70, 68, seed=9)
    want, _, want_res = O.stencil3d_iterate(gpu.MSL_ST3_HEAT7, x, 1, 0.0, 4)
    gpu.set_stencil3d_depth(2)
    gpu.set_stencil3d_zchunk(zchunk)
    try:
        a, b = dev(gpu, x), gpu.DeviceArray(x.shape, x.dtype)
        last, res = gpu.stencil3d_iterate(gpu.MSL_ST3_HEAT7, a, b, 1, 0.0, 4)
    finally:
        gpu.set_stencil3d_zchunk(0)
    assert bits_equal(last.download(), want)
    assert res == want_res


@pytest.mark.parametrize("cols", [72, 70])
@pytest.mark.parametrize("sweeps_per_launch", [2, 1])
def test_stencil3d_heat_special_values(gpu, sweeps_per_launch, cols):
    """Sums outside the fast division's range (zero, below 2^-122, subnormal,
    infinite) and negative cells: those cells take IEEE division, the rest of
    the warp the fast path; bit-identical to the oracle either way. Rows of 72
    cells (288 bytes) suit TMA, so two sweeps per launch run the z-marching
    kernel; rows of 70 cells run the plain-load tile kernel."""
    rng = np.random.default_rng(11)
    x = W.heat_cube(40, 64, cols, seed=5)
    u = rng.random(x.shape)
    x[u < 0.01] = np.float32(1e-38)
    x[(u >= 0.01) & (u < 0.02)] = np.float32(3e-40)
    x[(u >= 0.02) & (u < 0.025)] = np.float32(np.inf)
    x[(u >= 0.025) & (u < 0.05)] *= np.float32(-0.3)
    x[8:16, 16:24, 24:32] = 0.0
    # isolated cells in the zero block: a neighbour's sum is the cell alone,
    # just below, at and above the fast division's lower bound 2^-122, and
    # between it and 2^-121 (quotients near 2^-124)
    t = np.float32(2.0 ** -122)
    for k, f in enumerate((1.0, 1.25, 1.4999999, 1.5, 1.5000001, 2.0, 0.999999)):
        x[9 + (k % 3) * 2, 17 + k, 25 + (k % 2) * 3] = np.float32(f) * t * np.float32(1 if k % 2 else -1)
    x[20:28, 30:38, 40:48] = np.float32(-0.0)  # all six neighbours -0: the sum is +0 in the reference's order
    gpu.set_stencil3d_depth(sweeps_per_launch)
    try:
        for iters in (1, 2, 4):
            a, b = dev(gpu, x), gpu.DeviceArray(x.shape, x.dtype)
            last, _ = gpu.stencil3d_iterate(gpu.MSL_ST3_HEAT7, a, b, 1, 0.0, iters, residual=False)
            want = O.stencil3d_iterate(gpu.MSL_ST3_HEAT7, x, 1, 0.0, iters)[0]
            assert bits_equal(last.download(), want), iters
    finally:
        gpu.set_stencil3d_depth(2)


@pytest.mark.parametrize("persistent", [0, 1])
@pytest.mark.parametrize("r", [1, 2, 3])
@pytest.mark.parametrize("shape", [(9, 10, 11), (24, 20, 68)], ids=str)
def test_stencil3d_box(gpu, r, shape, persistent):
    x = W.heat_cube(*shape, seed=r)
    d, o = dev(gpu, x), gpu.DeviceArray(x.shape, x.dtype)
    gpu.set_stencil3d_persistent(persistent)
    try:
        for kind in (gpu.MSL_ST3_BOXSUM, gpu.MSL_ST3_BOXMEAN):
            for neutral in (0.5, 0.0):
                gpu.stencil3d(kind, d, o, r, neutral)
                assert bits_equal(o.download(), O.stencil3d(kind, x, r, neutral)), (kind, r, neutral)
    finally:
        gpu.set_stencil3d_persistent(-1)


def test_async_transfers_round_trip(gpu):
    """msl_upload_async / msl_download_async: stream-ordered copies between
    pinned host memory and the device, on a caller's stream and on the
    library stream (NULL)."""
    import ctypes
    torch = pytest.importorskip("torch")
    x = np.random.default_rng(3).random(1 << 20, dtype=np.float32)
    src = torch.from_numpy(x.copy()).pin_memory()
    dst = torch.empty_like(src).pin_memory()
    d = gpu.DeviceArray((x.size,), np.float32)
    side = torch.cuda.Stream()
    L = gpu.load()
    gpu.check(L.msl_upload_async(d.ptr, ctypes.c_void_p(src.data_ptr()), x.nbytes, ctypes.c_void_p(side.cuda_stream)),
              "msl_upload_async")
    side.synchronize()
    gpu.check(L.msl_download_async(ctypes.c_void_p(dst.data_ptr()), d.ptr, x.nbytes, None), "msl_download_async")
    gpu.sync()
    assert np.array_equal(dst.numpy(), x)
