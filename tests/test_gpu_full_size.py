"""The benchmark workloads at their full sizes, checked on the GPU.

DA<float>/DA<int> of 2^28 elements (map, zip, mapIndex, fold), the 8192^2
box-mean radius sweep, 200 Game-of-Life steps on 8192^2, 100 heat3D steps on
512^3 and the 1024^2 plain Jacobi with its residual. Outputs are compared
bit-exactly with numpy restatements of the same IEEE operations or with the
oracle; the box sweep uses an exact sampled check (the oracle would take
minutes at r = 10); float folds use the reordering bound.
"""
import math

import numpy as np
import pytest

from muesli4_gb300 import abi as A
from muesli4_gb300 import workloads as W
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu
N28 = 1 << 28


def f32(v):
    return np.float32(v)


def test_da_float_map_zip_fold_2p28(gpu):
    a = W.uniform_f32(N28, -1.0, 1.0, 42)
    b = W.uniform_f32(N28, -1.0, 1.0, 43)
    da, db = gpu.DeviceArray.from_host(a), gpu.DeviceArray.from_host(b)
    m = gpu.DeviceArray(a.shape, np.float32)
    gpu.map(gpu.MSL_MAP_AFFINE, da, m, (2.5, 1.0))
    want_m = a * f32(2.5) + f32(1.0)  # numpy float32: two roundings
    assert np.array_equal(m.download(), want_m)
    z = gpu.DeviceArray(a.shape, np.float32)
    gpu.zip(gpu.MSL_ZIP_MULADD, m, db, z)
    want_z = want_m * b + want_m
    got_z = z.download()
    assert np.array_equal(got_z, want_z)
    s = float(gpu.fold(gpu.MSL_FOLD_SUM, z))
    exact = float(np.sum(want_z, dtype=np.float64))
    s_abs = float(np.sum(np.abs(want_z), dtype=np.float64))
    sm, _, _ = gpu.device_info()
    d = math.ceil(N28 / (sm * 512)) + 64  # at least one 512-thread CTA per SM
    u = 2.0 ** -24
    assert abs(s - exact) <= d * u / (1 - d * u) * s_abs


def test_da_int_mapindex_fold_2p28(gpu):
    x = W.uniform_i32(N28, 0, 1000, 44)
    dx = gpu.DeviceArray.from_host(x)
    gpu.map_index(gpu.MSL_IDX_XOR_MASK, dx, dx, (1023,))  # mapIndexInPlace
    idx = np.arange(N28, dtype=np.int64)
    want = x ^ (idx & 1023).astype(np.int32)
    del idx
    assert np.array_equal(dx.download(), want)
    got = int(gpu.fold(gpu.MSL_FOLD_SUM, dx))
    exact = int(np.sum(want, dtype=np.int64))
    assert got == ((exact + (1 << 31)) % (1 << 32)) - (1 << 31)  # int32 wrap-around, bit-exact


@pytest.mark.parametrize("r", [1, 2, 4, 6, 8, 10])
def test_box_mean_8192(gpu, r):
    img = W.blur_image(8192, 8192, 42)
    d, o = gpu.DeviceArray.from_host(img), gpu.DeviceArray(img.shape, np.float32)
    gpu.stencil2d(gpu.MSL_ST2_BOXMEAN, d, o, r, 0.0)
    got = o.download()
    rng = np.random.default_rng(r)
    ys = np.concatenate([rng.integers(0, 8192, 4000), [0, 0, 8191, 8191, r, 8191 - r]])
    xs = np.concatenate([rng.integers(0, 8192, 4000), [0, 8191, 0, 8191, 8191 - r, r]])
    acc = np.zeros(ys.size, np.float32)
    for dx in range(-r, r + 1):
        for dy in range(-r, r + 1):
            yy, xx = ys + dy, xs + dx
            inside = (yy >= 0) & (yy < 8192) & (xx >= 0) & (xx < 8192)
            v = np.where(inside, img[np.clip(yy, 0, 8191), np.clip(xx, 0, 8191)], f32(0))
            acc = acc + v
    want = acc / f32((2 * r + 1) ** 2)
    assert np.array_equal(got[ys, xs], want)


@pytest.fixture(scope="module")
def life_8192():
    board = W.life_board(8192, 8192, 42)
    return board, O.stencil2d_iterate(A.MSL_ST2_LIFE, board, 1, 0, 200)[0]


@pytest.mark.parametrize("depth", [0, 8, 32])
def test_life_8192_200_steps(gpu, life_8192, depth):
    """Generations per launch: 0 = the autotuner's record or 1; 8 and 32 run
    the bit-packed kernel after the first generation."""
    board, want = life_8192
    gpu.set_temporal_depth(depth)
    try:
        a, b = gpu.DeviceArray.from_host(board), gpu.DeviceArray(board.shape, np.int32)
        last, _ = gpu.stencil2d_iterate(gpu.MSL_ST2_LIFE, a, b, 1, 0, 200, residual=False)
    finally:
        gpu.set_temporal_depth(0)
    assert np.array_equal(last.download(), want)


@pytest.fixture(scope="module")
def heat512():
    cube = W.heat_cube(512, 512, 512, 42)
    want, _, want_res = O.stencil3d_iterate(A.MSL_ST3_HEAT7, cube, 1, 0.0, 100)
    return cube, want, want_res


@pytest.mark.parametrize("sweeps_per_launch", [2, 1])
def test_heat3d_512_100_steps(gpu, heat512, sweeps_per_launch):
    """Both heat3D paths at full size: two sweeps per launch (the z-marching
    kernel, the default) and one."""
    cube, want, want_res = heat512
    gpu.set_stencil3d_depth(sweeps_per_launch)
    try:
        a, b = gpu.DeviceArray.from_host(cube), gpu.DeviceArray(cube.shape, np.float32)
        last, res = gpu.stencil3d_iterate(gpu.MSL_ST3_HEAT7, a, b, 1, 0.0, 100)
    finally:
        gpu.set_stencil3d_depth(2)
    assert np.array_equal(last.download(), want)
    assert res == want_res


def test_plain_jacobi_1024_100_sweeps(gpu):
    g = W.jacobi_grid(1024, 1024, 42)
    a, b = gpu.DeviceArray.from_host(g), gpu.DeviceArray(g.shape, np.float32)
    last, res = gpu.stencil2d_iterate(gpu.MSL_ST2_JACOBI5, a, b, 1, 0.0, 100)
    want, prev, want_res = O.stencil2d_iterate(gpu.MSL_ST2_JACOBI5, g, 1, 0.0, 100)
    assert np.array_equal(last.download(), want)
    assert res == want_res
    # the reference's float residual: zip(|new-old|) then fold(max)
    assert np.float32(res) == np.max(np.abs(want - prev))
