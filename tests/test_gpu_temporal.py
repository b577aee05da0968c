"""Temporal blocking (several sweeps per launch) and the autotuner.

Fused sweeps must be bit-identical to single sweeps: the oracle runs one sweep
at a time. Shapes include grids smaller than the staged window (every tile is
a boundary tile) and widths TMA cannot address.
"""
import numpy as np
import pytest

from muesli4_gb300 import workloads as W
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture
def depth(gpu):
    yield gpu.set_temporal_depth
    gpu.set_temporal_depth(0)
    gpu.set_tile_rows(0)
    gpu.set_tma(True)


def bits_equal(a, b):
    return a.shape == b.shape and a.dtype == b.dtype and np.array_equal(a.view(np.uint8), b.view(np.uint8))


@pytest.mark.parametrize("d", [2, 3, 4, 8])
@pytest.mark.parametrize("shape", [(3, 5), (33, 47), (64, 64), (130, 200), (257, 1000)], ids=str)
@pytest.mark.parametrize("tma", [True, False], ids=["tma", "plain"])
def test_jacobi_fused_sweeps(gpu, depth, d, shape, tma):
    depth(d)
    gpu.set_tma(tma)
    g = W.jacobi_grid(*shape, seed=d)
    a, b = gpu.DeviceArray.from_host(g), gpu.DeviceArray(g.shape, g.dtype)
    iters = 3 * d + 1  # full fused launches plus a remainder
    last, res = gpu.stencil2d_iterate(gpu.MSL_ST2_JACOBI5, a, b, 1, 0.0, iters)
    want, _, want_res = O.stencil2d_iterate(gpu.MSL_ST2_JACOBI5, g, 1, 0.0, iters)
    assert bits_equal(last.download(), want)
    assert res == want_res


@pytest.mark.parametrize("rows", [16, 64])
@pytest.mark.parametrize("d", [2, 5])
@pytest.mark.parametrize("shape", [(33, 47), (130, 200), (257, 1000)], ids=str)
@pytest.mark.parametrize("dtype", ["f32", "bf16"])
def test_tile_rows_do_not_change_results(gpu, depth, rows, d, shape, dtype):
    """The 64 x 16 (128 threads) and 64 x 64 (512 threads) tiles of the
    temporal-blocking kernel give the one-sweep-at-a-time results."""
    depth(d)
    gpu.set_tile_rows(rows)
    g = W.jacobi_grid(*shape, seed=rows + d)
    if dtype == "bf16":
        g = O.to_bf16(g)
    a, b = gpu.DeviceArray.from_host(g), gpu.DeviceArray(g.shape, g.dtype)
    iters = 3 * d + 1
    last, res = gpu.stencil2d_iterate(gpu.MSL_ST2_JACOBI5, a, b, 1, 0.0, iters)
    want, _, want_res = O.stencil2d_iterate(gpu.MSL_ST2_JACOBI5, g, 1, 0.0, iters)
    assert bits_equal(last.download(), want)
    assert res == want_res
    x = np.random.default_rng(d).random(shape, dtype=np.float32)
    a, b = gpu.DeviceArray.from_host(x), gpu.DeviceArray(x.shape, x.dtype)
    last, res = gpu.stencil2d_iterate(gpu.MSL_ST2_HEAT5, a, b, 1, 0.75, iters)
    want, _, want_res = O.stencil2d_iterate(gpu.MSL_ST2_HEAT5, x, 1, 0.75, iters)
    assert bits_equal(last.download(), want) and res == want_res


def test_tile_rows_setting_is_validated(gpu, depth):
    for bad in (8, 24, 128, -1):
        with pytest.raises(gpu.MslError) as e:
            gpu.set_tile_rows(bad)
        assert e.value.code == gpu.MSL_ERR_INVALID_ARGUMENT


@pytest.mark.parametrize("d", [2, 4, 6])
def test_heat2d_fused_with_neutral(gpu, depth, d):
    depth(d)
    x = np.random.default_rng(d).random((97, 300), dtype=np.float32)
    a, b = gpu.DeviceArray.from_host(x), gpu.DeviceArray(x.shape, x.dtype)
    last, res = gpu.stencil2d_iterate(gpu.MSL_ST2_HEAT5, a, b, 1, 0.75, 2 * d)
    want, _, want_res = O.stencil2d_iterate(gpu.MSL_ST2_HEAT5, x, 1, 0.75, 2 * d)
    assert bits_equal(last.download(), want)
    assert res == want_res


@pytest.mark.parametrize("d", [1, 2, 3, 4, 5, 6, 7, 8, 9, 12, 16, 24, 31, 32])
@pytest.mark.parametrize("shape", [(64, 80), (1000, 1024), (300, 1028), (130, 998), (7, 4), (200, 1925), (129, 961)],
                         ids=str)
def test_life_fused(gpu, depth, d, shape):
    """The first launch runs one generation cell by cell, every later one d
    generations on bit-packed cells; the iteration count leaves a remainder
    launch of 2 generations. Widths around the 960-cell block."""
    depth(d)
    board = W.life_board(*shape, seed=d)
    a, b = gpu.DeviceArray.from_host(board), gpu.DeviceArray(board.shape, np.int32)
    last, _ = gpu.stencil2d_iterate(gpu.MSL_ST2_LIFE, a, b, 1, 0, 4 * d + 3, residual=False)
    assert bits_equal(last.download(), O.stencil2d_iterate(gpu.MSL_ST2_LIFE, board, 1, 0, 4 * d + 3)[0])


def test_bf16_fused(gpu, depth):
    depth(4)
    h = O.to_bf16(W.jacobi_grid(96, 128, 42))
    a, b = gpu.DeviceArray.from_host(h), gpu.DeviceArray(h.shape, np.uint16)
    last, res = gpu.stencil2d_iterate(gpu.MSL_ST2_JACOBI5, a, b, 1, 0.0, 9)
    want, _, want_res = O.stencil2d_iterate(gpu.MSL_ST2_JACOBI5, h, 1, 0.0, 9)
    assert bits_equal(last.download(), want)
    assert res == want_res


@pytest.mark.parametrize("d", [8, 32])
def test_life_fused_with_residual(gpu, depth, d):
    """A residual makes the last launch run its generations cell by cell."""
    depth(d)
    board = W.life_board(100, 200, seed=d)
    a, b = gpu.DeviceArray.from_host(board), gpu.DeviceArray(board.shape, np.int32)
    last, res = gpu.stencil2d_iterate(gpu.MSL_ST2_LIFE, a, b, 1, 0, 2 * d + 5)
    want, _, want_res = O.stencil2d_iterate(gpu.MSL_ST2_LIFE, board, 1, 0, 2 * d + 5)
    assert bits_equal(last.download(), want)
    assert res == want_res


def test_depth_limit(gpu, depth):
    with pytest.raises(gpu.MslError) as e:
        depth(33)
    assert e.value.code == gpu.MSL_ERR_INVALID_ARGUMENT


def test_too_deep_is_an_error(gpu, depth):
    """depth 16 at radius 8 needs a 288-row window: rejected, nothing launched."""
    depth(16)
    x = gpu.DeviceArray((64, 64), np.float32)
    y = gpu.DeviceArray((64, 64), np.float32)
    with pytest.raises(gpu.MslError) as e:
        gpu.stencil2d_iterate(gpu.MSL_ST2_HEAT5, x, y, 8, 0.0, 20)
    assert e.value.code == gpu.MSL_ERR_INVALID_ARGUMENT


def test_autotuner_records_and_is_used(gpu, depth, tmp_path):
    best, rows, rate = gpu.autotune_stencil2d_shape(gpu.MSL_ST2_JACOBI5, gpu.MSL_F32, 1024, 1024, 1, 64)
    assert best in (1, 2, 3, 4, 6, 8, 12, 16, 24, 32) and rows in (16, 32, 64) and rate > 0
    assert best > 1 or rows == 32
    best2, rate2 = gpu.autotune_stencil2d(gpu.MSL_ST2_JACOBI5, gpu.MSL_F32, 1024, 1024, 1, 64)
    assert best2 in (1, 2, 3, 4, 6, 8, 12, 16, 24, 32) and rate2 > 0
    path = str(tmp_path / "tune.txt")
    gpu.autotune_save(path)
    gpu.autotune_load(path)
    depth(0)  # use the record
    g = W.jacobi_grid(1024, 1024, 42)
    a, b = gpu.DeviceArray.from_host(g), gpu.DeviceArray(g.shape, g.dtype)
    last, res = gpu.stencil2d_iterate(gpu.MSL_ST2_JACOBI5, a, b, 1, 0.0, 50)
    want, _, want_res = O.stencil2d_iterate(gpu.MSL_ST2_JACOBI5, g, 1, 0.0, 50)
    assert bits_equal(last.download(), want)
    assert res == want_res
