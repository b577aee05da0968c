"""Row / column skeletons of DM through the C ABI: row folds (reduceRows),
column folds, the matrix x per-row-vector zip, rotateRows, rotateCols and
setColumn, against the CPU oracle (bit-exact) on ragged shapes, and through
size-independent properties on a 1 GiB matrix.

The reference's golden vectors for these skeletons are checked in
tests/test_gpu_golden.py; here the oracle extends them to every lane count
of the row-fold order, every element type and the edge shapes.
"""
import numpy as np
import pytest

from oracle import pyoracle as O

pytestmark = pytest.mark.gpu

SHAPES = [(1, 1), (7, 1), (1, 7), (3, 2), (5, 3), (64, 63), (33, 64), (17, 65), (9, 129), (4, 1000), (3, 4097),
          (1000, 7), (2, 100000), (300, 33)]
TPBS = [1024, 512, 256, 64, 32, 8, 1]


def rand(shape, dtype, seed):
    g = np.random.default_rng(seed)
    if dtype == np.int32:
        return g.integers(-2**31, 2**31, shape, dtype=np.int64).astype(np.int32)
    return g.uniform(-1, 1, shape).astype(dtype)


@pytest.mark.parametrize("shape", SHAPES, ids=lambda s: f"{s[0]}x{s[1]}")
@pytest.mark.parametrize("dtype", [np.float32, np.float64, np.int32])
def test_fold_rows_matches_oracle(gpu, shape, dtype):
    x = rand(shape, dtype, 1 + shape[0] * 7 + shape[1])
    dx = gpu.DeviceArray.from_host(x)
    for op in (gpu.MSL_FOLD_SUM, gpu.MSL_FOLD_MAX, gpu.MSL_FOLD_MIN):
        for tpb in TPBS:
            got = gpu.fold_rows(op, dx, tpb).download()
            want = O.fold_rows(op, x, tpb)
            assert np.array_equal(got.view(np.uint8), want.view(np.uint8)), (op, tpb)


def test_fold_rows_is_element_seeded(gpu):
    x = -np.arange(1, 1 + 5 * 37, dtype=np.float32).reshape(5, 37)
    got = gpu.fold_rows(gpu.MSL_FOLD_MAX, gpu.DeviceArray.from_host(x)).download()
    assert np.array_equal(got, x.max(axis=1))  # a 0 seed would return 0


def test_fold_rows_rejects_bad_arguments(gpu):
    dx = gpu.DeviceArray.from_host(np.ones((4, 4), np.float32))
    with pytest.raises(gpu.MslError) as e:
        gpu.fold_rows(gpu.MSL_FOLD_SUM, dx, 1000)  # not a power of two
    assert e.value.code == gpu.MSL_ERR_INVALID_ARGUMENT
    with pytest.raises(gpu.MslError):
        gpu.fold_rows(gpu.MSL_FOLD_SUM, dx, 2048)
    out = gpu.DeviceArray((4,), np.float32)
    assert gpu.load().msl_fold_rows(gpu.MSL_F32, 0, dx.ptr, 0, 4, 1024, out.ptr) == gpu.MSL_ERR_INVALID_ARGUMENT
    assert gpu.load().msl_fold_rows(gpu.MSL_BF16, 0, dx.ptr, 4, 4, 1024, out.ptr) == gpu.MSL_ERR_INVALID_ARGUMENT


@pytest.mark.parametrize("shape", SHAPES, ids=lambda s: f"{s[0]}x{s[1]}")
@pytest.mark.parametrize("dtype", [np.float32, np.float64, np.int32])
def test_fold_cols_matches_oracle(gpu, shape, dtype):
    x = rand(shape, dtype, 3 + shape[0] + shape[1])
    dx = gpu.DeviceArray.from_host(x)
    for op in (gpu.MSL_FOLD_SUM, gpu.MSL_FOLD_MAX, gpu.MSL_FOLD_MIN):
        got = gpu.fold_cols(op, dx).download()
        assert np.array_equal(got.view(np.uint8), O.fold_cols(op, x).view(np.uint8)), op


@pytest.mark.parametrize("shape", [(1, 1), (5, 3), (64, 63), (9, 129), (3, 4097), (1000, 7)],
                         ids=lambda s: f"{s[0]}x{s[1]}")
@pytest.mark.parametrize("dtype", [np.float32, np.float64, np.int32])
def test_zip_rows_matches_oracle(gpu, shape, dtype):
    m = rand(shape, dtype, 5)
    v = rand((shape[0],), dtype, 6)
    dm, dv = gpu.DeviceArray.from_host(m), gpu.DeviceArray.from_host(v)
    out = gpu.DeviceArray(shape, dtype)
    for op in range(7):  # MSL_ZIP_ADD ... MSL_ZIP_MIN
        gpu.zip_rows(op, dm, dv, out)
        assert np.array_equal(out.download().view(np.uint8), O.zip_rows(op, m, v).view(np.uint8)), op
    gpu.zip_rows(gpu.MSL_ZIP_ADD, dm, dv, dm)  # in place
    assert np.array_equal(dm.download().view(np.uint8), O.zip_rows(gpu.MSL_ZIP_ADD, m, v).view(np.uint8))


ROT_SHAPES = [(1, 1), (2, 3), (11, 13), (64, 64), (5, 1000), (1000, 5), (257, 129)]


@pytest.mark.parametrize("shape", ROT_SHAPES, ids=lambda s: f"{s[0]}x{s[1]}")
@pytest.mark.parametrize("dtype", [np.float32, np.float64, np.int32, np.uint16])
def test_rotations_match_oracle(gpu, shape, dtype):
    rows, cols = shape
    x = np.random.default_rng(rows * 31 + cols).integers(0, 60000, shape).astype(dtype)
    dx = gpu.DeviceArray.from_host(x)
    out = gpu.DeviceArray(shape, dtype)
    for a in sorted({0, 1, -1, 2, -3, rows - 1, -(rows - 1), rows, -rows}):
        if abs(a) > rows:
            continue
        gpu.rotate_rows(dx, out, a)
        assert np.array_equal(out.download(), O.rotate_rows(x, a)), a
    for a in sorted({0, 1, -1, 3, -5, cols, -cols, cols + 2, -(2 * cols + 1), 1000003}):
        gpu.rotate_cols(dx, out, a)
        assert np.array_equal(out.download(), O.rotate_cols(x, a)), a


def test_rotate_rows_more_than_the_rows_is_refused(gpu):
    x = np.arange(12, dtype=np.int32).reshape(3, 4)
    dx, out = gpu.DeviceArray.from_host(x), gpu.DeviceArray((3, 4), np.int32)
    with pytest.raises(gpu.MslError) as e:
        gpu.rotate_rows(dx, out, 4)
    assert e.value.code == gpu.MSL_ERR_NOT_IMPLEMENTED
    with pytest.raises(gpu.MslError) as e:
        gpu.rotate_rows(dx, dx, 1)  # in place is refused: the copy would race
    assert e.value.code == gpu.MSL_ERR_INVALID_ARGUMENT


@pytest.mark.parametrize("dtype", [np.float32, np.float64, np.int32, np.uint16])
def test_set_column_matches_oracle(gpu, dtype):
    for rows, cols in [(1, 1), (17, 9), (1000, 3), (3, 5000)]:
        m = np.random.default_rng(rows).integers(0, 1000, (rows, cols)).astype(dtype)
        v = np.random.default_rng(cols).integers(0, 1000, rows).astype(dtype)
        for col in sorted({0, cols // 2, cols - 1}):
            dm, dv = gpu.DeviceArray.from_host(m), gpu.DeviceArray.from_host(v)
            gpu.set_column(dm, dv, col)
            assert np.array_equal(dm.download(), O.set_column(m, v, col))
    dm, dv = gpu.DeviceArray.from_host(np.zeros((4, 4), dtype)), gpu.DeviceArray.from_host(np.zeros(4, dtype))
    for bad in (-1, 4):
        with pytest.raises(gpu.MslError) as e:
            gpu.set_column(dm, dv, bad)
        assert e.value.code == gpu.MSL_ERR_INVALID_ARGUMENT


def test_full_size_properties(gpu):
    """16384 x 16384 int32 (1 GiB): row sums equal the int64 sums wrapped to
    32 bits (any order gives them), column maxima equal numpy's, and
    rotating by a then by -a (rows and columns) restores every byte."""
    rows = cols = 16384
    x = np.random.default_rng(9).integers(-2**31, 2**31, (rows, cols), dtype=np.int64).astype(np.int32)
    dx = gpu.DeviceArray.from_host(x)
    sums = gpu.fold_rows(gpu.MSL_FOLD_SUM, dx).download()
    want = (x.sum(axis=1, dtype=np.int64) & 0xFFFFFFFF).astype(np.uint32).view(np.int32)
    assert np.array_equal(sums, want)
    assert np.array_equal(gpu.fold_cols(gpu.MSL_FOLD_MAX, dx).download(), x.max(axis=0))
    t = gpu.DeviceArray((rows, cols), np.int32)
    gpu.rotate_rows(dx, t, 4097)
    gpu.rotate_rows(t, dx, -4097)
    gpu.rotate_cols(dx, t, -12345)
    gpu.rotate_cols(t, dx, 12345)
    assert np.array_equal(dx.download(), x)
