"""The CPU oracle against golden vectors produced by the Muesli reference itself.

tests/golden/*.npz were generated by tests/golden/make_golden.py, which runs the
reference's own OpenMP skeletons (oracle/_ref/ref_harness). Every comparison is
bit-exact: the oracle restates the reference's loops operation by operation.
"""
import glob
import os

import numpy as np
import pytest

from oracle import pyoracle as O

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
MSL_MAP_AFFINE = 0
MSL_ZIP_MULADD, MSL_ZIP_ABSDIFF, MSL_ZIP_MAX = 3, 4, 5
MSL_IDX_LINEAR, MSL_IDX_XOR_MASK = 0, 2
MSL_FOLD_SUM, MSL_FOLD_MAX = 0, 1
ST2_JACOBI5, ST2_HEAT5, ST2_BOXMEAN, ST2_LIFE = 0, 1, 2, 4
ST3_HEAT7, ST3_BOXSUM = 0, 1

# Coefficients of the non-commutative index functors of oracle/ref_harness.cpp.
DA_IDX = (3, -1)
DA_ZIPIDX = (1, 2, -3)
DM_IDX = (1000, 7, -1)
DM_ZIPIDX = (1000, 7, 2, -3)
DC_IDX = (7, 1000, 100000, -1)
DC_ZIPIDX = (7, 1000, 100000, 2, -3)


def load(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def wrap32(a):
    return (np.asarray(a, np.int64) & 0xFFFFFFFF).astype(np.uint32).view(np.int32)


BROADCAST = ("dm_zipindex_ma_", "dm_zipindex_aaa_", "dm_zipindex_a_", "dm_crosszip_", "da_mapindex_dmrows_",
             "da_zipindex_dmrows_")


def broadcast_restated(name, f):
    """The broadcast-zip fixtures (user functors of oracle/ref_harness.cpp,
    int32) restated with numpy: the skeletons' loops are element-wise, so
    the restatement is the functor applied to whole arrays."""
    rows, cols = (int(v) for v in f["ints"])
    a = f["in0"].astype(np.int64).reshape(rows, cols)
    r = np.arange(rows, dtype=np.int64)[:, None]
    c = np.arange(cols, dtype=np.int64)[None, :]
    if name.startswith("da_"):
        u, v = f["in1"].astype(np.int64), f["in2"].astype(np.int64)
        i = np.arange(rows, dtype=np.int64)
        if name.startswith("da_mapindex_dmrows_"):
            return wrap32(i + a.sum(axis=1) - u)
        return wrap32(a[i, i % cols] * v + u + i)
    b = f["in1"].astype(np.int64).reshape(rows, cols)
    u, v, w = (f[k].astype(np.int64)[:, None] for k in ("in2", "in3", "in4"))
    if name.startswith("dm_zipindex_ma_"):
        return wrap32(1000 * r + 7 * c + 2 * a - 3 * b + 5 * u)
    if name.startswith("dm_zipindex_aaa_"):
        return wrap32(1000 * r + 7 * c + a - 2 * u + 3 * v - 5 * w)
    if name.startswith("dm_zipindex_a_"):
        return wrap32(1000 * r + 7 * c - a + 11 * u)
    return wrap32(b.T + a)  # crossZipIndexInPlace


def oracle_for(name, f):
    """Recompute fixture `name` with the oracle; returns the flat result."""
    if name.startswith(BROADCAST):
        return broadcast_restated(name, f)
    x = f["in0"]
    y = f["in1"] if "in1" in f else None
    ints = [int(v) for v in f["ints"]]
    if name in ("da_map_affine", "da_map_inplace_affine"):
        return O.map(MSL_MAP_AFFINE, x, (2.5, 1.0))
    if name in ("da_zip_muladd", "da_zip_inplace_muladd"):
        return O.zip(MSL_ZIP_MULADD, x, y)
    if name == "da_fold_sum_f32":
        return np.array([O.fold(MSL_FOLD_SUM, x)])
    if name == "da_fold_max_f32":
        return np.array([O.fold(MSL_FOLD_MAX, x)])
    if name.startswith("da_fold_sum_i32"):
        return np.array([O.fold(MSL_FOLD_SUM, x)])
    if name == "da_mapindex_xor":
        return O.map_index(MSL_IDX_XOR_MASK, x, (1023,))
    if name == "da_mapindex_inplace":
        return O.map_index(MSL_IDX_LINEAR, x, DA_IDX)
    if name.startswith("da_zipindex"):
        return O.zip_index(MSL_IDX_LINEAR, x, y, DA_ZIPIDX)
    if name.startswith("dm_mapindex"):
        return O.map_index(MSL_IDX_LINEAR, x, DM_IDX)
    if name.startswith("dm_zipindex"):
        return O.zip_index(MSL_IDX_LINEAR, x, y, DM_ZIPIDX)
    if name.startswith("dc_mapindex"):
        return O.map_index(MSL_IDX_LINEAR, x, DC_IDX)
    if name.startswith("dc_zipindex"):
        return O.zip_index(MSL_IDX_LINEAR, x, y, DC_ZIPIDX)
    if name == "dm_jacobi5":
        return O.stencil2d_iterate(ST2_JACOBI5, x, 1, 0.0, ints[2])[0]
    if name == "dm_heat2d":
        return O.stencil2d_iterate(ST2_HEAT5, x, 1, ints[3] / 1000.0, ints[2])[0]
    if name == "dm_life8":
        return O.stencil2d_iterate(ST2_LIFE, x, 1, 0, ints[2])[0]
    if name.startswith("dm_boxmean"):
        return O.stencil2d_iterate(ST2_BOXMEAN, x, ints[2], 0.0, ints[3])[0]
    if name.startswith("dc_heat3d"):
        return O.stencil3d_iterate(ST3_HEAT7, x, 1, 0.0, ints[3])[0]
    if name.startswith("dc_boxsum"):
        return O.stencil3d_iterate(ST3_BOXSUM, x, ints[3], 0.0, ints[4])[0]
    if name.startswith("dm_reduce_rows_sum_i32"):
        return O.fold_rows(MSL_FOLD_SUM, x)
    if name == "dm_reduce_rows_max_f32":
        return O.fold_rows(MSL_FOLD_MAX, x)
    if name == "dm_reduce_two_columns":
        return O.reduce_two_columns_dot(x)
    if name.startswith("dm_rotate_rows"):
        if abs(ints[2]) > ints[0]:  # the reference refuses and leaves the matrix as it is
            with pytest.raises(RuntimeError):
                O.rotate_rows(x, ints[2])
            return x
        return O.rotate_rows(x, ints[2])
    if name.startswith("dm_rotate_cols"):
        return O.rotate_cols(x, ints[2])
    if name == "dm_set_column":
        return O.set_column(x, y, ints[2])
    raise KeyError(name)


CASES = sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))
CASES = [c for c in CASES if c != "dm_jacobi_residual"]


def test_fixtures_present():
    assert len(CASES) >= 30


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference(name):
    f = load(name)
    got = np.asarray(oracle_for(name, f)).ravel()
    want = f["out"].ravel()
    assert got.dtype == want.dtype
    assert np.array_equal(got.view(np.uint8), want.view(np.uint8)), name


def test_oracle_jacobi_residual_matches_reference():
    """100 Jacobi sweeps, then the reference's zip(|a-b|) + fold(max) in FP32;
    the oracle's FP64 residual rounds to the same float."""
    f = load("dm_jacobi_residual")
    last, prev, res64 = O.stencil2d_iterate(ST2_JACOBI5, f["in0"], 1, 0.0, 100)
    assert np.array_equal(last.ravel(), f["out"])
    assert np.float32(res64) == f["residual"][0]
    d = O.zip(MSL_ZIP_ABSDIFF, last.ravel(), prev.ravel())
    assert O.fold(MSL_FOLD_MAX, d) == f["residual"][0]


def test_oracle_fold_is_seeded_with_first_element():
    # max over all-negative values: a fold seeded with 0 would return 0.
    x = -np.arange(1, 11, dtype=np.float32)
    assert O.fold(MSL_FOLD_MAX, x) == np.float32(-1)
    with pytest.raises(RuntimeError):
        O.fold(MSL_FOLD_SUM, np.zeros(0, np.float32))


def test_oracle_planted_mistake_is_caught():
    """A wrong oracle result must fail the bit-exact comparison."""
    f = load("dm_heat2d")
    got = oracle_for("dm_heat2d", f).ravel().copy()
    got[7] = np.nextafter(got[7], np.float32(np.inf))
    assert not np.array_equal(got, f["out"].ravel())


@pytest.mark.skipif(not os.path.exists(O.REF_HARNESS), reason="reference harness not built here")
def test_golden_regenerates_identically(tmp_path):
    """Re-running the reference on a fixture's inputs reproduces its bytes."""
    import subprocess
    f = load("dm_life8")
    p = tmp_path / "in.bin"
    f["in0"].tofile(p)
    out = tmp_path / "out.bin"
    subprocess.run([O.REF_HARNESS, "dm_life8", *map(str, f["ints"]), "--", str(p), "--", str(out)],
                   check=True, stdout=subprocess.DEVNULL)
    assert np.array_equal(np.fromfile(out, np.int32), f["out"])
