"""GPU skeletons against the golden vectors produced by the Muesli reference.

Same fixtures as tests/test_oracle_golden.py, computed here through the C ABI
on the GPU. Every comparison is bit-exact.
"""
import glob
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
# The DM x DA broadcast-zip fixtures use user functors: the C++ front end
# checks them (tests/test_gpu_frontend.py); the C ABI has no such functors.
BROADCAST = ("dm_zipindex_ma_", "dm_zipindex_a_", "dm_zipindex_aaa_", "dm_crosszip_", "da_mapindex_dmrows_",
             "da_zipindex_dmrows_")
CASES = sorted(n for n in (os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))
               if not n.startswith(BROADCAST))

DA_IDX, DA_ZIPIDX = (3, -1), (1, 2, -3)
DM_IDX, DM_ZIPIDX = (1000, 7, -1), (1000, 7, 2, -3)
DC_IDX, DC_ZIPIDX = (7, 1000, 100000, -1), (7, 1000, 100000, 2, -3)


def run_on_gpu(A, name, f):
    x = f["in0"]
    y = f["in1"] if "in1" in f else None
    ints = [int(v) for v in f["ints"]]
    dx = A.DeviceArray.from_host(x)
    dy = A.DeviceArray.from_host(y) if y is not None else None
    out = A.DeviceArray(x.shape, x.dtype)
    inplace = "inplace" in name
    tgt = dx if inplace else out
    if name in ("da_map_affine", "da_map_inplace_affine"):
        A.map(A.MSL_MAP_AFFINE, dx, tgt, (2.5, 1.0))
    elif name in ("da_zip_muladd", "da_zip_inplace_muladd"):
        A.zip(A.MSL_ZIP_MULADD, dx, dy, tgt)
    elif name == "da_fold_sum_f32" or name.startswith("da_fold_sum_i32"):
        return np.array([A.fold(A.MSL_FOLD_SUM, dx)])
    elif name == "da_fold_max_f32":
        return np.array([A.fold(A.MSL_FOLD_MAX, dx)])
    elif name == "da_mapindex_xor":
        A.map_index(A.MSL_IDX_XOR_MASK, dx, tgt, (1023,))
    elif name == "da_mapindex_inplace":
        A.map_index(A.MSL_IDX_LINEAR, dx, tgt, DA_IDX)
    elif name.startswith("da_zipindex"):
        A.zip_index(A.MSL_IDX_LINEAR, dx, dy, tgt, DA_ZIPIDX)
    elif name.startswith("dm_mapindex"):
        A.map_index(A.MSL_IDX_LINEAR, dx, tgt, DM_IDX)
    elif name.startswith("dm_zipindex"):
        A.zip_index(A.MSL_IDX_LINEAR, dx, dy, tgt, DM_ZIPIDX)
    elif name.startswith("dc_mapindex"):
        A.map_index(A.MSL_IDX_LINEAR, dx, tgt, DC_IDX)
    elif name.startswith("dc_zipindex"):
        A.zip_index(A.MSL_IDX_LINEAR, dx, dy, tgt, DC_ZIPIDX)
    elif name == "dm_jacobi5":
        return A.stencil2d_iterate(A.MSL_ST2_JACOBI5, dx, out, 1, 0.0, ints[2], residual=False)[0].download()
    elif name == "dm_jacobi_residual":
        last, res = A.stencil2d_iterate(A.MSL_ST2_JACOBI5, dx, out, 1, 0.0, ints[2])
        return np.concatenate([last.download().ravel(), np.array([res], np.float32)])
    elif name == "dm_heat2d":
        return A.stencil2d_iterate(A.MSL_ST2_HEAT5, dx, out, 1, ints[3] / 1000.0, ints[2], residual=False)[0].download()
    elif name == "dm_life8":
        return A.stencil2d_iterate(A.MSL_ST2_LIFE, dx, out, 1, 0, ints[2], residual=False)[0].download()
    elif name.startswith("dm_boxmean"):
        return A.stencil2d_iterate(A.MSL_ST2_BOXMEAN, dx, out, ints[2], 0.0, ints[3], residual=False)[0].download()
    elif name.startswith("dc_heat3d"):
        return A.stencil3d_iterate(A.MSL_ST3_HEAT7, dx, out, 1, 0.0, ints[3], residual=False)[0].download()
    elif name.startswith("dc_boxsum"):
        return A.stencil3d_iterate(A.MSL_ST3_BOXSUM, dx, out, ints[3], 0.0, ints[4], residual=False)[0].download()
    elif name.startswith("dm_reduce_rows_sum_i32"):
        return A.fold_rows(A.MSL_FOLD_SUM, dx).download()
    elif name == "dm_reduce_rows_max_f32":
        return A.fold_rows(A.MSL_FOLD_MAX, dx).download()
    elif name == "dm_reduce_two_columns":
        pytest.skip("user-functor skeleton: checked through the C++ front end")
    elif name.startswith("dm_rotate_rows"):
        if abs(ints[2]) > ints[0]:  # the reference refuses and leaves the matrix as it is
            with pytest.raises(A.MslError) as e:
                A.rotate_rows(dx, out, ints[2])
            assert e.value.code == A.MSL_ERR_NOT_IMPLEMENTED
            return dx.download()
        A.rotate_rows(dx, out, ints[2])
    elif name.startswith("dm_rotate_cols"):
        A.rotate_cols(dx, out, ints[2])
    elif name == "dm_set_column":
        A.set_column(dx, dy, ints[2])
        return dx.download()
    else:
        raise KeyError(name)
    return tgt.download()


@pytest.mark.parametrize("tma", [True, False], ids=["tma", "plain-loads"])
@pytest.mark.parametrize("name", CASES)
def test_gpu_matches_reference_golden(gpu, name, tma):
    stencil = (name.startswith("dm_") or name.startswith("dc_")) and "index" not in name and not any(
        name.startswith(p) for p in ("dm_reduce", "dm_rotate", "dm_set_column"))
    if not tma and not stencil:
        pytest.skip("loader switch only affects stencils")
    f = np.load(os.path.join(GOLDEN, name + ".npz"))
    gpu.set_tma(tma)
    try:
        got = np.asarray(run_on_gpu(gpu, name, f)).ravel()
    finally:
        gpu.set_tma(True)
    want = f["out"].ravel()
    if name == "dm_jacobi_residual":
        want = np.concatenate([want, f["residual"]])
    assert got.dtype == want.dtype
    if name == "da_fold_sum_f32":
        # The reference folds left to right; the GPU folds a tree. Both are
        # within their error bound of the exact sum, so they differ by at most
        # (gamma_{n-1} + gamma_d) * sum|x| with d the GPU tree depth (< 100 here).
        x = f["in0"].astype(np.float64)
        u = 2.0 ** -24
        n, d = x.size, 100
        bound = ((n - 1) * u / (1 - (n - 1) * u) + d * u / (1 - d * u)) * np.abs(x).sum()
        assert abs(float(got[0]) - float(want[0])) <= bound
        assert abs(float(got[0]) - x.sum()) <= d * u / (1 - d * u) * np.abs(x).sum()
        return
    assert np.array_equal(got.view(np.uint8), want.view(np.uint8)), name
