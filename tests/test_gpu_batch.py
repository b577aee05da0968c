"""Batched plain-Jacobi solves (msl_batch_*) against the one-grid-at-a-time path.

Every grid in a batch must come out bit-identical to msl_stencil2d_iterate run
on that grid alone with the same residual checks (same sweep count, same FP64
residual): its result does not depend on the other grids in the batch. Shapes
mix CTA-resident grids and work-list grids; FP32 and bfloat16 storage.
"""
import numpy as np
import pytest

from muesli4_gb300 import workloads as W
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu

SHAPES = [(64, 64), (96, 128), (150, 160), (33, 200), (200, 300), (257, 333), (512, 512), (64, 1000)]


def plain(gpu, g, storage, tol, max_iters, check_every):
    if storage == "bf16":
        h = O.to_bf16(g)
        a, b = gpu.DeviceArray.from_host(h), gpu.DeviceArray(h.shape, np.uint16)
        out, it, res = gpu.solve_plain(gpu.MSL_ST2_JACOBI5, a, b, tol, max_iters, check_every)
        return O.from_bf16(out.download()), it, res
    a, b = gpu.DeviceArray.from_host(g), gpu.DeviceArray(g.shape, np.float32)
    out, it, res = gpu.solve_plain(gpu.MSL_ST2_JACOBI5, a, b, tol, max_iters, check_every)
    return out.download(), it, res


@pytest.mark.parametrize("storage", ["f32", "bf16"])
@pytest.mark.parametrize("depth", [1, 2, 5])
def test_batch_equals_plain_path(gpu, storage, depth):
    tol, max_iters, check_every = 2e-3, 3000, 50
    grids = [W.jacobi_grid(r, c, 7000 + i) for i, (r, c) in enumerate(SHAPES)]
    st = gpu.MSL_F32 if storage == "f32" else gpu.MSL_BF16
    batch = gpu.Batch(SHAPES, storage=st)
    info = batch.info()
    assert 0 < info["resident"] < len(SHAPES)  # both solver paths are exercised
    for i, g in enumerate(grids):
        batch.set_grid(i, g)
    batch.solve(tol, max_iters, check_every, depth)
    for i, g in enumerate(grids):
        got, it, res = batch.get_grid(i)
        want, want_it, want_res = plain(gpu, g, storage, tol, max_iters, check_every)
        assert it == want_it, (SHAPES[i], it, want_it)
        assert res == want_res, (SHAPES[i], res, want_res)
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), SHAPES[i]
    batch.close()


def test_batch_grid_alone_equals_in_the_mix(gpu):
    tol, max_iters, check_every = 1e-3, 2000, 100
    shapes = SHAPES[:5]
    grids = [W.jacobi_grid(r, c, 11 + i) for i, (r, c) in enumerate(shapes)]
    mix = gpu.Batch(shapes)
    for i, g in enumerate(grids):
        mix.set_grid(i, g)
    mix.solve(tol, max_iters, check_every, 2)
    for i, g in enumerate(grids):
        alone = gpu.Batch([shapes[i]])
        alone.set_grid(0, g)
        alone.solve(tol, max_iters, check_every, 2)
        a, ia, ra = alone.get_grid(0)
        m, im, rm = mix.get_grid(i)
        assert (ia, ra) == (im, rm) and np.array_equal(a, m)
        alone.close()
    mix.close()


def test_batch_matches_oracle_small(gpu):
    """A short batched solve against the CPU oracle sweep by sweep."""
    shapes = [(48, 64), (300, 260)]
    grids = [W.jacobi_grid(r, c, 3 + i) for i, (r, c) in enumerate(shapes)]
    batch = gpu.Batch(shapes)
    for i, g in enumerate(grids):
        batch.set_grid(i, g)
    batch.solve(0.0, 120, 40, 4)  # tol 0: runs all 120 sweeps
    for i, g in enumerate(grids):
        got, it, res = batch.get_grid(i)
        want, _, want_res = O.stencil2d_iterate(0, g, 1, 0.0, 120)
        assert it == 120 and res == want_res
        assert np.array_equal(got, want)


def test_batch_budget_and_arguments(gpu):
    with pytest.raises(gpu.MslError) as e:
        gpu.Batch([(1024, 1024)], hbm_budget=1 << 20)
    assert e.value.code == gpu.MSL_ERR_BUDGET
    b = gpu.Batch([(64, 64)])
    with pytest.raises(gpu.MslError):
        b.solve(1e-4, 1000, 300)  # check_every must divide max_iters
    b.close()


def test_batch_reset_restores_initial_values(gpu):
    shapes = [(64, 64), (300, 260)]
    grids = [W.jacobi_grid(r, c, 5 + i) for i, (r, c) in enumerate(shapes)]
    b = gpu.Batch(shapes)
    for i, g in enumerate(grids):
        b.set_grid(i, g)
    b.solve(1e-3, 1000, 50, 2)
    first = [b.get_grid(i) for i in range(2)]
    b.reset()
    for i, g in enumerate(grids):
        assert np.array_equal(b.get_grid(i)[0], g)
    b.solve(1e-3, 1000, 50, 2)
    for i in range(2):
        again = b.get_grid(i)
        assert again[1:] == first[i][1:] and np.array_equal(again[0], first[i][0])
    b.close()


DC_SHAPES = [(48, 64), (64, 64), (33, 200), (150, 200), (257, 333), (96, 700)]


@pytest.mark.parametrize("depth", [1, 3, 4])
def test_defect_correction_batch_matches_oracle(gpu, depth):
    """MSL_BF16_DC (FP32 solution, bfloat16 corrections) against the CPU
    restatement of the same defect correction: solution bits, sweep count
    and FP64 residual, for CTA-resident and work-list grids, at several
    temporal depths of the correction sweeps (which change nothing)."""
    tol, max_iters, cycle = 1e-3, 2000, 20
    grids = [W.jacobi_grid(r, c, 900 + i) for i, (r, c) in enumerate(DC_SHAPES)]
    batch = gpu.Batch(DC_SHAPES, storage=gpu.MSL_BF16_DC)
    info = batch.info()
    assert 0 < info["resident"] < len(DC_SHAPES)
    for i, g in enumerate(grids):
        batch.set_grid(i, g)
    batch.solve(tol, max_iters, cycle, depth)
    for i, g in enumerate(grids):
        got, it, res = batch.get_grid(i)
        want, want_it, want_res = O.jacobi_defect_bf16(g, tol, max_iters, cycle)
        assert (it, res) == (want_it, want_res), (DC_SHAPES[i], it, want_it, res, want_res)
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), DC_SHAPES[i]
    batch.close()


def test_defect_correction_alone_equals_in_the_mix(gpu):
    tol, max_iters, cycle = 1e-3, 2000, 16
    shapes = DC_SHAPES[2:]
    grids = [W.jacobi_grid(r, c, 40 + i) for i, (r, c) in enumerate(shapes)]
    mix = gpu.Batch(shapes, storage=gpu.MSL_BF16_DC)
    for i, g in enumerate(grids):
        mix.set_grid(i, g)
    mix.solve(tol, max_iters, cycle, 4)
    for i, g in enumerate(grids):
        alone = gpu.Batch([shapes[i]], storage=gpu.MSL_BF16_DC)
        alone.set_grid(0, g)
        alone.solve(tol, max_iters, cycle, 4)
        a, ia, ra = alone.get_grid(0)
        m, im, rm = mix.get_grid(i)
        assert (ia, ra) == (im, rm) and np.array_equal(a.view(np.uint32), m.view(np.uint32))
        alone.close()
    mix.close()


def jacobi_defect_f64(u):
    """max |J(u) - u| over the inside cells, in FP64 on the host."""
    v = u.astype(np.float64)
    j = (((v[1:-1, :-2] + v[1:-1, 2:]) + v[:-2, 1:-1]) + v[2:, 1:-1]) * 0.25
    return float(np.max(np.abs(j - v[1:-1, 1:-1])))


# Bound on the defect-correction solution's distance from the FP64 Jacobi
# iterate after the same number of sweeps: ten times the residual tolerance.
# Each cycle's correction carries a bfloat16 rounding error relative to the
# correction itself (2^-9 per stored value); the corrections shrink with the
# residual, so the accumulated deviation stays a small multiple of tol.
DC_FP64_BOUND = 10 * 1e-4


@pytest.mark.parametrize("shape", [(64, 64), (128, 128), (150, 200)])
def test_defect_correction_reaches_tolerance_near_fp64(gpu, shape):
    """A bfloat16-storage solve reaches an FP64 residual <= 1e-4 (checked
    again on the host from the returned FP32 solution) and stays within
    DC_FP64_BOUND of the FP64 oracle's Jacobi iterate after the same sweeps."""
    tol, cycle = 1e-4, 20
    g = W.jacobi_grid(*shape, 77)
    batch = gpu.Batch([shape], storage=gpu.MSL_BF16_DC)
    batch.set_grid(0, g)
    batch.solve(tol, 400_000, cycle, 4)
    u, it, res = batch.get_grid(0)
    batch.close()
    assert res <= tol and it < 400_000
    assert jacobi_defect_f64(u) == res
    ref, _, _ = O.stencil2d_iterate(0, g.astype(np.float64), 1, 0.0, it)
    err = float(np.max(np.abs(u.astype(np.float64) - ref)))
    assert err <= DC_FP64_BOUND, err


@pytest.mark.parametrize("storage", ["f32", "bf16", "bf16dc"])
def test_checkpoint_and_resume_equal_one_solve(gpu, storage, tmp_path):
    """Solve 400 sweeps, checkpoint to a file, restore into a new batch and
    continue to 1200: every grid equals one uninterrupted 1200-sweep solve
    (same sweep count, residual and bits). A second solve on the same batch
    continues the same way."""
    tol, check_every = 1e-4, (20 if storage == "bf16dc" else 100)
    grids = [W.jacobi_grid(r, c, 500 + i) for i, (r, c) in enumerate(SHAPES)]
    st = {"f32": gpu.MSL_F32, "bf16": gpu.MSL_BF16, "bf16dc": gpu.MSL_BF16_DC}[storage]
    whole = gpu.Batch(SHAPES, storage=st)
    part = gpu.Batch(SHAPES, storage=st)
    for i, g in enumerate(grids):
        whole.set_grid(i, g)
        part.set_grid(i, g)
    whole.solve(tol, 1200, check_every, 2)
    part.solve(tol, 400, check_every, 2)
    assert all(part.get_grid(i)[1] <= 400 for i in range(len(SHAPES)))
    path = str(tmp_path / "batch.ckpt")
    part.checkpoint(path)
    resumed = gpu.Batch.restore(path)
    assert resumed.shapes == SHAPES
    resumed.solve(tol, 1200, check_every, 5)  # another temporal depth: same sweeps
    part.solve(tol, 1200, check_every, 2)
    for i in range(len(SHAPES)):
        want, want_it, want_res = whole.get_grid(i)
        for b in (resumed, part):
            got, it, res = b.get_grid(i)
            assert it == want_it and res == want_res, (SHAPES[i], it, want_it)
            assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), SHAPES[i]
    resumed.reset()  # the initial values travel in the checkpoint too
    resumed.solve(tol, 1200, check_every, 2)
    for i in range(len(SHAPES)):
        assert np.array_equal(resumed.get_grid(i)[0].view(np.uint32), whole.get_grid(i)[0].view(np.uint32))
    for b in (whole, part, resumed):
        b.close()


def test_restore_rejects_bad_files(gpu, tmp_path):
    bad = tmp_path / "bad.ckpt"
    bad.write_bytes(b"not a checkpoint")
    with pytest.raises(gpu.MslError) as e:
        gpu.Batch.restore(str(bad))
    assert e.value.code == gpu.MSL_ERR_INVALID_ARGUMENT
    b = gpu.Batch([(64, 64), (300, 300)])
    b.set_grid(0, W.jacobi_grid(64, 64, 1))
    b.set_grid(1, W.jacobi_grid(300, 300, 2))
    good = tmp_path / "good.ckpt"
    b.checkpoint(str(good))
    data = good.read_bytes()
    trunc = tmp_path / "trunc.ckpt"
    trunc.write_bytes(data[:-100])
    with pytest.raises(gpu.MslError):
        gpu.Batch.restore(str(trunc))
    with pytest.raises(gpu.MslError) as e:
        gpu.Batch.restore(str(good), hbm_budget=1 << 16)
    assert e.value.code == gpu.MSL_ERR_BUDGET
    b.close()
