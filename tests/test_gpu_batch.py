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


@pytest.mark.parametrize("storage", ["f32", "bf16"])
def test_checkpoint_and_resume_equal_one_solve(gpu, storage, tmp_path):
    """Solve 400 sweeps, checkpoint to a file, restore into a new batch and
    continue to 1200: every grid equals one uninterrupted 1200-sweep solve
    (same sweep count, residual and bits). A second solve on the same batch
    continues the same way."""
    tol, check_every = 1e-4, 100
    grids = [W.jacobi_grid(r, c, 500 + i) for i, (r, c) in enumerate(SHAPES)]
    st = gpu.MSL_F32 if storage == "f32" else gpu.MSL_BF16
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
