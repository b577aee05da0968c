"""The stencil-solve server (msl_server_*): continuous batching of plain-Jacobi
(2-D) and heat3D (3-D) solves.

Each request's result must be bit-identical to the one-request path
(msl_stencil2d_iterate / msl_stencil3d_iterate in chunks of check_every
sweeps) -- alone, in a mix of other requests, and when it arrives while other
requests are already running or has to wait for memory under a small HBM
budget.
"""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL, MAX_ITERS, CHECK = 1e-4, 1000, 100


def request_init(shape, seed):
    return np.random.default_rng(seed).random(shape, dtype=np.float32)


def plain(gpu, init):
    kind = gpu.MSL_ST3_HEAT7 if init.ndim == 3 else gpu.MSL_ST2_JACOBI5
    a, b = gpu.DeviceArray.from_host(init), gpu.DeviceArray(init.shape, np.float32)
    out, it, res = gpu.solve_plain(kind, a, b, TOL, MAX_ITERS, CHECK)
    return out.download(), it, res


SHAPES = [(64, 64), (100, 300), (257, 129), (16, 16, 16), (24, 40, 70), (33, 17, 64), (512, 512), (40, 40, 40),
          (1024, 1024), (72, 160, 128)]  # the last two fill the GPU alone: one-request kernels


def assert_same(got, want):
    out, it, res = got[:3]
    w_out, w_it, w_res = want
    assert it == w_it and res == w_res
    assert np.array_equal(out.view(np.uint32), w_out.view(np.uint32))


def test_mix_equals_one_request_path(gpu):
    inits = [request_init(s, 100 + i) for i, s in enumerate(SHAPES)]
    srv = gpu.Server(tol=TOL, max_iters=MAX_ITERS, check_every=CHECK)
    ids = [srv.submit(x) for x in inits]
    for rid in ids:
        srv.wait(rid, 120.0)
    for rid, x in zip(ids, inits):
        assert_same(srv.result(rid), plain(gpu, x))
    st = srv.stats()
    assert st["completed"] == len(SHAPES) and st["active"] == 0 and st["queued"] == 0
    srv.stop()


def test_alone_equals_in_the_mix(gpu):
    inits = [request_init(s, 200 + i) for i, s in enumerate(SHAPES[:6])]
    mix = gpu.Server(tol=TOL, max_iters=MAX_ITERS, check_every=CHECK)
    ids = [mix.submit(x) for x in inits]
    for rid in ids:
        mix.wait(rid, 120.0)
    for rid, x in zip(ids, inits):
        alone = gpu.Server(tol=TOL, max_iters=MAX_ITERS, check_every=CHECK)
        one = alone.submit(x)
        alone.wait(one, 120.0)
        assert_same(mix.result(rid), alone.result(one)[:3])
        alone.stop()
    mix.stop()


def test_arrivals_while_running_and_budget_queueing(gpu):
    inits = [request_init(s, 300 + i) for i, s in enumerate(SHAPES)]
    biggest = max(2 * x.size * 4 for x in inits)
    srv = gpu.Server(hbm_budget=2 * biggest + (1 << 20), tol=TOL, max_iters=MAX_ITERS, check_every=CHECK)
    ids = []
    for x in inits:  # staggered arrivals: later requests join running ones
        ids.append(srv.submit(x))
        time.sleep(0.002)
    for rid in ids:
        srv.wait(rid, 120.0)
    queued = 0
    for rid, x in zip(ids, inits):
        got = srv.result(rid)
        queued += got[4] > 0.0
        assert_same(got, plain(gpu, x))
        srv.release(rid)
    assert srv.stats()["device_bytes"] == 0
    srv.stop()


def test_request_larger_than_budget_is_rejected(gpu):
    srv = gpu.Server(hbm_budget=1 << 20, tol=TOL, max_iters=MAX_ITERS, check_every=CHECK)
    with pytest.raises(gpu.MslError) as e:
        srv.submit(request_init((1024, 1024), 1))
    assert e.value.code == gpu.MSL_ERR_BUDGET
    with pytest.raises(gpu.MslError):
        srv.wait(12345, 0.1)  # unknown request
    srv.stop()


def test_checkpoint_and_restore_equal_uninterrupted(gpu, tmp_path):
    """A checkpoint taken while requests run (some queued behind a small HBM
    budget) restores into a new server whose results equal the live server's
    and the one-request path: same sweeps, residual and bits."""
    tol, max_iters, check = 1e-7, 20000, 100
    shapes = [(1024, 1024)] * 4 + [(96, 96, 96), (64, 80, 72)]
    inits = [request_init(sh, 400 + i) for i, sh in enumerate(shapes)]
    budget = 3 * 2 * 1024 * 1024 * 4 + (1 << 22)  # three 2-D requests at a time
    live = gpu.Server(hbm_budget=budget, tol=tol, max_iters=max_iters, check_every=check)
    ids = [live.submit(x) for x in inits]
    time.sleep(0.15)
    path = str(tmp_path / "server.ckpt")
    live.checkpoint(path)
    recs = gpu.Server.read_checkpoint_records(path)
    assert sorted(r[0] for r in recs) == sorted(ids)
    assert all(r[6] % check == 0 for r in recs)
    assert any(r[2] == 1 and 0 < r[6] < max_iters for r in recs)  # caught mid-solve
    restored = gpu.Server.restore(path)
    for rid in ids:
        live.wait(rid, 300.0)
        restored.wait(rid, 300.0)
    for rid, x in zip(ids, inits):
        want = live.result(rid)
        got = restored.result(rid)
        assert got[1] == want[1] and got[2] == want[2]
        assert np.array_equal(got[0].view(np.uint32), want[0].view(np.uint32))
        w_out, w_it, w_res = plain_with(gpu, x, tol, max_iters, check)
        assert want[1] == w_it and want[2] == w_res
        assert np.array_equal(want[0].view(np.uint32), w_out.view(np.uint32))
    live.stop()
    restored.stop()


def plain_with(gpu, init, tol, max_iters, check):
    kind = gpu.MSL_ST3_HEAT7 if init.ndim == 3 else gpu.MSL_ST2_JACOBI5
    a, b = gpu.DeviceArray.from_host(init), gpu.DeviceArray(init.shape, np.float32)
    out, it, res = gpu.solve_plain(kind, a, b, tol, max_iters, check)
    return out.download(), it, res


def test_checkpoint_with_halt(gpu, tmp_path):
    """halt stops the worker after the write: unfinished requests report it,
    new submissions are refused, and the restored server finishes them."""
    inits = [request_init((512, 512), 500 + i) for i in range(3)]
    srv = gpu.Server(tol=1e-7, max_iters=20000, check_every=100)
    ids = [srv.submit(x) for x in inits]
    time.sleep(0.05)
    path = str(tmp_path / "halt.ckpt")
    srv.checkpoint(path, halt=True)
    unfinished = [r[0] for r in gpu.Server.read_checkpoint_records(path) if r[2] != 2]
    for rid in unfinished:
        with pytest.raises(gpu.MslError):
            srv.wait(rid, 1.0)
    with pytest.raises(gpu.MslError):
        srv.submit(inits[0])
    srv.stop()
    back = gpu.Server.restore(path)
    for rid, x in zip(ids, inits):
        back.wait(rid, 300.0)
        got = back.result(rid)
        w_out, w_it, w_res = plain_with(gpu, x, 1e-7, 20000, 100)
        assert got[1] == w_it and got[2] == w_res
        assert np.array_equal(got[0].view(np.uint32), w_out.view(np.uint32))
    back.stop()


def test_restore_rejects_bad_files(gpu, tmp_path):
    p = tmp_path / "bad.ckpt"
    p.write_bytes(b"MSLSRV01" + b"\0" * 10)
    with pytest.raises(gpu.MslError) as e:
        gpu.Server.restore(str(p))
    assert e.value.code == gpu.MSL_ERR_INVALID_ARGUMENT
