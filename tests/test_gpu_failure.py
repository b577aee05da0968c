"""Failure detection without faulting or hanging the GPU.

* Bounded device waits: a CTA waits on an mbarrier whose phase nothing
  completes; the wait gives up after its poll limit, the kernel reports the
  timeout in the context's error word, the host call returns MSL_ERR_TIMEOUT
  and the context keeps working. A TMA stencil run with a poll limit of one
  either finishes or reports the timeout, never leaves the context broken.
* Server: a request cancelled while queued or running leaves the other
  requests' results bit-identical to the one-request path; an allocation
  failure at admission (injected on the host) fails that request alone.
"""
import ctypes

import numpy as np
import pytest

from muesli4_gb300 import workloads as W
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu

TOL, MAX_ITERS, CHECK = 1e-4, 1000, 100


def test_wait_that_nothing_completes_reports_timeout(gpu):
    L = gpu.load()
    assert L.msl_wait_selftest(2000, 0) == gpu.MSL_ERR_TIMEOUT
    assert b"gave up" in L.msl_last_error_string()
    assert L.msl_wait_selftest(2000, 1) == gpu.MSL_OK  # the bit was cleared; a completed phase passes
    assert L.msl_sync() == gpu.MSL_OK
    g = W.jacobi_grid(64, 96, 3)
    a, b = gpu.DeviceArray.from_host(g), gpu.DeviceArray(g.shape, np.float32)
    last, res = gpu.stencil2d_iterate(gpu.MSL_ST2_JACOBI5, a, b, 1, 0.0, 7)
    want, _, want_res = O.stencil2d_iterate(0, g, 1, 0.0, 7)
    assert np.array_equal(last.download(), want) and res == want_res


def test_tma_stencil_under_a_poll_limit_of_one(gpu):
    """With one poll per wait a CTA may give up before its TMA tile lands; it
    then lets the copy land and returns. Every call ends, with MSL_OK or
    MSL_ERR_TIMEOUT, and the default limit restores correct results."""
    L = gpu.load()
    g = W.jacobi_grid(512, 512, 9)
    a, b = gpu.DeviceArray.from_host(g), gpu.DeviceArray(g.shape, np.float32)
    gpu.set_tma(True)
    seen = set()
    try:
        assert L.msl_set_wait_limit(1) == gpu.MSL_OK
        for _ in range(8):
            assert L.msl_stencil2d(gpu.MSL_F32, gpu.MSL_ST2_JACOBI5, a.ptr, b.ptr, 512, 512, 1, 0.0) == gpu.MSL_OK
            rc = L.msl_sync()
            assert rc in (gpu.MSL_OK, gpu.MSL_ERR_TIMEOUT), rc
            seen.add(rc)
    finally:
        assert L.msl_set_wait_limit(0) == gpu.MSL_OK
    assert L.msl_sync() == gpu.MSL_OK
    gpu.stencil2d(gpu.MSL_ST2_JACOBI5, a, b, 1, 0.0)
    assert np.array_equal(b.download(), O.stencil2d(0, g, 1, 0.0))
    print("statuses under a one-poll limit:", sorted(seen))


def request_init(shape, seed):
    return np.random.default_rng(seed).random(shape, dtype=np.float32)


def plain(gpu, init):
    kind = gpu.MSL_ST3_HEAT7 if init.ndim == 3 else gpu.MSL_ST2_JACOBI5
    a, b = gpu.DeviceArray.from_host(init), gpu.DeviceArray(init.shape, np.float32)
    out, it, res = gpu.solve_plain(kind, a, b, TOL, MAX_ITERS, CHECK)
    return out.download(), it, res


def assert_same(got, want):
    out, it, res = got[:3]
    w_out, w_it, w_res = want
    assert it == w_it and res == w_res
    assert np.array_equal(out.view(np.uint32), w_out.view(np.uint32))


def test_cancelled_requests_leave_the_others_unchanged(gpu):
    """A budget that admits one large request at a time keeps the later ones
    queued: one queued request and one running request are cancelled, every
    other result equals the one-request path."""
    shapes = [(1024, 1024), (512, 512), (300, 200), (64, 64), (40, 40, 40), (256, 256)]
    inits = [request_init(s, 700 + i) for i, s in enumerate(shapes)]
    budget = 2 * 1024 * 1024 * 4 + (1 << 20)  # both iterates of the 1024^2 request, plus a little
    srv = gpu.Server(hbm_budget=budget, tol=TOL, max_iters=MAX_ITERS, check_every=CHECK)
    ids = [srv.submit(x) for x in inits]
    srv.cancel(ids[3])  # still queued behind the 1024^2 request
    srv.cancel(ids[0])  # admitted first: running or about to run
    for k, rid in enumerate(ids):
        if k in (0, 3):
            with pytest.raises(gpu.MslError) as e:
                srv.wait(rid, 120.0)
            assert e.value.code == gpu.MSL_ERR_CANCELLED
            with pytest.raises(gpu.MslError) as e:
                srv.result(rid)
            assert e.value.code == gpu.MSL_ERR_CANCELLED
            continue
        srv.wait(rid, 120.0)
        assert_same(srv.result(rid), plain(gpu, inits[k]))
    with pytest.raises(gpu.MslError):
        srv.cancel(ids[1])  # finished: nothing to cancel
    st = srv.stats()
    assert st["active"] == 0 and st["queued"] == 0 and st["device_bytes"] == 0
    srv.stop()


def test_admission_allocation_failure_fails_one_request(gpu):
    L = gpu.load()
    srv = gpu.Server(tol=TOL, max_iters=MAX_ITERS, check_every=CHECK)
    first, second, third = (request_init((96, 128), 800 + i) for i in range(3))
    r1 = srv.submit(first)
    srv.wait(r1, 60.0)
    try:
        assert L.msl_debug_fail_allocs(0) == gpu.MSL_OK
        r2 = srv.submit(second)
        with pytest.raises(gpu.MslError) as e:
            srv.wait(r2, 60.0)
        assert e.value.code == gpu.MSL_ERR_OUT_OF_MEMORY
    finally:
        L.msl_debug_fail_allocs(-1)
    r3 = srv.submit(third)
    srv.wait(r3, 60.0)
    assert_same(srv.result(r1), plain(gpu, first))
    assert_same(srv.result(r3), plain(gpu, third))
    assert srv.stats()["device_bytes"] == 0
    srv.stop()
