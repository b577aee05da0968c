"""The multi-process (replicas) side of bench.py on CPU: two ranks over the
gloo backend, as `torchrun --nproc-per-node 2 bench.py` runs them.

The path does not shard, so ranks share nothing but the timing: a barrier
around the timed region, the maximum of the per-rank times and the sum of
the per-rank work. The reference arm runs on rank 0 only; the other ranks
exit without work.
"""
import multiprocessing as mp
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def rank_env(rank, world, port):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    if ROOT not in sys.path:
        sys.path.insert(0, ROOT)


def timing_worker(rank, world, port, q):
    rank_env(rank, world, port)
    import bench
    d = bench.Dist()
    d.barrier()
    t = d.max(0.5 + rank)          # per-rank time of the timed region
    work = d.sum(1000.0 * (rank + 1))  # per-rank cell updates
    d.barrier()
    q.put((rank, d.world, t, work))
    d.close()


def reference_worker(rank, world, port, q):
    rank_env(rank, world, port)
    import bench

    class Args:
        workload, steps, warmup, gpus = "box", 1, 0, world

    d = bench.Dist()
    if d.rank != 0:  # must return at once: no oracle build, no output
        bench.run_reference(Args, d)
        q.put((rank, "returned"))
    else:
        q.put((rank, "rank0"))
    d.close()


def run_ranks(target, world=2):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=target, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    return sorted(out)


def test_two_replicas_reduce_timings_over_gloo():
    pytest.importorskip("torch.distributed")
    out = run_ranks(timing_worker)
    assert [o[0] for o in out] == [0, 1]
    for _, world, t, work in out:
        assert world == 2
        assert t == 1.5          # the slowest rank's time
        assert work == 3000.0    # whole-job work


def test_reference_arm_runs_on_rank_zero_only():
    pytest.importorskip("torch.distributed")
    out = run_ranks(reference_worker)
    assert out == [(0, "rank0"), (1, "returned")]
