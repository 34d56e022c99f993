"""The N>1 path of bench.py on CPU: two gloo ranks (replicas). The barrier
and the max-over-ranks time work across ranks, the whole-job value is the
units of all ranks over the slowest rank's time, and the reference arm runs
on rank 0 only (the other ranks exit 0 without work)."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    r, w, _ = bench.env_rank()
    bench.dist_init(w, "gloo")
    bench.dist_barrier(w)
    ms = bench.max_over_ranks(10.0 + 5.0 * r, w, "cpu")  # rank 1 is slower
    steps = 7
    value = w * steps / (ms / 1e3)  # iterations of all ranks over the slowest time
    import torch.distributed as dist
    dist.barrier()
    dist.destroy_process_group()

    class A:
        gpus, steps, warmup = w, 3, 3
    ref = bench.run_reference(A) if r == 1 else None  # rank 1 returns before any work
    q.put((r, ms, value, ref))


def test_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[1] for o in out] == [15.0, 15.0]  # both ranks see the max
    assert out[0][2] == pytest.approx(2 * 7 / 0.015)
    assert out[1][3] == 0
