"""Replica harness of bench.py with world size 2 on CPU (gloo): every rank
sees the max duration over ranks and the whole-job rate; the reference arm's
non-zero ranks exit without work."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    sys.path.insert(0, ROOT)
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = [120.0, 80.0][rank]
    mx = bench.max_over_ranks(ms, dist, "cpu")
    rate = bench.whole_job_rate(world, 5, mx)
    dist.barrier()
    q.put((rank, mx, rate))
    dist.destroy_process_group()


def test_max_over_ranks_and_rate_with_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, mx, rate in out:
        assert mx == 120.0
        assert abs(rate - 2 * 5 / 0.12) < 1e-9


def test_reference_arm_nonzero_rank_exits_without_work(monkeypatch):
    sys.path.insert(0, ROOT)
    import bench

    monkeypatch.setenv("RANK", "1")

    class A:
        steps, warmup, gpus = 1, 0, 2

    assert bench.run_reference(A(), [4, 4, 4, 4]) == 0
