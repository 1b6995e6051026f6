"""Replica (N > 1) host logic of bench.py on CPU: two gloo ranks.

The path does not shard, so bench.py runs one independent sparse-FFT replica
per rank; what the ranks share is the timing reduction (the job's time is the
slowest rank's) and the whole-job rate.  The reference arm runs on rank 0
only; other ranks exit without work."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, times, out_q):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    t = bench.max_over_ranks(times[rank], dist, "cpu")
    rate = bench.job_rate(world, 10, t)
    dist.barrier()
    dist.destroy_process_group()
    out_q.put((rank, t, rate))


def test_two_rank_timing_reduction():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    times = [0.5, 0.8]
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, times, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t, rate in res:
        assert t == pytest.approx(0.8)               # slowest replica
        assert rate == pytest.approx(2 * 10 / 0.8)   # all ranks' steps over that time


def test_reference_arm_other_ranks_exit(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("LOCAL_RANK", "1")

    class A:
        steps, warmup = 1, 3
    assert bench.run_reference(A(), dict(bench.CFG)) == 0
    assert capsys.readouterr().out == ""  # no line, no work
