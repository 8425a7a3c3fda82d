"""The multi-GPU path is replicas only: every rank advances its own channel and
bench.py reports all ranks' time steps over the slowest rank's time.  Its host
logic (barrier, max over ranks, the whole-job value) runs here over two gloo
ranks on the CPU; the reference arm does its work on rank 0 only."""
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
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        bench.barrier(world)
        ms = bench.max_over_ranks(10.0 * (rank + 1), world)   # rank r "took" 10 (r + 1) ms
        q.put((rank, ms, bench.replica_value(world, 4, ms)))
        bench.barrier(world)
    finally:
        dist.destroy_process_group()


def test_replica_timing_over_two_gloo_ranks():
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
    assert [p.exitcode for p in procs] == [0, 0]
    assert [o[1] for o in out] == [20.0, 20.0]             # every rank sees the slowest rank's time
    assert out[0][2] == pytest.approx(2 * 4 / 0.020)      # both ranks' steps over that time


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5, 1) == 3.5
    assert bench.replica_value(1, 3, 250.0) == pytest.approx(12.0)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")
    assert bench.run_reference(None) is None   # returns before touching its arguments
    assert capsys.readouterr().out == ""
