"""Multi-process host logic on CPU (gloo, world size 2), no GPU.

The benchmark runs one replica per GPU (the 2D update does not shard here:
replicas only).  Its host logic is the timing reduction (the job ends when
the slowest replica does) and the whole-job rate (every rank's cell updates
over that time).  Two ranks with different local times must both get the
slower one, and the rate must count both ranks' work.
"""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        local_ms = [250.0, 400.0][rank]
        ms = bench.max_over_ranks(local_ms, world, "cpu")
        rate = bench.whole_job_rate(10**9, world, ms)
        q.put((rank, ms, rate))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_and_whole_job_rate_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    got = sorted(q.get(timeout=5) for _ in range(2))
    for rank, ms, rate in got:
        assert ms == 400.0, (rank, ms)
        assert rate == pytest.approx(2 * 10**9 / 0.4 / 1e9)  # 5 Gcell-updates/s over both ranks


def test_single_rank_needs_no_process_group():
    import bench
    assert bench.max_over_ranks(123.0, 1, "cpu") == 123.0
    assert bench.whole_job_rate(10**9, 1, 1000.0) == pytest.approx(1.0)
