"""Host logic of the multi-GPU bench path, run as two CPU ranks over gloo.

The path does not shard: each rank traces its own full frame (replicas), the
job's time is the slowest rank's and its throughput is the rays of all
replicas over that time (bench.py slowest_ms / whole_job_mrays).
"""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
mp = pytest.importorskip("torch.multiprocessing")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, times, out_q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        t = bench.slowest_ms(times[rank], world)
        dist.barrier()
        out_q.put((rank, t, bench.whole_job_mrays(world, 1_000_000, t)))
    finally:
        dist.destroy_process_group()


def test_two_replicas_report_the_slowest_rank():
    world, times = 2, [1.25, 2.5]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, times, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [2.5, 2.5]
    # 2 replicas x 1M rays in 2.5 ms
    assert abs(res[0][2] - 800.0) < 1e-9 and res[0][2] == res[1][2]


def test_single_rank_needs_no_process_group():
    import bench
    assert bench.slowest_ms(3.0, 1) == 3.0
    assert bench.whole_job_mrays(1, 2_000_000, 2.0) == 1000.0
