"""Multi-rank path of bench.py on CPU: world_size 2 over gloo (127.0.0.1).

The library does not shard (one box per GPU, replicas only), so the only
cross-rank logic is the timing: the slowest replica's time, the whole-job
rate over all replicas, and rank 0 alone printing.
"""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

import bench


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    w, r, loc = bench.dist_setup()
    elapsed = bench.max_over_ranks(1.0 + r, w, device="cpu")  # rank 1 is the slow replica
    rate = bench.whole_job_rate(8_388_608, 4, w, elapsed)
    dist.barrier()
    q.put((r, w, loc, elapsed, rate))
    dist.destroy_process_group()


def test_two_replicas_take_the_slowest_time():
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
    assert [o[0] for o in out] == [0, 1] and all(o[1] == 2 for o in out)
    for _, _, _, elapsed, rate in out:
        assert elapsed == 2.0
        assert rate == pytest.approx(8_388_608 * 4 * 2 / 2.0 / 1e6)


def test_single_rank_needs_no_process_group():
    assert bench.max_over_ranks(3.5, 1) == 3.5
    assert bench.whole_job_rate(10**6, 2, 1, 2.0) == pytest.approx(1.0)
