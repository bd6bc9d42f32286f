"""bench.py's multi-GPU form on the CPU: two gloo ranks.

A realisation does not shard, so `bench.py --gpus N` runs N independent
replicas, one per GPU; the ranks only meet at the barriers around the timed
region and in the max-over-ranks reduction of the timing. This checks that
host logic with world size 2 over gloo (127.0.0.1), and that the reference
arm does its work on rank 0 only.
"""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench

    ws, r, local = bench.dist_env()
    dist = bench.init_dist(ws)
    bench.barrier(dist)
    # per-rank elapsed times; every rank must see the slowest
    t = bench.reduce_max(dist, 10.0 + 5.0 * r)
    bench.barrier(dist)

    class Args:
        workload = "c0"

    # the reference arm runs on rank 0 only; other ranks leave without work
    rc_ref = bench.run_reference(Args, ws, r) if r != 0 else None
    dist.destroy_process_group()
    out.put((r, ws, local, t, rc_ref))


def test_two_gloo_ranks_time_as_the_slowest_replica():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [x[0] for x in res] == [0, 1]
    assert all(x[1] == 2 for x in res)
    assert [x[2] for x in res] == [0, 1]
    assert all(x[3] == pytest.approx(15.0) for x in res)
    assert res[1][4] == 0


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.init_dist(1) is None
    assert bench.reduce_max(None, 3.5) == 3.5
    bench.barrier(None)
