"""bench.py --gpus N runs N independent replicas (no data-path collective): the
host side takes the slowest rank's time and reports the whole-job rate.  The
multi-process path is exercised here with two gloo ranks on the CPU."""
import os
import socket
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, REPO)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import bench
    dist = bench.replica_group(world)
    got = bench.max_over_ranks([1.0 + rank, 10.0 - rank, 0.5 * rank], dist)
    dist.barrier()
    dist.destroy_process_group()
    out.put((rank, got.tolist()))


def test_max_over_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = dict(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in range(2):
        assert res[r] == [2.0, 10.0, 0.5]


def test_single_process_needs_no_group():
    import bench
    assert bench.replica_group(1) is None
    assert np.array_equal(bench.max_over_ranks([3.0, 4.0], None), [3.0, 4.0])


def test_whole_job_rate_is_weak_scaling_aggregate():
    import bench
    # 4096 QPs per rank and step, 3 steps, 2 ranks, slowest rank 30 s
    assert bench.whole_job_rate(4096 * 3, 2, 30.0) == pytest.approx(819.2)
