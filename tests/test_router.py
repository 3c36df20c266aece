"""Multi-device split of independent QPs (osqp_gb300/router.py): the
cost-balanced contiguous partition, and two gloo ranks on the CPU that each
solve their share and gather the results -- identical, in the caller's order,
to one process solving everything.  The per-rank solver here is the FP64
oracle (CPU), standing in for a rank's device batch: what is tested is the
partition and the ordered gather."""
import os
import socket
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, REPO)

from osqp_gb300.router import partition, qp_cost, gather_in_order  # noqa: E402

SETTINGS = dict(eps_abs=1e-3, eps_rel=1e-3, rho_is_vec=1, check_termination=5, adaptive_rho_tolerance=5.0,
                max_iter=4000, check_dualgap=1, linsys_solver=1)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_partition_is_contiguous_balanced_and_complete():
    rng = np.random.default_rng(0)
    for count, parts in ((100, 7), (10, 3), (5, 5), (4096, 8), (3, 2)):
        w = rng.uniform(1.0, 10.0, count)
        rs = partition(w, parts)
        assert len(rs) == parts
        assert rs[0].start == 0 and rs[-1].stop == count
        assert all(a.stop == b.start for a, b in zip(rs, rs[1:]))
        assert all(len(r) > 0 for r in rs)
        loads = np.array([w[r.start:r.stop].sum() for r in rs])
        assert loads.max() <= w.sum() / parts + w.max() + 1e-9


def test_single_process_gather_is_identity():
    d = {"x": np.arange(5.0), "status": np.array([1, 1, 2], np.int32)}
    g = gather_in_order(d, None)
    assert all(np.array_equal(g[k], d[k]) for k in d)


def _problems():
    from osqp_gb300 import problems as pb
    return [pb.mpc(np.random.default_rng([17, i])) for i in range(10)]


def _solve(problems):
    from osqp_gb300.api import Library, OSQP
    lib = Library(os.path.join(REPO, "oracle", "_build", "liboracle.so"), 64)
    xs, st = [], []
    for d in problems:
        s = OSQP(lib)
        assert s.setup(*d, **SETTINGS) == 0
        r = s.solve()
        xs.append(np.asarray(r.x)); st.append(r.info["status_val"])
    return {"x": np.concatenate(xs), "status": np.array(st, np.int32)}


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist
    dist.init_process_group("gloo")
    probs = _problems()
    share = partition([qp_cost(p) for p in probs], world)[rank]
    local = _solve([probs[i] for i in share])
    got = gather_in_order(local, dist)
    dist.barrier()
    dist.destroy_process_group()
    out.put((rank, got["x"].tobytes(), got["status"].tolist()))


def test_two_gloo_ranks_gather_in_caller_order(oracle_lib):
    pytest.importorskip("torch")
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = dict((r, (x, s)) for r, x, s in (q.get(timeout=300) for _ in ps))
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    ref = _solve(_problems())
    for r in range(2):
        x = np.frombuffer(res[r][0], dtype=ref["x"].dtype)
        assert np.array_equal(x, ref["x"])            # bit-identical, same order
        assert res[r][1] == ref["status"].tolist()
