"""Request serving (osqp_gb300_server_*): continuous batching over resident pools.

Bars: a request's result is bit-identical whether it is served alone or in a
mix of concurrent requests (same pool state, same inputs); served results meet
the batch engine's parity bars against the FP64 oracle; pool set-up is refused
cleanly when free device memory cannot hold it.
"""
import numpy as np
import pytest

from osqp_gb300 import load
from osqp_gb300 import problems as pb
from osqp_gb300.api import Batch, Server, SOLVED, objective
from test_batch_gpu import WORKLOAD, _mix, check_against_oracles

pytestmark = pytest.mark.gpu

SERVE = dict(WORKLOAD, warm_starting=1)


def _requests(probs, rounds, seed):
    """Per round and QP: new bounds (MPC: new x0) or a new linear cost."""
    rg = np.random.default_rng(seed)
    out = []
    for r in range(rounds):
        row = []
        for (P, q, A, l, u) in probs:
            rowlen = np.diff(A.tocsr().indptr)
            if A.shape[0] and rowlen[0] == 1 and np.all(l[:1] == u[:1]):
                nx = int(np.argmax(rowlen != 1)) or 1
                l2, u2 = pb.mpc_x0_bounds(l, u, rg.uniform(-1.0, 1.0, nx))
                row.append((None, l2, u2))
            else:
                row.append((q * (1.0 + 0.1 * rg.standard_normal(q.size)), None, None))
        out.append(row)
    return out


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_served_alone_and_in_mix_identical(prec):
    lib = load(prec)
    probs = _mix(10, seed=5)
    reqs = _requests(probs, 3, seed=6)
    pa, pb_ = Batch(lib), Batch(lib)
    assert pa.setup(probs, **SERVE) == 0 and pb_.setup(probs, **SERVE) == 0
    srv = Server(lib, concurrency=4)
    ia, ib = srv.add_pool(pa), srv.add_pool(pb_)
    ns = [p[0].shape[0] for p in probs]
    for row in reqs:
        alone = []
        for k, (q, l, u) in enumerate(row):     # one request at a time
            t = srv.submit(ia, k, q, l, u)
            alone.append(srv.wait(t, ns[k]))
        tickets = [srv.submit(ib, k, q, l, u) for k, (q, l, u) in enumerate(row)]   # all at once
        mixed = [srv.wait(t, ns[k]) for k, t in enumerate(tickets)]
        for a, m in zip(alone, mixed):
            assert a[1] == m[1] and a[2] == m[2]
            assert np.array_equal(a[0], m[0])
    srv.close()


def test_served_results_match_oracle(oracle_lib):
    lib = load("f32")
    probs = _mix(8, seed=7)
    reqs = _requests(probs, 2, seed=8)
    pool = Batch(lib)
    assert pool.setup(probs, **SERVE) == 0
    srv = Server(lib, concurrency=3)
    pid = srv.add_pool(pool)
    cur = [list(p) for p in probs]
    for row in reqs:
        tickets = []
        for k, (q, l, u) in enumerate(row):
            if q is not None:
                cur[k][1] = q
            if l is not None:
                cur[k][3], cur[k][4] = l, u
            tickets.append(srv.submit(pid, k, q, l, u))
        for k, t in enumerate(tickets):
            x, status, it, obj, lat = srv.wait(t, probs[k][0].shape[0])
            assert lat > 0.0
            d = tuple(cur[k])
            obj_gpu = objective(d[0], d[1], x.astype(np.float64)) if status == SOLVED else None
            check_against_oracles(oracle_lib, d, status, obj_gpu, "f32")
    srv.close()


def test_submit_validates_inputs():
    lib = load("f32")
    probs = _mix(3, seed=9)
    pool = Batch(lib)
    assert pool.setup(probs, **SERVE) == 0
    srv = Server(lib, concurrency=1)
    pid = srv.add_pool(pool)
    with pytest.raises(ValueError):
        srv.submit(pid + 1, 0)
    with pytest.raises(ValueError):
        srv.submit(pid, 3)
    P, q, A, l, u = probs[0]
    with pytest.raises(ValueError):
        srv.submit(pid, 0, None, u + 1.0, u)      # l > u
    srv.close()


def test_pool_admission_by_free_memory():
    torch = pytest.importorskip("torch")
    lib = load("f32")
    probs = _mix(4, seed=10)
    free, _ = torch.cuda.mem_get_info()
    hog = torch.empty(int(free - (48 << 20)), dtype=torch.uint8, device="cuda")
    try:
        b = Batch(lib)
        assert b.setup(probs, **SERVE) != 0          # refused: the pool would not fit
    finally:
        del hog
        torch.cuda.empty_cache()
    b = Batch(lib)
    assert b.setup(probs, **SERVE) == 0
    assert b.solve() == 0


def test_new_structure_admitted_while_serving(oracle_lib):
    """A QP of a structure no pool holds is admitted while requests are in
    flight: set up as a one-QP pool and added to the running server (the
    per-request counterpart of osqp_setup, src/osqp_api.c:332-631).  Its
    results meet the oracle's bars, and a matrix update of that pool between
    its requests (osqp_gb300_batch_update_data_mat) is served with the new
    values."""
    from osqp_gb300.api import DIRECT_SOLVER, OSQP
    lib = load("f64")
    st = dict(SERVE, linsys_solver=DIRECT_SOLVER)
    probs = pb.mpc_batch(6, seed=40)
    pool = Batch(lib)
    assert pool.setup(probs, **st) == 0
    srv = Server(lib, concurrency=3)
    pid = srv.add_pool(pool)
    busy = [srv.submit(pid, k) for k in range(len(probs))]          # requests in flight
    new = pb.mpc(np.random.default_rng(41))
    one = Batch(lib)
    assert one.setup([new], **st) == 0
    nid = srv.add_pool(one)                                          # admitted while serving
    x, status, it, obj, lat = srv.wait(srv.submit(nid, 0), new[0].shape[0])
    o = OSQP(oracle_lib)
    assert o.setup(*new, **st) == 0
    r = o.solve()
    assert status == r.info["status_val"] == SOLVED
    assert abs(objective(new[0], new[1], x) - r.info["obj_val"]) <= 1e-7 * max(1.0, abs(r.info["obj_val"]))
    assert it == r.info["iter"]
    for k, t in enumerate(busy):
        srv.wait(t, probs[k][0].shape[0])
    # new A values for the admitted QP, between its requests
    A = new[2].tocsc()
    ax = A.data * 1.03
    assert one.update_mat(0, Ax=ax) == 0
    assert o.update(Ax=ax) == 0
    x, status, it, obj, lat = srv.wait(srv.submit(nid, 0), new[0].shape[0])
    r = o.solve()
    assert status == r.info["status_val"] == SOLVED
    assert abs(objective(new[0], new[1], x) - r.info["obj_val"]) <= 1e-7 * max(1.0, abs(r.info["obj_val"]))
    assert it == r.info["iter"]
    srv.close()
