"""Direct KKT solver of the batched engine (linsys_solver = OSQP_DIRECT_SOLVER)
against the FP64 oracle's builtin algebra (direct LDL' KKT solve, the
reference's own default): same status per QP, objective within 1e-4 relative
(FP32; 1e-7 FP64), ADMM iteration count within 10 %, through updates of the
bounds; results independent of the batch; non-convex QPs end NON_CVX."""
import numpy as np
import pytest
import scipy.sparse as sp

from osqp_gb300 import load
from osqp_gb300 import problems as pb
from osqp_gb300.api import OSQP, Batch, SOLVED, NON_CVX, DIRECT_SOLVER, objective

pytestmark = pytest.mark.gpu

WORKLOAD = dict(rho=0.1, sigma=1e-6, alpha=1.6, scaling=10, eps_abs=1e-3, eps_rel=1e-3, rho_is_vec=1,
                check_termination=5, adaptive_rho_tolerance=5.0, max_iter=4000, check_dualgap=1)
OBJ_TOL = {"f32": 1e-4, "f64": 1e-7}


def oracle_solve(oracle_lib, d, settings=WORKLOAD):
    s = OSQP(oracle_lib)
    assert s.setup(*d, linsys_solver=DIRECT_SOLVER, **settings) == 0
    return s, s.solve()


def compare(oracle_results, probs, sol, xs, prec, report):
    """Per QP: status, objective (relative to max(1, |obj|)), iterations."""
    bad_status, obj_err, it_ratio = [], [], []
    for k, (d, r) in enumerate(zip(probs, oracle_results)):
        st_o = r.info["status_val"]
        if sol["status"][k] != st_o:
            bad_status.append((k, int(sol["status"][k]), st_o))
            continue
        if st_o != SOLVED:
            continue
        og = objective(d[0], d[1], xs[k].astype(np.float64))
        oo = r.info["obj_val"]
        obj_err.append(abs(og - oo) / max(1.0, abs(oo)))
        it_ratio.append(sol["iter"][k] / max(1, r.info["iter"]))
    obj_err = np.array(obj_err)
    it_ratio = np.array(it_ratio)
    report(f"[{prec}] {len(probs)} QPs: status mismatches {len(bad_status)}; objective rel err median "
           f"{np.median(obj_err):.2e} max {obj_err.max():.2e}; iteration ratio {it_ratio.min():.3f}.."
           f"{it_ratio.max():.3f}")
    return bad_status, obj_err, it_ratio


@pytest.mark.parametrize("prec,count", [("f32", 256), ("f64", 64)])
def test_direct_batch_mpc_matches_builtin(prec, count, oracle_lib, capsys):
    probs = pb.mpc_batch(count, seed=5)
    b = Batch(load(prec))
    assert b.setup(probs, linsys_solver=DIRECT_SOLVER, **WORKLOAD) == 0
    assert b.solve() == 0
    sol = b.solution()
    xs = b.split(sol["x"], "n")
    res = [oracle_solve(oracle_lib, d)[1] for d in probs]
    with capsys.disabled():
        bad, err, ratio = compare(res, probs, sol, xs, prec, print)
    assert not bad, bad
    assert err.max() <= OBJ_TOL[prec], err.max()
    assert np.all(np.abs(ratio - 1.0) <= 0.10), ratio
    b.cleanup()


def test_direct_receding_horizon_updates(oracle_lib, capsys):
    """Three steps of new initial states (new l, u) through
    osqp_gb300_batch_update_data_vec; the oracle is updated the same way."""
    probs = pb.mpc_batch(48, seed=9)
    b = Batch(load("f32"))
    assert b.setup(probs, linsys_solver=DIRECT_SOLVER, **WORKLOAD) == 0
    orc = [oracle_solve(oracle_lib, d)[0] for d in probs]
    nxs = [int(np.argmax(np.diff(d[2].tocsr().indptr) != 1)) for d in probs]
    for step in range(3):
        rg = np.random.default_rng([9, step])
        ls, us = [], []
        for d, nx in zip(probs, nxs):
            l2, u2 = pb.mpc_x0_bounds(d[3], d[4], rg.uniform(-1.0, 1.0, nx))
            ls.append(l2); us.append(u2)
        assert b.update(l=np.concatenate(ls), u=np.concatenate(us)) == 0
        assert b.solve() == 0
        sol = b.solution()
        xs = b.split(sol["x"], "n")
        res = []
        for s, l2, u2 in zip(orc, ls, us):
            s.update(l=l2, u=u2)
            res.append(s.solve())
        cur = [(d[0], d[1], d[2], l2, u2) for d, l2, u2 in zip(probs, ls, us)]
        with capsys.disabled():
            bad, err, ratio = compare(res, cur, sol, xs, f"f32 step {step}", print)
        assert not bad, bad
        assert err.max() <= OBJ_TOL["f32"], err.max()
    b.cleanup()


def test_direct_alone_and_in_mix_identical():
    probs = pb.mpc_batch(12, seed=13)
    lib = load("f32")
    b = Batch(lib)
    assert b.setup(probs, linsys_solver=DIRECT_SOLVER, **WORKLOAD) == 0 and b.solve() == 0
    mix = b.split(b.solution()["x"], "n")
    b.cleanup()
    for k in (0, 5, 11):
        a = Batch(lib)
        assert a.setup([probs[k]], linsys_solver=DIRECT_SOLVER, **WORKLOAD) == 0 and a.solve() == 0
        alone = a.solution()["x"]
        a.cleanup()
        assert np.array_equal(alone.view(np.uint32), mix[k].view(np.uint32))


def test_direct_nonconvex_status():
    # indefinite P: K = P + sigma I + rho A'A is not positive definite
    P = sp.csc_matrix(np.array([[2.0, 5.0], [5.0, 1.0]]))
    A = sp.eye(2, format="csc")
    d_bad = (sp.triu(P, format="csc"), np.array([1.0, 1.0]), A, -np.ones(2), np.ones(2))
    d_ok = pb.mpc(np.random.default_rng(1))
    b = Batch(load("f32"))
    assert b.setup([d_ok, d_bad], linsys_solver=DIRECT_SOLVER, **dict(WORKLOAD, scaling=0)) == 0
    assert b.solve() == 0
    st = b.solution()["status"]
    assert st[0] == SOLVED and st[1] == NON_CVX, st
    b.cleanup()


def test_direct_rejects_dense_coupling():
    # a budget row over every asset makes one block of all of them
    b = Batch(load("f32"))
    rc = b.setup([pb.portfolio(4, n=400)], linsys_solver=DIRECT_SOLVER, **WORKLOAD)
    assert rc == 3   # OSQP_LINSYS_SOLVER_INIT_ERROR
