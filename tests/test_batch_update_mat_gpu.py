"""New P / A values for QPs of a batch (osqp_gb300_batch_update_data_mat)
against the oracle's osqp_update_data_mat (src/osqp_api.c:1309-1409), run
through the same sequence on both sides: set-up, solve, new matrix values
(all entries, or some by index), solve.  The update re-scales the QP and
refactors it, keeping rho and the iterates, as the reference does.

Bars.  FP64 build, direct solver: the builtin's trajectory -- same status, same
ADMM iteration count and objective within 1e-7 relative on every QP.  FP32
build, PCG: same status, objective within the eps class (1e-2 relative at
eps 1e-3).  Bad counts and out-of-range indices are rejected with the
reference's codes and change nothing."""
import numpy as np
import pytest
import scipy.sparse as sp

from osqp_gb300 import load
from osqp_gb300 import problems as pb
from osqp_gb300.api import OSQP, Batch, SOLVED, DIRECT_SOLVER, INDIRECT_SOLVER, objective

pytestmark = pytest.mark.gpu

WORKLOAD = dict(rho=0.1, sigma=1e-6, alpha=1.6, scaling=10, eps_abs=1e-3, eps_rel=1e-3, rho_is_vec=1,
                check_termination=5, adaptive_rho_tolerance=5.0, max_iter=4000, check_dualgap=1)


def new_values(d, seed):
    """Perturbed P (upper triangle) and A values of an MPC QP, in CSC order."""
    rg = np.random.default_rng(seed)
    P, A = sp.csc_matrix(d[0]), sp.csc_matrix(d[2])
    return P.data * (1.0 + 0.2 * rg.uniform(0.0, 1.0, P.nnz)), A.data * (1.0 + 0.05 * rg.uniform(-1.0, 1.0, A.nnz))


def with_values(d, px, ax):
    P, A = sp.csc_matrix(d[0]).copy(), sp.csc_matrix(d[2]).copy()
    P.data = np.asarray(px, dtype=np.float64).copy()
    A.data = np.asarray(ax, dtype=np.float64).copy()
    return (P, d[1], A, d[3], d[4])


def check(sol, xs, cur, res, obj_tol, same_iter):
    for k, (d, r) in enumerate(zip(cur, res)):
        assert sol["status"][k] == r.info["status_val"], (k, sol["status"][k], r.info["status_val"])
        if r.info["status_val"] != SOLVED:
            continue
        og = objective(d[0], d[1], xs[k].astype(np.float64))
        oo = r.info["obj_val"]
        assert abs(og - oo) / max(1.0, abs(oo)) <= obj_tol, (k, og, oo)
        if same_iter:
            assert sol["iter"][k] == r.info["iter"], (k, sol["iter"][k], r.info["iter"])


def run_sequence(prec, solver, oracle_lib, partial):
    probs = pb.mpc_batch(16, seed=21)
    b = Batch(load(prec))
    assert b.setup(probs, linsys_solver=solver, **WORKLOAD) == 0
    assert b.solve() == 0
    orc = []
    for d in probs:
        s = OSQP(oracle_lib)
        assert s.setup(*d, linsys_solver=solver, **WORKLOAD) == 0
        s.solve()
        orc.append(s)
    cur = list(probs)
    for k, d in enumerate(probs):
        if k % 4 == 3:
            continue   # some QPs keep their matrices
        px, ax = new_values(d, 100 + k)
        if partial and k % 2:
            # every third A entry and the first half of P's, by index
            ai = np.arange(0, ax.size, 3)
            pi = np.arange(0, px.size // 2)
            assert b.update_mat(k, Px=px[pi], Px_idx=pi, Ax=ax[ai], Ax_idx=ai) == 0
            assert orc[k].update(Px=px[pi], Px_idx=pi, Ax=ax[ai], Ax_idx=ai) == 0
            P0, A0 = sp.csc_matrix(d[0]).data.copy(), sp.csc_matrix(d[2]).data.copy()
            P0[pi] = px[pi]
            A0[ai] = ax[ai]
            cur[k] = with_values(d, P0, A0)
        else:
            assert b.update_mat(k, Px=px, Ax=ax) == 0
            assert orc[k].update(Px=px, Ax=ax) == 0
            cur[k] = with_values(d, px, ax)
    assert b.solve() == 0
    sol = b.solution()
    xs = b.split(sol["x"], "n")
    res = [s.solve() for s in orc]
    b.cleanup()
    return sol, xs, cur, res


@pytest.mark.parametrize("partial", [False, True])
def test_update_mat_direct_f64_follows_builtin(partial, oracle_lib):
    sol, xs, cur, res = run_sequence("f64", DIRECT_SOLVER, oracle_lib, partial)
    check(sol, xs, cur, res, 1e-7, True)


def test_update_mat_pcg_f32_eps_class(oracle_lib):
    sol, xs, cur, res = run_sequence("f32", INDIRECT_SOLVER, oracle_lib, False)
    check(sol, xs, cur, res, 1e-2, False)


def test_update_mat_rejects_bad_counts_and_indices():
    """Rejected updates leave the batch as a control batch that never saw them."""
    probs = pb.mpc_batch(3, seed=22)
    lib = load("f64")
    b, c = Batch(lib), Batch(lib)
    for x in (b, c):
        assert x.setup(probs, linsys_solver=DIRECT_SOLVER, **WORKLOAD) == 0
        assert x.solve() == 0
    px, ax = new_values(probs[1], 7)
    # a count beyond the QP's entries: 1 for P, 2 for A (the reference's codes)
    assert b.update_mat(1, Px=np.zeros(px.size + 1)) == 1
    assert b.update_mat(1, Ax=np.zeros(ax.size + 1)) == 2
    # an index outside the QP's entries, or a QP outside the batch
    assert b.update_mat(1, Ax=ax[:2], Ax_idx=np.array([0, ax.size])) != 0
    assert b.update_mat(1, Px=px[:1], Px_idx=np.array([-1])) != 0
    assert b.update_mat(3, Px=px) != 0
    assert b.solve() == 0 and c.solve() == 0
    sb, sc = b.solution(), c.solution()
    assert np.array_equal(sb["x"], sc["x"]) and np.array_equal(sb["iter"], sc["iter"])
    b.cleanup()
    c.cleanup()
