"""The single-QP benchmark shapes against the FP64 oracle: the large sparse QP
(PCG path; reduced size against the FP64 restatement of the same PCG
algorithm, full size by status and FP64 host residuals) and the sparse SVM at
eps 1e-5 with polish (reduced size against the builtin algorithm: same
solve status, objective within 1e-6 relative; polish outcome as the
reference's CUDA-backend algorithm)."""
import numpy as np
import pytest
import scipy.sparse as sp

from osqp_gb300 import load
from osqp_gb300 import problems as pb
from osqp_gb300.api import OSQP, SOLVED, DIRECT_SOLVER, INDIRECT_SOLVER, objective

pytestmark = pytest.mark.gpu

BASE = dict(rho=0.1, sigma=1e-6, alpha=1.6, scaling=10, rho_is_vec=1, check_termination=5,
            adaptive_rho_tolerance=5.0, check_dualgap=1, warm_starting=0)


def host_residuals(d, x, y):
    P, q, A, l, u = d
    Pu = sp.csc_matrix(P)
    Pf = Pu + sp.triu(Pu, 1).T
    Ax = A @ x
    prim = np.max(np.abs(Ax - np.clip(Ax, l, u)))
    dual = np.max(np.abs(Pf @ x + q + A.T @ y))
    return prim, dual, max(np.max(np.abs(Ax)), 1e-30), max(np.max(np.abs(Pf @ x)), np.max(np.abs(A.T @ y)),
                                                          np.max(np.abs(q)))


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_large_sparse_reduced_matches_fp64_pcg(prec, oracle_lib):
    d = pb.large_sparse(seed=2, n=5000, m=10000)
    st = dict(BASE, eps_abs=1e-3, eps_rel=1e-3, max_iter=4000, linsys_solver=INDIRECT_SOLVER)
    g = OSQP(load(prec))
    assert g.setup(*d, **st) == 0
    rg = g.solve()
    o = OSQP(oracle_lib)
    assert o.setup(*d, **st) == 0
    ro = o.solve()
    assert rg.info["status_val"] == ro.info["status_val"] == SOLVED
    og = objective(d[0], d[1], rg.x.astype(np.float64))
    rel = abs(og - ro.info["obj_val"]) / max(1.0, abs(ro.info["obj_val"]))
    assert rel <= 1e-3, rel    # eps 1e-3: both stop inside the eps-class ball of the optimum
    prim, dual, sp_, sd_ = host_residuals(d, rg.x.astype(np.float64), rg.y.astype(np.float64))
    # the eps tests of auxil.c:808-945 in FP64 on the host (10 % slack for the FP32 iterates)
    assert prim <= 1.1 * (1e-3 + 1e-3 * sp_) and dual <= 1.1 * (1e-3 + 1e-3 * sd_), (prim, dual)


def test_large_sparse_full_size_status_and_residuals():
    d = pb.large_sparse()
    st = dict(BASE, eps_abs=1e-3, eps_rel=1e-3, max_iter=4000, linsys_solver=INDIRECT_SOLVER)
    g = OSQP(load("f32"))
    assert g.setup(*d, **st) == 0
    rg = g.solve()
    assert rg.info["status_val"] == SOLVED
    prim, dual, sp_, sd_ = host_residuals(d, rg.x.astype(np.float64), rg.y.astype(np.float64))
    assert prim <= 1.1 * (1e-3 + 1e-3 * sp_) and dual <= 1.1 * (1e-3 + 1e-3 * sd_), (prim, dual)


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_svm_reduced_with_polish_matches_builtin(prec, oracle_lib):
    """Same solve status as the builtin algorithm, objective within 1e-6 of
    the builtin's polished objective, eps-accurate FP64 residuals, and the
    polish outcome of the reference's CUDA-backend algorithm (the FP64 oracle
    in INDIRECT mode).  The polish reduced KKT system P + delta I +
    A_red' A_red / delta (delta = 1e-6) is solved by the reduced-KKT PCG, as
    in the CUDA backend (cuda_pcg_interface.cu:149-156); on this QP that
    solve does not reach the accuracy at which the polished point beats the
    ADMM residuals (the acceptance test of polish.c:462-473), there and here,
    while the builtin's direct LDL' does."""
    d = pb.svm(seed=5, m=4000, n=200)
    infty = 1e17 if prec == "f32" else 1e30
    P, q, A, l, u = d
    d = (P, q, A, pb.clip_inf(l, infty), pb.clip_inf(u, infty))
    st = dict(BASE, eps_abs=1e-5, eps_rel=1e-5, max_iter=20000, polishing=1)
    g = OSQP(load(prec))
    assert g.setup(*d, **dict(st, linsys_solver=INDIRECT_SOLVER)) == 0
    rg = g.solve()
    do = (P, q, A, pb.clip_inf(l, 1e30), pb.clip_inf(u, 1e30))
    o = OSQP(oracle_lib)
    assert o.setup(*do, **dict(st, linsys_solver=DIRECT_SOLVER)) == 0
    ro = o.solve()
    oi = OSQP(oracle_lib)
    assert oi.setup(*do, **dict(st, linsys_solver=INDIRECT_SOLVER)) == 0
    roi = oi.solve()
    assert rg.info["status_val"] == ro.info["status_val"] == SOLVED
    assert rg.info["status_polish"] == roi.info["status_polish"], (rg.info["status_polish"], roi.info["status_polish"])
    og = objective(P, q, rg.x.astype(np.float64))
    rel = abs(og - ro.info["obj_val"]) / max(1.0, abs(ro.info["obj_val"]))
    assert rel <= 1e-6, rel
    prim, dual, sp_, sd_ = host_residuals(do, rg.x.astype(np.float64), rg.y.astype(np.float64))
    assert prim <= 1.1 * (1e-5 + 1e-5 * sp_) and dual <= 1.1 * (1e-5 + 1e-5 * sd_), (prim, dual)
