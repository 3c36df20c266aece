"""Block-Jacobi preconditioner (cg_precond = 2) in the FP64 oracle: the blocks
are the inverted 32 x 32 diagonal blocks of K = P + sigma I + A' R A, and a
solve with them reaches the same status and answer as the builtin (direct)
algebra.  The GPU solver's blocks and solves are checked against these in
test_block_precond_gpu.py."""
import ctypes as C

import numpy as np
import pytest
import scipy.sparse as sp

from osqp_gb300 import problems as pb
from osqp_gb300.api import OSQP, DIRECT_SOLVER, INDIRECT_SOLVER, BLOCK_DIAGONAL_PRECONDITIONER, SOLVED

SETTINGS = dict(rho=0.1, sigma=1e-6, alpha=1.6, scaling=10, eps_abs=1e-3, eps_rel=1e-3, rho_is_vec=1,
                check_termination=25, adaptive_rho_tolerance=5.0, max_iter=4000)


def oracle_blocks(oracle_lib, solver):
    f = oracle_lib.lib.oracle_block_inverse
    f.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
    f.restype = C.c_int64
    cnt = int(f(C.cast(solver._solver, C.c_void_p), None))
    out = np.zeros(cnt)
    if cnt:
        f(C.cast(solver._solver, C.c_void_p), out.ctypes.data_as(C.POINTER(C.c_double)))
    return out.reshape(-1, 32, 32)


def oracle_pcg_iters(oracle_lib, solver):
    f = oracle_lib.lib.oracle_last_pcg_iters
    f.argtypes = [C.c_void_p]
    f.restype = C.c_int64
    return int(f(C.cast(solver._solver, C.c_void_p)))


def kkt_blocks(P, A, sigma, rho):
    """Inverted 32 x 32 diagonal blocks of P + sigma I + rho A'A (numpy, FP64)."""
    n = P.shape[0]
    Pf = sp.triu(P, format="csc")
    Pf = (Pf + sp.triu(Pf, 1).T).toarray()
    K = Pf + sigma * np.eye(n) + rho * (A.T @ A).toarray()
    nb = (n + 31) // 32
    out = np.zeros((nb, 32, 32))
    for b in range(nb):
        i0, i1 = 32 * b, min(n, 32 * b + 32)
        out[b, : i1 - i0, : i1 - i0] = np.linalg.inv(K[i0:i1, i0:i1])
    return out


@pytest.mark.parametrize("n,m", [(70, 140), (64, 100), (20, 30)])
def test_oracle_blocks_are_inverse_kkt_blocks(oracle_lib, n, m):
    """Unscaled data and a scalar rho: the blocks equal numpy's inverses (the
    last block short when 32 does not divide n)."""
    P, q, A, l, u = pb.random_qp(3, n=n, m=m)
    s = OSQP(oracle_lib)
    assert s.setup(P, q, A, l, u, linsys_solver=INDIRECT_SOLVER, cg_precond=BLOCK_DIAGONAL_PRECONDITIONER,
                   **dict(SETTINGS, scaling=0, rho_is_vec=0)) == 0
    got = oracle_blocks(oracle_lib, s)
    want = kkt_blocks(P, A, 1e-6, 0.1)
    assert got.shape == want.shape
    for b in range(got.shape[0]):
        scale = np.max(np.abs(want[b]))
        assert np.max(np.abs(got[b] - want[b])) <= 1e-9 * scale, b


def _solve(oracle_lib, d, **st):
    s = OSQP(oracle_lib)
    assert s.setup(*d, **dict(SETTINGS, **st)) == 0
    r = s.solve()
    return r, oracle_pcg_iters(oracle_lib, s)


CASES = {
    "random_qp_s1": lambda: pb.random_qp(1, n=100, m=200),
    "random_qp_s7": lambda: pb.random_qp(7, n=60, m=120),
    "mpc_s1": lambda: pb.mpc(1),
}


@pytest.mark.parametrize("case", sorted(CASES))
def test_oracle_block_mode_solves_like_direct(oracle_lib, case):
    """Same status as the builtin (direct) algebra, objective within the
    eps = 1e-3 accuracy class of it."""
    d = CASES[case]()
    rd, _ = _solve(oracle_lib, d, linsys_solver=DIRECT_SOLVER)
    rb, it_b = _solve(oracle_lib, d, linsys_solver=INDIRECT_SOLVER, cg_precond=BLOCK_DIAGONAL_PRECONDITIONER)
    assert rb.info["status_val"] == rd.info["status_val"] == SOLVED
    assert it_b > 0
    scale = max(1.0, abs(rd.info["obj_val"]))
    assert abs(rb.info["obj_val"] - rd.info["obj_val"]) <= 1e-3 * scale


@pytest.mark.parametrize("case", sorted(CASES))
def test_oracle_block_mode_needs_fewer_pcg_iterations(oracle_lib, case):
    """Fewer PCG iterations per ADMM iteration than the diagonal preconditioner."""
    d = CASES[case]()
    rj, it_j = _solve(oracle_lib, d, linsys_solver=INDIRECT_SOLVER)
    rb, it_b = _solve(oracle_lib, d, linsys_solver=INDIRECT_SOLVER, cg_precond=BLOCK_DIAGONAL_PRECONDITIONER)
    assert it_b / rb.info["iter"] < it_j / rj.info["iter"]


def test_oracle_switch_to_block_mode_by_settings_update(oracle_lib):
    d = pb.random_qp(7, n=60, m=120)
    s = OSQP(oracle_lib)
    assert s.setup(*d, linsys_solver=INDIRECT_SOLVER, **SETTINGS) == 0
    assert oracle_blocks(oracle_lib, s).size == 0
    assert s.update_settings(cg_precond=BLOCK_DIAGONAL_PRECONDITIONER) == 0
    assert oracle_blocks(oracle_lib, s).shape == (2, 32, 32)
    assert s.solve().info["status_val"] == SOLVED
