"""Reference suites restated against the FP64 oracle (CPU): the four cases of
tests/primal_dual_infeasibility/test_primal_dual_infeasibility.cpp and the
non-convex detection of tests/non_cvx/test_non_cvx.cpp, on the generators'
data (tests/golden/ref_tests.npz).  The GPU runs the same cases in
test_reference_suites_gpu.py."""
import numpy as np
import pytest

from osqp_gb300 import problems as pb
from osqp_gb300.api import (OSQP, SOLVED, PRIMAL_INFEASIBLE, DUAL_INFEASIBLE, NON_CVX, MAX_ITER_REACHED,
                            DIRECT_SOLVER, INDIRECT_SOLVER)
from conftest import csc_from, problem_from

# OSQPTestFixture settings (tests/osqp_tester.h:60-80)
FIXTURE = dict(rho=0.1, alpha=1.6, max_iter=2000, scaling=1, eps_abs=1e-5, eps_rel=1e-5)
TESTS_TOL = 1e-4          # FP64 (tests/osqp_tester.h:12-16)
NONCVX_ERROR = 4          # OSQP_NONCVX_ERROR (osqp_api_constants.h, osqp_error_type)
PDI = "primal_dual_infeasibility/data/"
# case -> (A, u, polishing, expected statuses) (test_primal_dual_infeasibility.cpp:11-135)
PDI_CASES = {1: ("A12", "u1", 1, (SOLVED,)), 2: ("A12", "u2", 0, (PRIMAL_INFEASIBLE,)),
             3: ("A34", "u3", 0, (DUAL_INFEASIBLE,)), 4: ("A34", "u4", 0, (PRIMAL_INFEASIBLE, DUAL_INFEASIBLE))}


def pdi_problem(ref_tests, case):
    a, u, polish, expect = PDI_CASES[case]
    data = (csc_from(ref_tests, PDI + "P"), np.asarray(ref_tests[PDI + "q"]), csc_from(ref_tests, PDI + a),
            np.asarray(ref_tests[PDI + "l"]), np.asarray(ref_tests[PDI + u]))
    return data, polish, expect


def solve(lib, data, inf, **st):
    P, q, A, l, u = data
    s = OSQP(lib)
    rc = s.setup(P, q, A, pb.clip_inf(l, inf), pb.clip_inf(u, inf), **st)
    return rc, (s.solve() if rc == 0 else None)


@pytest.mark.parametrize("lin", [DIRECT_SOLVER, INDIRECT_SOLVER])
@pytest.mark.parametrize("case", [1, 2, 3, 4])
def test_primal_dual_infeasibility(oracle_lib, ref_tests, lin, case):
    data, polish, expect = pdi_problem(ref_tests, case)
    rc, r = solve(oracle_lib, data, 1e30, linsys_solver=lin, **dict(FIXTURE, polishing=polish, scaling=0))
    assert rc == 0
    assert r.info["status_val"] in expect
    if case == 1:
        assert np.max(np.abs(r.x - ref_tests[PDI + "x1"])) < TESTS_TOL
        assert np.max(np.abs(r.y - ref_tests[PDI + "y1"])) < TESTS_TOL
        assert abs(r.info["obj_val"] - float(ref_tests[PDI + "obj_value1"])) < TESTS_TOL


def test_nonconvex_setup_detection(oracle_lib, ref_tests):
    """Direct solver: (P + sigma I) with a negative eigenvalue fails at set-up;
    with sigma_new it does not (test_non_cvx.cpp:10-45)."""
    data = problem_from(ref_tests, "non_cvx")
    st = dict(FIXTURE, adaptive_rho=0, linsys_solver=DIRECT_SOLVER)
    rc, _ = solve(oracle_lib, data, 1e30, **dict(st, sigma=1e-6))
    assert rc == NONCVX_ERROR
    rc, _ = solve(oracle_lib, data, 1e30, **dict(st, sigma=float(ref_tests["non_cvx/sols/sigma_new"])))
    assert rc == 0


def test_nonconvex_solve(oracle_lib, ref_tests):
    """Solve with sigma_new: status non-convex, objective NaN (test_non_cvx.cpp:48-78).
    The same PCG algorithm in FP64 diverges too, but with OSQP_INFTY = 1e30
    its residuals (2.8e18 at 2000 iterations) stay below the divergence test."""
    data = problem_from(ref_tests, "non_cvx")
    st = dict(FIXTURE, adaptive_rho=0, sigma=float(ref_tests["non_cvx/sols/sigma_new"]))
    _, rd = solve(oracle_lib, data, 1e30, linsys_solver=DIRECT_SOLVER, **st)
    assert rd.info["status_val"] == NON_CVX and np.isnan(rd.info["obj_val"])
    _, ri = solve(oracle_lib, data, 1e30, linsys_solver=INDIRECT_SOLVER, **st)
    assert ri.info["status_val"] == MAX_ITER_REACHED
    assert ri.info["prim_res"] > 1e17 and ri.info["dual_res"] > 1e17


def large_qp():
    """tests/large_qp/large_qp_data.c (prob1, n = 160, m = 270), read as text by
    tests/golden/make_large_qp.py."""
    import os
    import scipy.sparse as sp
    d = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "large_qp.npz"))
    n, m = int(d["n"]), int(d["m"])
    P = sp.csc_matrix((d["P_csc_x"], d["P_csc_i"], d["P_csc_p"]), shape=(n, n))
    A = sp.csc_matrix((d["A_csc_x"], d["A_csc_i"], d["A_csc_p"]), shape=(m, n))
    return (P, d["q_val"], A, d["l_val"], d["u_val"]), float(d["obj_val"])


@pytest.mark.parametrize("lin", [DIRECT_SOLVER, INDIRECT_SOLVER])
def test_large_qp(oracle_lib, lin):
    """Solved, objective within TESTS_TOL relative of 0.106081 (test_large_qp.cpp:10-37)."""
    data, obj = large_qp()
    rc, r = solve(oracle_lib, data, 1e30, linsys_solver=lin, **FIXTURE)
    assert rc == 0 and r.info["status_val"] == SOLVED
    assert abs(r.info["obj_val"] - obj) / abs(obj) < TESTS_TOL


UPD = "update_matrices/data/test_solve_"
# section -> (update P, update A, index vectors, counts of 0 = "all", expected answers)
# (tests/update_matrices/test_update_matrices.cpp:94-383)
UPDATE_SECTIONS = {
    "P_idx": (True, False, True, False, "P_new"), "P_all": (True, False, False, False, "P_new"),
    "P_nnz0": (True, False, False, True, "P_new"), "A_idx": (False, True, True, False, "A_new"),
    "A_all": (False, True, False, False, "A_new"), "A_nnz0": (False, True, False, True, "A_new"),
    "PA_idx": (True, True, True, False, "P_A_new"), "PA_all": (True, True, False, False, "P_A_new"),
    "PA_nnz0": (True, True, False, True, "P_A_new"),
}


def update_matrices(s, Px, Px_idx, pn, Ax, Ax_idx, an):
    """osqp_update_data_mat with explicit counts (0 with values = all entries)."""
    import ctypes as C
    L = s.L
    arr = lambda a, dt, T: None if a is None else np.ascontiguousarray(a, dtype=dt).ctypes.data_as(C.POINTER(T))
    keep = [None if a is None else np.ascontiguousarray(a) for a in (Px, Px_idx, Ax, Ax_idx)]
    rc = L.lib.osqp_update_data_mat(s._solver, arr(Px, L.np_float, L.F), arr(Px_idx, np.int32, L.I), pn,
                                    arr(Ax, L.np_float, L.F), arr(Ax_idx, np.int32, L.I), an)
    del keep
    return int(rc)


def run_update_section(lib, ref_tests, section, inf, tol, **extra):
    upd_p, upd_a, with_idx, zero, ans = UPDATE_SECTIONS[section]
    Pu, A = csc_from(ref_tests, UPD + "Pu"), csc_from(ref_tests, UPD + "A")
    q, l, u = (np.asarray(ref_tests[UPD + k]) for k in ("q", "l", "u"))
    s = OSQP(lib)
    assert s.setup(Pu, q, A, pb.clip_inf(l, inf), pb.clip_inf(u, inf), **dict(FIXTURE, max_iter=1000, **extra)) == 0
    r = s.solve()
    assert r.info["status_val"] == SOLVED
    assert np.max(np.abs(r.x - ref_tests[UPD + "x"])) < tol
    assert np.max(np.abs(r.y - ref_tests[UPD + "y"])) < tol
    Pn, An = csc_from(ref_tests, UPD + "Pu_new"), csc_from(ref_tests, UPD + "A_new")
    nP, nA = Pn.nnz, A.nnz
    args = [None, None, 0, None, None, 0]
    if upd_p:
        args[0:3] = [Pn.data, np.arange(nP) if with_idx else None, 0 if zero else nP]
    if upd_a:
        args[3:6] = [An.data, np.arange(nA) if with_idx else None, 0 if zero else nA]
    assert update_matrices(s, *args) == 0
    r = s.solve()
    assert r.info["status_val"] == SOLVED
    assert np.max(np.abs(r.x - ref_tests[UPD + ans + "_x"])) < tol
    assert np.max(np.abs(r.y - ref_tests[UPD + ans + "_y"])) < tol


@pytest.mark.parametrize("lin", [DIRECT_SOLVER, INDIRECT_SOLVER])
@pytest.mark.parametrize("section", sorted(UPDATE_SECTIONS))
def test_update_matrices(oracle_lib, ref_tests, lin, section):
    run_update_section(oracle_lib, ref_tests, section, 1e30, TESTS_TOL, linsys_solver=lin)


# ---- tests/basic_qp/test_basic_qp.cpp and tests/basic_qp2/test_basic_qp2.cpp ----
DATA_VALIDATION_ERROR = 1   # OSQP_DATA_VALIDATION_ERROR (osqp_api_constants.h, osqp_error_type)


def _basic(ref_tests, name="basic_qp"):
    return problem_from(ref_tests, name)


def _close_rel(v, ref, tol):
    return np.max(np.abs(v - ref)) / max(np.max(np.abs(ref)), 1e-12) < tol


@pytest.mark.parametrize("lin", [DIRECT_SOLVER, INDIRECT_SOLVER])
def test_basic_qp_termination(oracle_lib, ref_tests, lin):
    """check_termination = 0: the loop runs max_iter iterations and the final
    check still finds the solution (test_basic_qp.cpp:718-775)."""
    data = _basic(ref_tests)
    st = dict(max_iter=400, alpha=1.6, polishing=0, scaling=0, check_termination=0, warm_starting=0)
    rc, r = solve(oracle_lib, data, 1e30, linsys_solver=lin, **st)
    assert rc == 0 and r.info["iter"] == 400 and r.info["status_val"] == SOLVED
    assert np.max(np.abs(r.x - ref_tests["basic_qp/sols/x_test"])) < TESTS_TOL
    assert np.max(np.abs(r.y - ref_tests["basic_qp/sols/y_test"])) < TESTS_TOL
    assert abs(r.info["obj_val"] - float(ref_tests["basic_qp/sols/obj_value_test"])) < TESTS_TOL


def test_basic_qp_update_validation(oracle_lib, ref_tests):
    """Flipped bounds are refused and leave the problem as it was
    (test_basic_qp.cpp:608-716)."""
    P, q, A, l, u = _basic(ref_tests)
    s = OSQP(oracle_lib)
    assert s.setup(P, q, A, pb.clip_inf(l, 1e30), pb.clip_inf(u, 1e30),
                   **dict(FIXTURE, max_iter=200, polishing=1, scaling=0, warm_starting=0)) == 0
    u_new, l_new = ref_tests["basic_qp/sols/u_new"], ref_tests["basic_qp/sols/l_new"]
    assert s.update(l=pb.clip_inf(u_new, 1e30), u=pb.clip_inf(l_new, 1e30)) == DATA_VALIDATION_ERROR
    assert s.update(l=pb.clip_inf(u_new, 1e30)) == DATA_VALIDATION_ERROR
    r = s.solve()
    assert r.info["status_val"] == SOLVED
    assert np.max(np.abs(r.x - ref_tests["basic_qp/sols/x_test"])) < TESTS_TOL


@pytest.mark.parametrize("lin", [DIRECT_SOLVER, INDIRECT_SOLVER])
def test_basic_qp_update_rho(oracle_lib, ref_tests, lin):
    """A solver set up with rho 0.7 and one set up with 0.1 then updated to 0.7
    take the same iterations to the same answer (test_basic_qp.cpp:776-888)."""
    data = _basic(ref_tests)
    st = dict(adaptive_rho=0, eps_abs=5e-5, eps_rel=5e-5, check_termination=1, linsys_solver=lin)
    rc, r1 = solve(oracle_lib, data, 1e30, rho=0.7, **st)
    P, q, A, l, u = data
    s = OSQP(oracle_lib)
    assert s.setup(P, q, A, pb.clip_inf(l, 1e30), pb.clip_inf(u, 1e30), rho=0.1, **st) == 0
    assert s.update_rho(0.7) == 0
    r2 = s.solve()
    for r in (r1, r2):
        assert r.info["status_val"] == SOLVED
        assert _close_rel(r.x, ref_tests["basic_qp/sols/x_test"], TESTS_TOL)
        assert _close_rel(r.y, ref_tests["basic_qp/sols/y_test"], TESTS_TOL)
    assert r1.info["iter"] == r2.info["iter"]


def test_basic_qp_warm_start(oracle_lib, ref_tests):
    """Warm start from zero repeats the cold iteration count; from the
    solution the solve takes one iteration (test_basic_qp.cpp:945-993)."""
    P, q, A, l, u = _basic(ref_tests)
    s = OSQP(oracle_lib)
    assert s.setup(P, q, A, pb.clip_inf(l, 1e30), pb.clip_inf(u, 1e30),
                   **dict(FIXTURE, check_termination=1, adaptive_rho=0)) == 0
    it = s.solve().info["iter"]
    assert s.warm_start(x=np.zeros(2), y=np.zeros(4)) == 0
    assert s.solve().info["iter"] == it
    assert s.warm_start(x=np.array([0.3, 0.7])) == 0
    assert s.warm_start(y=np.array([-2.9, 0.0, 0.2, 0.0])) == 0
    assert s.solve().info["iter"] == 1


@pytest.mark.parametrize("lin", [DIRECT_SOLVER, INDIRECT_SOLVER])
def test_basic_qp2_update_vectors(oracle_lib, ref_tests, lin):
    """New q and u, warm-started and polished (test_basic_qp2.cpp:74-140)."""
    P, q, A, l, u = _basic(ref_tests, "basic_qp2")
    s = OSQP(oracle_lib)
    assert s.setup(P, q, A, pb.clip_inf(l, 1e30), pb.clip_inf(u, 1e30), linsys_solver=lin,
                   warm_starting=1, polishing=1) == 0
    assert s.update(q=ref_tests["basic_qp2/sols/q_new"]) == 0
    assert s.update(u=pb.clip_inf(ref_tests["basic_qp2/sols/u_new"], 1e30)) == 0
    r = s.solve()
    assert r.info["status_val"] == SOLVED and r.info["status_polish"] == 1
    assert _close_rel(r.x, ref_tests["basic_qp2/sols/x_test_new"], TESTS_TOL)
    assert _close_rel(r.y, ref_tests["basic_qp2/sols/y_test_new"], TESTS_TOL)
    obj = float(ref_tests["basic_qp2/sols/obj_value_test_new"])
    assert abs(r.info["obj_val"] - obj) / abs(obj) < TESTS_TOL
