"""Pin the FP64 oracle restatement to the reference.

The oracle (oracle/osqp_oracle.c) must reproduce (a) the expected answers that
the reference's own test generators hold (tests/*/generate_problem.py) and
(b) the outputs of the reference build itself (oracle/_ref, committed as
tests/golden/ref_outputs.npz by tests/golden/make_golden.py).
"""
import numpy as np
import pytest

from osqp_gb300.api import OSQP, SOLVED, PRIMAL_INFEASIBLE, DIRECT_SOLVER, INDIRECT_SOLVER, objective
from osqp_gb300 import problems as pb
from conftest import problem_from

FIXTURE_SETTINGS = dict(rho=0.1, alpha=1.6, max_iter=2000, scaling=1, eps_abs=1e-5, eps_rel=1e-5)
PINNED = dict(rho=0.1, sigma=1e-6, alpha=1.6, scaling=10, eps_abs=1e-3, eps_rel=1e-3,
              rho_is_vec=1, check_termination=25, adaptive_rho_tolerance=5.0, max_iter=4000)


def _solve(lib, data, **st):
    s = OSQP(lib)
    P, q, A, l, u = data
    assert s.setup(P, q, A, pb.clip_inf(l, 1e30), pb.clip_inf(u, 1e30), **st) == 0
    return s.solve()


@pytest.mark.parametrize("name", ["basic_qp", "basic_qp2", "basic_lp", "unconstrained", "no_active_set"])
@pytest.mark.parametrize("polish", [0, 1])
def test_reference_test_answers(oracle_lib, ref_tests, name, polish):
    """Expected x / objective of the reference generators (tests/<name>/generate_problem.py)."""
    data = problem_from(ref_tests, name)
    r = _solve(oracle_lib, data, polishing=polish, **FIXTURE_SETTINGS)
    assert r.info["status_val"] == SOLVED
    x_exp = ref_tests[f"{name}/sols/x_test"]
    obj_exp = float(ref_tests[f"{name}/sols/obj_value_test"])
    # tests/basic_qp/test_basic_qp.cpp:37-46 compare with TESTS_TOL = 1e-4 (FP64)
    assert np.max(np.abs(r.x - x_exp)) / max(1.0, np.max(np.abs(x_exp))) < 1e-3
    assert abs(r.info["obj_val"] - obj_exp) / max(1.0, abs(obj_exp)) < 1e-3


@pytest.mark.parametrize("lin", [DIRECT_SOLVER, INDIRECT_SOLVER])
def test_primal_infeasibility_status(oracle_lib, ref_tests, lin):
    data = problem_from(ref_tests, "primal_infeasibility")
    r = _solve(oracle_lib, data, linsys_solver=lin, **FIXTURE_SETTINGS)
    assert r.info["status_val"] == PRIMAL_INFEASIBLE


@pytest.mark.parametrize("case", ["basic_qp", "basic_qp2", "basic_lp", "unconstrained", "no_active_set",
                                  "primal_infeasibility"])
@pytest.mark.parametrize("polish", [0, 1])
def test_matches_reference_build_on_reference_problems(oracle_lib, ref_tests, ref_outputs, case, polish):
    data = problem_from(ref_tests, case)
    r = _solve(oracle_lib, data, polishing=polish, **FIXTURE_SETTINGS)
    pre = f"{case}/pol{polish}"
    assert r.info["status_val"] == int(ref_outputs[pre + "/status_val"])
    assert r.info["iter"] == int(ref_outputs[pre + "/iter"])
    if r.info["status_val"] == SOLVED:
        assert np.allclose(r.x, ref_outputs[pre + "/x"], rtol=1e-7, atol=1e-9)
        assert np.allclose(r.y, ref_outputs[pre + "/y"], rtol=1e-7, atol=1e-9)


@pytest.mark.parametrize("case", ["random_qp_s1", "random_qp_s7", "mpc_s0", "mpc_s2", "portfolio_s1"])
@pytest.mark.parametrize("polish", [0, 1])
def test_matches_reference_build_on_workloads(oracle_lib, ref_outputs, case, polish):
    data = problem_from(ref_outputs, case, data_prefix=f"{case}/data")
    r = _solve(oracle_lib, data, polishing=polish, **PINNED)
    pre = f"{case}/pol{polish}"
    assert r.info["status_val"] == int(ref_outputs[pre + "/status_val"])
    assert r.info["iter"] == int(ref_outputs[pre + "/iter"])
    assert r.info["status_polish"] == int(ref_outputs[pre + "/status_polish"])
    ref_obj = float(ref_outputs[pre + "/obj_val"])
    assert abs(r.info["obj_val"] - ref_obj) <= 1e-8 * max(1.0, abs(ref_obj))
    assert np.allclose(r.x, ref_outputs[pre + "/x"], rtol=1e-6, atol=1e-8)


def test_indirect_oracle_agrees_with_direct(oracle_lib):
    """The reduced-KKT PCG path (the algorithm the GPU runs) reaches the same optimum."""
    data = pb.random_qp(3, n=120, m=240)
    rd = _solve(oracle_lib, data, linsys_solver=DIRECT_SOLVER, **dict(PINNED, eps_abs=1e-6, eps_rel=1e-6))
    ri = _solve(oracle_lib, data, linsys_solver=INDIRECT_SOLVER, **dict(PINNED, eps_abs=1e-6, eps_rel=1e-6))
    assert rd.info["status_val"] == ri.info["status_val"] == SOLVED
    assert abs(rd.info["obj_val"] - ri.info["obj_val"]) < 1e-4 * max(1.0, abs(rd.info["obj_val"]))
    P = data[0]
    assert abs(objective(P, data[1], ri.x) - ri.info["obj_val"]) < 1e-3 * max(1.0, abs(ri.info["obj_val"]))
