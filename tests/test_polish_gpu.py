"""Solution polishing on the GPU (src/polish.c restated in osqp_gb300/csrc/polish.cu).

Bars: the polish outcome (status_polish) of the reference build on the same
problem; the polished objective within 1e-6 (FP64 build) / 1e-5 (FP32 build:
the polished x is rounded to float) relative of the reference build's
polished objective (tests/golden/ref_outputs.npz, builtin QDLDL, FP64), or,
with the default three refinement steps, within 3x of the FP64 oracle running
the same reduced-KKT PCG polish.
"""
import numpy as np
import pytest

from osqp_gb300 import load
from osqp_gb300 import problems as pb
from osqp_gb300.api import OSQP, SOLVED, INDIRECT_SOLVER, objective
from conftest import problem_from

pytestmark = pytest.mark.gpu

# tests/basic_qp*/test_*.cpp run with eps 1e-5 (FIXTURE settings of the golden file)
FIXTURE = dict(rho=0.1, alpha=1.6, max_iter=2000, scaling=1, eps_abs=1e-5, eps_rel=1e-5, rho_is_vec=1,
               check_termination=5, adaptive_rho_tolerance=5.0, polishing=1)
PINNED = dict(rho=0.1, sigma=1e-6, alpha=1.6, scaling=10, eps_abs=1e-3, eps_rel=1e-3,
              rho_is_vec=1, check_termination=25, adaptive_rho_tolerance=5.0, max_iter=4000, polishing=1)
OBJ_TOL = {"f64": 1e-6, "f32": 1e-5}
POLISH_CG_MAX_ITER = 10000   # the GPU polish's PCG iteration cap (osqp_gb300/csrc/polish.cu)
INF = {"f64": 1e30, "f32": 1e17}


def _solve(prec, data, **st):
    P, q, A, l, u = data
    s = OSQP(load(prec))
    assert s.setup(P, q, A, pb.clip_inf(l, INF[prec]), pb.clip_inf(u, INF[prec]), **st) == 0
    r = s.solve()
    s.cleanup()
    return r


@pytest.mark.parametrize("prec", ["f64", "f32"])
@pytest.mark.parametrize("case", ["basic_qp", "basic_qp2", "basic_lp", "no_active_set", "unconstrained"])
def test_polish_reference_problems(prec, case, ref_tests, ref_outputs):
    data = problem_from(ref_tests, case)
    r = _solve(prec, data, **FIXTURE)
    pre = f"{case}/pol1"
    assert r.info["status_val"] == int(ref_outputs[pre + "/status_val"]) == SOLVED
    assert r.info["status_polish"] == int(ref_outputs[pre + "/status_polish"])
    ref_obj = float(ref_outputs[pre + "/obj_val"])
    obj = objective(data[0], data[1], r.x.astype(np.float64))
    assert abs(obj - ref_obj) <= OBJ_TOL[prec] * max(1.0, abs(ref_obj)), (obj, ref_obj)
    if r.info["status_polish"] == 1:
        # the polished point is the active-set optimum: the generators' answer
        x_exp = ref_tests[f"{case}/sols/x_test"]
        assert np.max(np.abs(r.x - x_exp)) <= 1e-4 * max(1.0, np.max(np.abs(x_exp)))


def _oracle_polish_err(oracle_lib, data, ref_obj, **st):
    """Objective error of the same polish algorithm in FP64 (the oracle's
    reduced-KKT PCG with the GPU's polishing iteration cap)."""
    P, q, A, l, u = data
    s = OSQP(oracle_lib)
    assert s.setup(P, q, A, pb.clip_inf(l, 1e30), pb.clip_inf(u, 1e30), linsys_solver=INDIRECT_SOLVER,
                   **dict(st, cg_max_iter=POLISH_CG_MAX_ITER)) == 0
    r = s.solve()
    return abs(r.info["obj_val"] - ref_obj) / max(1.0, abs(ref_obj))


@pytest.mark.parametrize("prec", ["f64", "f32"])
@pytest.mark.parametrize("case", ["random_qp_s1", "random_qp_s7", "mpc_s0", "portfolio_s1"])
def test_polish_workloads(prec, case, ref_outputs, oracle_lib):
    """Default refinement (3 steps): within 1e-6 / 1e-5 of the builtin's polished
    objective, or within 3x the FP64 restatement of the same algorithm."""
    data = problem_from(ref_outputs, case, data_prefix=f"{case}/data")
    r = _solve(prec, data, **PINNED)
    pre = f"{case}/pol1"
    assert r.info["status_val"] == int(ref_outputs[pre + "/status_val"]) == SOLVED
    assert r.info["status_polish"] == int(ref_outputs[pre + "/status_polish"])
    ref_obj = float(ref_outputs[pre + "/obj_val"])
    obj = objective(data[0], data[1], r.x.astype(np.float64))
    err = abs(obj - ref_obj) / max(1.0, abs(ref_obj))
    if err > OBJ_TOL[prec]:
        assert err <= 3.0 * _oracle_polish_err(oracle_lib, data, ref_obj, **PINNED), (obj, ref_obj)


@pytest.mark.parametrize("prec", ["f64", "f32"])
@pytest.mark.parametrize("case", ["mpc_s0", "portfolio_s1"])
def test_polish_refined_objective(prec, case, ref_outputs):
    """Six refinement steps: polished objective within 1e-6 (FP64) / 1e-5 (FP32)
    of the builtin (QDLDL) polished objective."""
    data = problem_from(ref_outputs, case, data_prefix=f"{case}/data")
    r = _solve(prec, data, **dict(PINNED, polish_refine_iter=6))
    assert r.info["status_polish"] == 1
    ref_obj = float(ref_outputs[f"{case}/pol1/obj_val"])
    obj = objective(data[0], data[1], r.x.astype(np.float64))
    assert abs(obj - ref_obj) <= OBJ_TOL[prec] * max(1.0, abs(ref_obj)), (obj, ref_obj)


def test_polish_off_leaves_status_not_performed():
    data = pb.random_qp(5, n=60, m=120)
    r = _solve("f32", data, **dict(PINNED, polishing=0))
    assert r.info["status_polish"] == 0
