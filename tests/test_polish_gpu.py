"""Solution polishing on the GPU (src/polish.c restated in osqp_gb300/csrc/polish.cu).

Bar: the polish outcome (status_polish) of the reference build on the same
problem, and a polished objective within 1e-6 (FP64 build) / 1e-5 (FP32
build: the polished x is rounded to float) relative of the reference build's
polished objective (tests/golden/ref_outputs.npz, builtin QDLDL, FP64).
"""
import numpy as np
import pytest

from osqp_gb300 import load
from osqp_gb300 import problems as pb
from osqp_gb300.api import OSQP, SOLVED, objective
from conftest import problem_from

pytestmark = pytest.mark.gpu

# tests/basic_qp*/test_*.cpp run with eps 1e-5 (FIXTURE settings of the golden file)
FIXTURE = dict(rho=0.1, alpha=1.6, max_iter=2000, scaling=1, eps_abs=1e-5, eps_rel=1e-5, rho_is_vec=1,
               check_termination=5, adaptive_rho_tolerance=5.0, polishing=1)
PINNED = dict(rho=0.1, sigma=1e-6, alpha=1.6, scaling=10, eps_abs=1e-3, eps_rel=1e-3,
              rho_is_vec=1, check_termination=25, adaptive_rho_tolerance=5.0, max_iter=4000, polishing=1)
OBJ_TOL = {"f64": 1e-6, "f32": 1e-5}
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


@pytest.mark.parametrize("prec", ["f64", "f32"])
@pytest.mark.parametrize("case", ["random_qp_s1", "random_qp_s7", "mpc_s0", "portfolio_s1"])
def test_polish_workloads(prec, case, ref_outputs):
    data = problem_from(ref_outputs, case, data_prefix=f"{case}/data")
    r = _solve(prec, data, **PINNED)
    pre = f"{case}/pol1"
    assert r.info["status_val"] == int(ref_outputs[pre + "/status_val"]) == SOLVED
    assert r.info["status_polish"] == int(ref_outputs[pre + "/status_polish"])
    ref_obj = float(ref_outputs[pre + "/obj_val"])
    obj = objective(data[0], data[1], r.x.astype(np.float64))
    assert abs(obj - ref_obj) <= OBJ_TOL[prec] * max(1.0, abs(ref_obj)), (obj, ref_obj)
    assert abs(r.info["obj_val"] - ref_obj) <= 10 * OBJ_TOL[prec] * max(1.0, abs(ref_obj))


def test_polish_off_leaves_status_not_performed():
    data = pb.random_qp(5, n=60, m=120)
    r = _solve("f32", data, **dict(PINNED, polishing=0))
    assert r.info["status_polish"] == 0
