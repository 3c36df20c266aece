"""Reference suites on the GPU, through the C ABI: primal/dual infeasibility
(tests/primal_dual_infeasibility), non-convex detection in the solve
(tests/non_cvx/test_non_cvx.cpp:48-78), the time limit
(tests/basic_qp/test_basic_qp.cpp:889-940) and device-resident inputs and
outputs (tests/basic_qp/test_cuda_io.cpp:14-195), plus the batched solver's
raw-pointer entry points against its host-array path."""
import ctypes as C

import numpy as np
import pytest
import scipy.sparse as sp

from osqp_gb300 import load
from osqp_gb300 import problems as pb
from osqp_gb300.api import OSQP, Batch, SOLVED, NON_CVX, MAX_ITER_REACHED, TIME_LIMIT_REACHED
from conftest import problem_from
from test_reference_suites import FIXTURE, PDI, PDI_CASES, pdi_problem, solve

pytestmark = pytest.mark.gpu

TESTS_TOL = {"f32": 1e-3, "f64": 1e-4}   # tests/osqp_tester.h:12-16
INF = {"f32": 1e17, "f64": 1e30}          # OSQP_INFTY of each build


@pytest.mark.parametrize("prec", ["f32", "f64"])
@pytest.mark.parametrize("case", [1, 2, 3, 4])
def test_primal_dual_infeasibility(prec, case, ref_tests):
    data, polish, expect = pdi_problem(ref_tests, case)
    rc, r = solve(load(prec), data, INF[prec], **dict(FIXTURE, polishing=polish, scaling=0))
    assert rc == 0
    assert r.info["status_val"] in expect, r.info["status"]
    if case == 1:
        tol = TESTS_TOL[prec]
        assert np.max(np.abs(r.x - ref_tests[PDI + "x1"])) < tol
        assert np.max(np.abs(r.y - ref_tests[PDI + "y1"])) < tol
        assert abs(r.info["obj_val"] - float(ref_tests[PDI + "obj_value1"])) < tol


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_nonconvex_solve(prec, ref_tests):
    """P + sigma_new I is positive definite but P is not: the iterates diverge.
    FP32 build (OSQP_INFTY 1e17): status non-convex and a NaN objective, as the
    reference asserts.  FP64 build (OSQP_INFTY 1e30): the same diverging
    trajectory as the FP64 oracle's PCG, which reaches the iteration limit
    with residuals past 1e17 (test_reference_suites.py), or non-convex."""
    data = problem_from(ref_tests, "non_cvx")
    st = dict(FIXTURE, adaptive_rho=0, sigma=float(ref_tests["non_cvx/sols/sigma_new"]))
    rc, r = solve(load(prec), data, INF[prec], **st)
    assert rc == 0
    if prec == "f32":
        assert r.info["status_val"] == NON_CVX and np.isnan(r.info["obj_val"])
    else:
        assert r.info["status_val"] in (NON_CVX, MAX_ITER_REACHED)
        if r.info["status_val"] == MAX_ITER_REACHED:
            assert r.info["prim_res"] > 1e17 and r.info["dual_res"] > 1e17


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_time_limit(prec, ref_tests):
    """No limit: the basic QP solves.  Then time_limit 1e-7 s with eps 1e-12 and
    no termination checks: the run stops on the time limit (the reference sets
    max_iter 2e9; 1e7 here keeps the run bounded should the limit not fire)."""
    data = problem_from(ref_tests, "basic_qp")
    P, q, A, l, u = data
    s = OSQP(load(prec))
    assert s.setup(P, q, A, pb.clip_inf(l, INF[prec]), pb.clip_inf(u, INF[prec]),
                   **dict(FIXTURE, rho=20.0, adaptive_rho=0)) == 0
    assert s.solve().info["status_val"] == SOLVED
    assert s.update_settings(time_limit=1e-7, eps_abs=1e-12, eps_rel=1e-12, max_iter=10_000_000,
                             check_termination=0) == 0
    s.cold_start()
    r = s.solve()
    assert r.info["status_val"] == TIME_LIMIT_REACHED
    assert r.info["iter"] < 10_000_000
    s.cleanup()


def _dev(torch, a, dtype):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dtype, device="cuda")


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_device_resident_data_and_solution(prec, ref_tests):
    """P, A, q, l, u in device memory, no solution allocated by the solver
    (allocate_solution = 0), the solution copied into device buffers by
    osqp_get_solution; x, y and the objective within TESTS_TOL of the
    generator's answers (test_cuda_io.cpp:14-195)."""
    torch = pytest.importorskip("torch")
    L = load(prec)
    fdt = torch.float32 if prec == "f32" else torch.float64
    P, q, A, l, u = problem_from(ref_tests, "basic_qp")
    Pu = sp.triu(P, format="csc")
    Pu.sort_indices()
    A = sp.csc_matrix(A)
    A.sort_indices()
    n, m = P.shape[0], A.shape[0]
    keep = {
        "Pp": _dev(torch, Pu.indptr, torch.int32), "Pi": _dev(torch, Pu.indices, torch.int32),
        "Px": _dev(torch, Pu.data, fdt), "Ap": _dev(torch, A.indptr, torch.int32),
        "Ai": _dev(torch, A.indices, torch.int32), "Ax": _dev(torch, A.data, fdt),
        "q": _dev(torch, q, fdt), "l": _dev(torch, pb.clip_inf(l, INF[prec]), fdt),
        "u": _dev(torch, pb.clip_inf(u, INF[prec]), fdt),
    }
    ptr = lambda t, T: C.cast(C.c_void_p(t.data_ptr()), C.POINTER(T))
    Pc = L.CscMatrix(n, n, ptr(keep["Pp"], L.I), ptr(keep["Pi"], L.I), ptr(keep["Px"], L.F), Pu.nnz, -1, 0)
    Ac = L.CscMatrix(m, n, ptr(keep["Ap"], L.I), ptr(keep["Ai"], L.I), ptr(keep["Ax"], L.F), A.nnz, -1, 0)
    st = L.default_settings()
    for k, v in dict(FIXTURE, verbose=0, allocate_solution=0, polishing=1, scaling=0, warm_starting=0).items():
        setattr(st, k, v)
    solver = C.POINTER(L.Solver)()
    torch.cuda.synchronize()
    assert L.lib.osqp_setup(C.byref(solver), C.byref(Pc), ptr(keep["q"], L.F), C.byref(Ac), ptr(keep["l"], L.F),
                            ptr(keep["u"], L.F), m, n, C.byref(st)) == 0
    try:
        assert not bool(solver.contents.solution)           # allocate_solution = 0
        assert L.lib.osqp_solve(solver) == 0
        info = solver.contents.info.contents
        assert info.status_val == SOLVED
        out = {k: torch.full((sz,), float("nan"), dtype=fdt, device="cuda")
               for k, sz in (("x", n), ("y", m), ("pc", m), ("dc", n))}
        sol = L.Solution(ptr(out["x"], L.F), ptr(out["y"], L.F), ptr(out["pc"], L.F), ptr(out["dc"], L.F))
        assert L.lib.osqp_get_solution(solver, C.byref(sol)) == 0
        tol = TESTS_TOL[prec]
        x, y = out["x"].cpu().double().numpy(), out["y"].cpu().double().numpy()
        assert np.max(np.abs(x - ref_tests["basic_qp/sols/x_test"])) < tol
        assert np.max(np.abs(y - ref_tests["basic_qp/sols/y_test"])) < tol
        assert abs(info.obj_val - float(ref_tests["basic_qp/sols/obj_value_test"])) < tol
    finally:
        L.lib.osqp_cleanup(solver)


def test_batch_device_pointers_match_host_arrays():
    """osqp_gb300_batch_update_data_vec / _get_solution with device addresses
    give the same bits as with host arrays."""
    torch = pytest.importorskip("torch")
    lib = load("f32")
    probs = [pb.mpc(900 + k) for k in range(4)]
    rg = np.random.default_rng(9)
    ls, us = [], []
    for (P, q, A, l, u) in probs:
        rowlen = np.diff(A.tocsr().indptr)
        nx = int(np.argmax(rowlen != 1))
        l2, u2 = pb.mpc_x0_bounds(l, u, rg.uniform(-1.0, 1.0, nx))
        ls.append(l2); us.append(u2)
    l_all = pb.clip_inf(np.concatenate(ls), 1e17).astype(np.float32)
    u_all = pb.clip_inf(np.concatenate(us), 1e17).astype(np.float32)
    st = dict(rho=0.1, sigma=1e-6, alpha=1.6, scaling=10, eps_abs=1e-3, eps_rel=1e-3, rho_is_vec=1,
              check_termination=5, adaptive_rho_tolerance=5.0, max_iter=4000)
    host, dev = Batch(lib), Batch(lib)
    assert host.setup(probs, **st) == 0 and dev.setup(probs, **st) == 0
    assert host.update(l=l_all, u=u_all) == 0 and host.solve() == 0
    x_host = host.solution()["x"]
    dl, du = _dev(torch, l_all, torch.float32), _dev(torch, u_all, torch.float32)
    torch.cuda.synchronize()
    assert dev.update_ptr(l_ptr=dl.data_ptr(), u_ptr=du.data_ptr()) == 0 and dev.solve() == 0
    x_dev = torch.zeros(x_host.size, dtype=torch.float32, device="cuda")
    assert dev.solution_ptr(x_ptr=x_dev.data_ptr()) == 0
    assert np.array_equal(x_dev.cpu().numpy(), x_host)
    host.cleanup(); dev.cleanup()


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_large_qp(prec):
    """Solved, objective within TESTS_TOL relative of 0.106081 (test_large_qp.cpp:10-37)."""
    from test_reference_suites import large_qp
    data, obj = large_qp()
    rc, r = solve(load(prec), data, INF[prec], **FIXTURE)
    assert rc == 0 and r.info["status_val"] == SOLVED
    assert abs(r.info["obj_val"] - obj) / abs(obj) < TESTS_TOL[prec]
