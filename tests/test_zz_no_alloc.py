"""The allocation-free reduced-KKT solve (osqp_gb300_linsys_solve_noalloc).

Some callers cannot allocate device memory where they solve: real-time loops
whose device memory is fixed before they start (an allocation could block or
fail mid-loop), or programs sharing a GPU under a budget granted up front.
This entry point keeps its work vectors in a fixed device array inside the
library; here it is called through the C ABI and checked against the regular
linear-system solver (a fresh LinSysSolver.solve) on the same data, on two
calls in a row (the second call sees the scratch the first one left behind),
and against an FP64 host solve of the same system (scipy), within the error
bound that the PCG's stopping tolerance implies.
"""
import ctypes as C

import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg  # noqa: F401

pytestmark = pytest.mark.gpu

TOL = {"f32": 1e-3, "f64": 1e-4}   # TESTS_TOL of the reference tests


def _bind(alg):
    fn = alg.lib.osqp_gb300_linsys_solve_noalloc
    fn.restype = alg.I
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(alg.Settings), C.c_void_p]
    return fn


@pytest.mark.parametrize("prec", ["f32", "f64"])
@pytest.mark.parametrize("vector_rho", [True, False])
@pytest.mark.parametrize("precond", [1, 2])   # diagonal, block-Jacobi
def test_noalloc_matches_linsys_solver(prec, vector_rho, precond):
    from osqp_gb300.algebra import AlgebraLib
    alg = AlgebraLib(prec)
    noalloc = _bind(alg)
    rng = np.random.default_rng(11)
    n, m = 60, 90
    M = sp.random(n, n, density=0.2, random_state=rng)
    P = (M @ M.T + 0.5 * sp.eye(n)).tocsc()
    A = sp.random(m, n, density=0.15, random_state=rng, format="csc")
    MP, MA = alg.mat(P, triu=True), alg.mat(A)
    st = alg.default_settings()
    st.rho, st.sigma = 0.1, 1e-6
    st.cg_precond = precond
    rho = alg.vec(np.where(np.arange(m) % 3 == 0, 100.0, 0.1)) if vector_rho else None
    for call in range(2):
        rhs = np.random.default_rng(100 + call).standard_normal(n + m)
        # regular entry point: a fresh solver, solve(b, admm_iter = 1)
        s = C.POINTER(alg.LinSysSolver)()
        pr, dr = alg.F(0.0), alg.F(0.0)
        assert alg.lib.osqp_algebra_init_linsys_solver(C.byref(s), MP, MA, rho, C.byref(st), C.byref(pr),
                                                       C.byref(dr), 0) == 0
        b_ref = alg.vec(rhs)
        assert s.contents.solve(s, b_ref, 1) == 0
        s.contents.free(s)
        # allocation-free entry point
        b = alg.vec(rhs)
        assert noalloc(MP, MA, rho, C.byref(st), b) == 0
        got, exp = alg.get(b), alg.get(b_ref)
        assert np.max(np.abs(got - exp)) <= TOL[prec] * max(1.0, np.max(np.abs(exp))), call
        # and it solved the system to the CG tolerance of a first ADMM iteration:
        # ||K x - rhs||_inf <= cg_tol_fraction * ||rhs||_inf (cuda_pcg_interface.cu:41-47)
        rv = np.where(np.arange(m) % 3 == 0, 100.0, 0.1) if vector_rho else np.full(m, 0.1)
        x = got[:n]
        K = (P + 1e-6 * sp.eye(n) + A.T @ sp.diags(rv) @ A)
        rhs_red = rhs[:n] + A.T @ (rv * rhs[n:])
        r = K @ x - rhs_red
        assert np.max(np.abs(r)) <= 1.05 * st.cg_tol_fraction * np.max(np.abs(rhs_red))
        # independent FP64 solve: ||x - x*||_2 <= ||K x - rhs||_2 / lambda_min(K)
        x_star = sp.linalg.spsolve(K.tocsc(), rhs_red)
        lam_min = np.linalg.eigvalsh(K.toarray())[0]
        assert np.linalg.norm(x - x_star) <= 1.01 * np.linalg.norm(r) / lam_min + TOL[prec] * np.linalg.norm(x_star)
        assert np.allclose(got[n:], A @ x, atol=TOL[prec] * max(1.0, np.max(np.abs(A @ x))))


@pytest.mark.parametrize("prec", ["f32"])
def test_noalloc_rejects_oversize(prec):
    from osqp_gb300.algebra import AlgebraLib
    alg = AlgebraLib(prec)
    noalloc = _bind(alg)
    n = 200_000                     # 8 x 800 KB of work vectors > the 4 MiB maximum
    MP = alg.mat(sp.eye(n, format="csc"), triu=True)
    MA = alg.mat(sp.csc_matrix((0, n)))
    st = alg.default_settings()
    b = alg.vec(np.ones(n))
    assert noalloc(MP, MA, None, C.byref(st), b) != 0
    assert np.all(alg.get(b) == 1.0)   # untouched
