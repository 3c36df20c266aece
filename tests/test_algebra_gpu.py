"""Conformance of the algebra / linear-system ABI (libosqp_gb300_algebra*.so)
with the reference's own lin_alg and solve_linsys tests
(tests/lin_alg/testcases/*.cpp, tests/lin_alg/test_mat_vec.cpp,
tests/lin_alg/test_matrix.cpp, tests/solve_linsys/test_solve_linsys.h), on
the data of their generators (tests/lin_alg/generate_problem.py)."""
import ctypes as C

import numpy as np
import pytest
import scipy.sparse as sp


pytestmark = pytest.mark.gpu

TOL = {"f32": 1e-3, "f64": 1e-4}   # TESTS_TOL, tests/osqp_tester.h:12-16


@pytest.fixture(scope="module", params=["f32", "f64"])
def alg(request):
    from osqp_gb300.algebra import AlgebraLib
    return AlgebraLib(request.param)


@pytest.fixture(scope="module")
def la(ref_tests):
    pre = "lin_alg/data/"
    return {k[len(pre):]: ref_tests[k] for k in ref_tests.files if k.startswith(pre)}


def close(a, b, tol):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return np.max(np.abs(a - b)) <= tol * max(1.0, np.max(np.abs(b))) if b.size else a.size == 0


def test_vector_ops(alg, la):
    L, t = alg.lib, TOL[alg.precision]
    v1, v2, v3 = alg.vec(la["test_vec_ops_v1"]), alg.vec(la["test_vec_ops_v2"]), alg.vec(la["test_vec_ops_v3"])
    sc1, sc2, sc3 = float(la["test_vec_ops_sc1"]), float(la["test_vec_ops_sc2"]), float(la["test_vec_ops_sc3"])
    n = int(la["test_vec_ops_n"])
    assert abs(L.OSQPVectorf_norm_1(v1) - la["test_vec_ops_norm_1"]) < t
    assert abs(L.OSQPVectorf_norm_2(v1) - la["test_vec_ops_norm_2"]) < t
    assert abs(L.OSQPVectorf_norm_inf(v1) - la["test_vec_ops_norm_inf"]) < t
    assert abs(L.OSQPVectorf_scaled_norm_inf(v2, v1) - la["test_vec_ops_norm_inf_scaled"]) < t
    assert abs(L.OSQPVectorf_norm_inf_diff(v1, v2) - la["test_vec_ops_norm_inf_diff"]) < t
    assert abs(L.OSQPVectorf_dot_prod(v1, v2) - la["test_vec_ops_vec_dot"]) < t
    assert abs(L.OSQPVectorf_dot_prod_signed(v1, v2, 1) - la["test_vec_ops_vec_dot_pos"]) < t
    assert abs(L.OSQPVectorf_dot_prod_signed(v1, v2, -1) - la["test_vec_ops_vec_dot_neg"]) < t
    r = L.OSQPVectorf_malloc(n)
    L.OSQPVectorf_add_scaled(r, sc1, v1, sc2, v2)
    assert close(alg.get(r), la["test_vec_ops_add_scaled"], t)
    L.OSQPVectorf_add_scaled3(r, sc1, v1, sc2, v2, sc3, v3)
    assert close(alg.get(r), la["test_vec_ops_add_scaled3"], t)
    L.OSQPVectorf_plus(r, v1, v2)
    assert close(alg.get(r), la["test_vec_ops_add"], t)
    L.OSQPVectorf_minus(r, v1, v2)
    assert close(alg.get(r), la["test_vec_ops_sub"], t)
    L.OSQPVectorf_ew_prod(r, v1, v2)
    assert close(alg.get(r), la["test_vec_ops_ew_prod"], t)
    L.OSQPVectorf_ew_bound_vec(r, v1, v3, v2)   # min(v2, max(v1, v3))
    assert close(alg.get(r), la["test_vec_ops_ew_bound_vec"], t)
    L.OSQPVectorf_ew_max_vec(r, v1, v2)
    assert close(alg.get(r), la["test_vec_ops_ew_max_vec"], t)
    L.OSQPVectorf_ew_min_vec(r, v1, v2)
    assert close(alg.get(r), la["test_vec_ops_ew_min_vec"], t)
    L.OSQPVectorf_ew_reciprocal(r, v1)
    assert close(alg.get(r), la["test_vec_ops_ew_reciprocal"], t)
    s1 = alg.vec(la["test_vec_ops_shift_v1"])
    L.OSQPVectorf_ew_sqrt(s1)
    assert close(alg.get(s1), la["test_vec_ops_ew_sqrt"], t)
    L.OSQPVectorf_set_scalar_if_lt(r, v1, sc1, sc2)
    assert close(alg.get(r), la["test_vec_ops_sca_lt"], t)
    L.OSQPVectorf_set_scalar_if_gt(r, v1, sc1, sc2)
    assert close(alg.get(r), la["test_vec_ops_sca_gt"], t)
    cond = alg.ivec(la["test_vec_ops_sca_cond"])
    L.OSQPVectorf_set_scalar_conditional(r, cond, sc1, sc2, sc3)
    exp = np.where(la["test_vec_ops_sca_cond"] < 0, sc1, np.where(la["test_vec_ops_sca_cond"] == 0, sc2, sc3))
    assert close(alg.get(r), exp, t)
    c = L.OSQPVectorf_copy_new(v1)
    L.OSQPVectorf_mult_scalar(c, sc1)
    assert close(alg.get(c), la["test_vec_ops_sca_prod"], t)
    assert L.OSQPVectorf_is_eq(v1, v1, 1e-12) == 1 and L.OSQPVectorf_is_eq(v1, v2, 1e-12) == 0
    # views and concatenation
    view = L.OSQPVectorf_view(v1, 2, 5)
    assert close(alg.get(view), la["test_vec_ops_v1"][2:7], 1e-7)
    L.OSQPVectorf_view_free(view)
    cat = L.OSQPVectorf_concat(v1, v2)
    assert close(alg.get(cat), np.concatenate([la["test_vec_ops_v1"], la["test_vec_ops_v2"]]), 1e-7)
    sub = L.OSQPVectorf_subvector_byrows(v1, alg.ivec(la["test_vec_subvec_ind5"]))
    assert close(alg.get(sub), la["test_vec_subvec_5"], 1e-7)
    for h in (r, c, s1, cat, sub, v1, v2, v3):
        L.OSQPVectorf_free(h)


def test_vector_cones_and_bounds(alg):
    L = alg.lib
    l = np.array([-1e30, -1.0, 0.0, -1e30, 2.0])
    u = np.array([1e30, 1e30, 0.0, 3.0, 2.0])
    y = np.array([0.5, -2.0, 4.0, 1.5, -0.5])
    inf = 1e25 if alg.precision == "f64" else 1e13
    vl, vu, vy = alg.vec(l), alg.vec(u), alg.vec(y)
    L.OSQPVectorf_project_polar_reccone(vy, vl, vu, inf)
    assert np.allclose(alg.get(vy), [0.0, -2.0, 4.0, 1.5, -0.5])
    assert L.OSQPVectorf_all_leq(vl, vu) == 1 and L.OSQPVectorf_all_leq(vu, vl) == 0
    t = L.OSQPVectori_calloc(5)
    changed = L.OSQPVectorf_ew_bounds_type(t, vl, vu, 1e-4, inf)
    types = np.zeros(5, np.int32)
    L.OSQPVectori_to_raw(types.ctypes.data_as(C.POINTER(alg.I)), t)
    assert changed == 1 and list(types) == [-1, 0, 1, 0, 1]
    assert L.OSQPVectorf_ew_bounds_type(t, vl, vu, 1e-4, inf) == 0
    yin = alg.vec([0.0, -1.0, 0.0, 0.5, 0.0])
    assert L.OSQPVectorf_in_reccone(alg.vec([0.0, 0.0, 0.0, 0.0, 0.0]), vl, vu, inf, 1e-6) == 1
    assert L.OSQPVectorf_in_reccone(yin, vl, vu, inf, 1e-6) == 0


def test_matrix_ops(alg, la):
    L, t = alg.lib, TOL[alg.precision]
    A = sp.csc_matrix((la["test_mat_ops_A/data"], la["test_mat_ops_A/indices"], la["test_mat_ops_A/indptr"]),
                      shape=tuple(la["test_mat_ops_A/shape"]))
    d = la["test_mat_ops_d"]
    M = alg.mat(A)
    vd = alg.vec(d)
    L.OSQPMatrix_lmult_diag(M, vd)
    E = alg.vec(np.zeros(A.shape[0]))
    L.OSQPMatrix_row_norm_inf(M, E)
    assert close(alg.get(E), np.max(np.abs(sp.diags(d) @ A), axis=1).toarray().ravel(), t)
    L.OSQPMatrix_free(M)
    M = alg.mat(A)
    L.OSQPMatrix_rmult_diag(M, vd)
    Ec = alg.vec(np.zeros(A.shape[1]))
    L.OSQPMatrix_col_norm_inf(M, Ec)
    assert close(alg.get(Ec), np.max(np.abs(A @ sp.diags(d)), axis=0).toarray().ravel(), t)
    L.OSQPMatrix_free(M)
    M = alg.mat(A)
    L.OSQPMatrix_col_norm_inf(M, Ec)
    assert close(alg.get(Ec), la["test_mat_ops_inf_norm_cols"], t)
    L.OSQPMatrix_row_norm_inf(M, E)
    assert close(alg.get(E), la["test_mat_ops_inf_norm_rows"], t)
    L.OSQPMatrix_mult_scalar(M, 2.0)
    L.OSQPMatrix_row_norm_inf(M, E)
    assert close(alg.get(E), 2.0 * la["test_mat_ops_inf_norm_rows"], t)
    L.OSQPMatrix_free(M)


def test_mat_vec(alg, la):
    L, t = alg.lib, TOL[alg.precision]
    mk = lambda p: sp.csc_matrix((la[p + "/data"], la[p + "/indices"], la[p + "/indptr"]), shape=tuple(la[p + "/shape"]))
    A, Pu = mk("test_mat_vec_A"), mk("test_mat_vec_Pu")
    x, y = la["test_mat_vec_x"], la["test_mat_vec_y"]
    MA, MP = alg.mat(A), alg.mat(Pu, triu=True)
    vx, vy = alg.vec(x), alg.vec(y)
    out = alg.vec(np.zeros(A.shape[0]))
    L.OSQPMatrix_Axpy(MA, vx, out, 1.0, 0.0)
    assert close(alg.get(out), la["test_mat_vec_Ax"], t)
    o2 = alg.vec(y)
    L.OSQPMatrix_Axpy(MA, vx, o2, 1.0, 1.0)
    assert close(alg.get(o2), la["test_mat_vec_Ax_cum"], t)
    outn = alg.vec(np.zeros(A.shape[1]))
    L.OSQPMatrix_Atxpy(MA, vy, outn, 1.0, 0.0)
    assert close(alg.get(outn), la["test_mat_vec_ATy"], t)
    o3 = alg.vec(x)
    L.OSQPMatrix_Atxpy(MA, vy, o3, 1.0, 1.0)
    assert close(alg.get(o3), la["test_mat_vec_ATy_cum"], t)
    o4 = alg.vec(np.zeros(Pu.shape[0]))
    L.OSQPMatrix_Axpy(MP, vx, o4, 1.0, 0.0)
    assert close(alg.get(o4), la["test_mat_vec_Px"], t)
    o5 = alg.vec(x)
    L.OSQPMatrix_Axpy(MP, vx, o5, 1.0, 1.0)
    assert close(alg.get(o5), la["test_mat_vec_Px_cum"], t)


@pytest.mark.parametrize("case", ["A4", "A5", "A3", "A0"])
def test_submatrix_byrows(alg, la, case):
    L = alg.lib
    mk = lambda p: sp.csc_matrix((la[p + "/data"], la[p + "/indices"], la[p + "/indptr"]), shape=tuple(la[p + "/shape"]))
    full = mk("test_mat_vec_A")
    ind = la[f"test_submat_{case}_ind"]
    exp = mk(f"test_submat_{case}")
    M = alg.mat(full)
    S = L.OSQPMatrix_submatrix_byrows(M, alg.ivec(ind))
    assert L.OSQPMatrix_get_m(S) == exp.shape[0] and L.OSQPMatrix_get_nz(S) == exp.nnz
    x = np.arange(full.shape[1], dtype=float) + 1.0
    out = alg.vec(np.zeros(max(exp.shape[0], 1)))
    if exp.shape[0]:
        L.OSQPMatrix_Axpy(S, alg.vec(x), out, 1.0, 0.0)
        assert close(alg.get(out), exp @ x, TOL[alg.precision])


def test_empty_matrices(alg, la):
    L = alg.lib
    mk = lambda p: sp.csc_matrix((la[p + "/data"], la[p + "/indices"], la[p + "/indptr"]), shape=tuple(la[p + "/shape"]))
    for name in ("test_mat_no_entries", "test_mat_no_rows", "test_mat_no_cols"):
        A = mk(name)
        M = alg.mat(A)
        assert L.OSQPMatrix_get_m(M) == A.shape[0] and L.OSQPMatrix_get_n(M) == A.shape[1]
        y = alg.vec(np.ones(A.shape[0]))
        L.OSQPMatrix_Axpy(M, alg.vec(np.ones(A.shape[1])), y, 1.0, 0.0)
        assert np.all(alg.get(y) == 0.0)
        L.OSQPMatrix_free(M)


def test_solve_linsys(alg, ref_tests):
    """Reduced-KKT PCG behind LinSysSolver.solve (tests/solve_linsys/test_solve_linsys.h)."""
    L = alg.lib
    pre = "solve_linsys/data/"
    d = {k[len(pre):]: ref_tests[k] for k in ref_tests.files if k.startswith(pre)}
    mk = lambda p: sp.csc_matrix((d[p + "/data"], d[p + "/indices"], d[p + "/indptr"]), shape=tuple(d[p + "/shape"]))
    A, Pu = mk("test_solve_KKT_A"), mk("test_solve_KKT_Pu")
    m, n = A.shape
    st = alg.default_settings()
    st.rho, st.sigma = float(d["test_solve_KKT_rho"]), float(d["test_solve_KKT_sigma"])
    rho = alg.vec(np.full(m, st.rho))
    MP, MA = alg.mat(Pu, triu=True), alg.mat(A)
    pr, dr = alg.F(1e-7), alg.F(1e-7)
    s = C.POINTER(alg.LinSysSolver)()
    assert L.osqp_algebra_init_linsys_solver(C.byref(s), MP, MA, rho, C.byref(st), C.byref(pr), C.byref(dr), 0) == 0
    b = alg.vec(d["test_solve_KKT_rhs"])
    assert s.contents.solve(s, b, 2) == 0
    assert close(alg.get(b), d["test_solve_KKT_x"], TOL[alg.precision])
    s.contents.free(s)
