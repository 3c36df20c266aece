"""Integer work of the set-up, bit-exact: the CSR row structures derived from
the caller's CSC arrays (the reference's csr_transpose / csr_triu_to_full,
algebra/cuda/src/cuda_csr.cu:489-628) in all three places they are built --
the algebra library's OSQPMatrix, the single-QP engine and the batched engine
-- against scipy: row pointers, column indices (ascending per row), the
input position of every entry (A -> rows of A, triu(P) -> full symmetric P
with its mirror entries and structural diagonals) and the diagonal positions.
Inputs: the reference's lin_alg matrix, the benchmark shapes and the edge
cases (empty columns and rows, P without some diagonal entries, m = 0)."""
import ctypes as C

import numpy as np
import pytest
import scipy.sparse as sp

from conftest import csc_from
from osqp_gb300 import load
from osqp_gb300 import problems as pb
from osqp_gb300.api import OSQP, Batch, _ptr

pytestmark = pytest.mark.gpu


def expected_rows_A(A):
    """CSR of A with, per entry, its position in A's CSC arrays."""
    A = sp.csc_matrix(A)
    A.sort_indices()
    pos = sp.csc_matrix((np.arange(A.nnz, dtype=np.float64) + 1, A.indices, A.indptr), shape=A.shape)
    R = pos.tocsr()
    R.sort_indices()
    return R.indptr.astype(np.int32), R.indices.astype(np.int32), (R.data - 1).astype(np.int32)


def expected_rows_P(P):
    """Full symmetric P with an explicit diagonal: CSR, per entry the position
    in triu(P)'s CSC arrays (-1: structural diagonal), diagonal positions."""
    T = sp.triu(sp.csc_matrix(P), format="csc")
    T.sort_indices()
    n = T.shape[0]
    cols = np.repeat(np.arange(n), np.diff(T.indptr))
    rows = T.indices
    pos = np.arange(T.nnz)
    off = rows != cols
    r = np.concatenate([rows, cols[off]])
    c = np.concatenate([cols, rows[off]])
    s = np.concatenate([pos, pos[off]])
    missing = np.setdiff1d(np.arange(n), rows[~off])
    r = np.concatenate([r, missing]); c = np.concatenate([c, missing]); s = np.concatenate([s, -np.ones(missing.size, int)])
    o = np.lexsort((c, r))
    r, c, s = r[o], c[o], s[o]
    rowptr = np.concatenate([[0], np.cumsum(np.bincount(r, minlength=n))]).astype(np.int32)
    diag = np.array([rowptr[i] + np.flatnonzero(c[rowptr[i]:rowptr[i + 1]] == i)[0] for i in range(n)], np.int32)
    return rowptr, c.astype(np.int32), s.astype(np.int32), diag


def cases(ref_tests):
    A_ref = csc_from(ref_tests, "lin_alg/data/test_sp_matrix_A")
    n0 = A_ref.shape[1]
    M = sp.random(n0, n0, density=0.3, random_state=np.random.default_rng(4))
    out = [("lin_alg A", sp.triu(M @ M.T + sp.eye(n0), format="csc"), A_ref)]
    d = pb.random_qp(1)
    out.append(("random_qp n=200", d[0], d[2]))
    d = pb.mpc(np.random.default_rng(3))
    out.append(("mpc", d[0], d[2]))
    d = pb.portfolio(5, n=150)
    out.append(("portfolio", d[0], d[2]))
    # P missing diagonal entries (zero columns), A with empty columns and rows
    rng = np.random.default_rng(7)
    P = sp.random(30, 30, density=0.1, random_state=rng)
    P = sp.triu(P + P.T, format="csc")
    P = sp.csc_matrix(P.toarray() * (np.arange(30) % 3 != 0)[None, :])
    P.eliminate_zeros()
    A = sp.random(25, 30, density=0.1, random_state=rng, format="csc")
    A = sp.csc_matrix(A.toarray() * (np.arange(30) % 4 != 0)[None, :] * (np.arange(25) % 5 != 0)[:, None])
    A.eliminate_zeros()
    out.append(("edge: missing diagonals, empty rows and columns", P, A))
    out.append(("edge: m = 0", sp.triu(sp.eye(12) * 2.0, format="csc"), sp.csc_matrix((0, 12))))
    return out


def _data(P, A):
    n, m = P.shape[0], A.shape[0]
    return P, np.ones(n), A, -np.ones(m), np.ones(m)


def _get(fn, rows, nz, extra):
    rp = np.zeros(rows + 1, np.int32)
    col = np.zeros(max(nz, 1), np.int32)
    src = np.zeros(max(nz, 1), np.int32)
    diag = np.zeros(max(extra, 1), np.int32)
    I = C.c_int32
    got = fn(_ptr(rp, I), _ptr(col, I), _ptr(src, I), _ptr(diag, I))
    return got, rp, col[:nz], src[:nz], diag[:extra]


def check(name, P, A, fetch):
    n, m = P.shape[0], A.shape[0]
    erp, ecol, esrc, ediag = expected_rows_P(P)
    got, rp, col, src, diag = _get(lambda *a: fetch(0, *a), n, len(ecol), n)
    assert got == len(ecol), name
    assert np.array_equal(rp, erp) and np.array_equal(col, ecol), name
    assert np.array_equal(src, esrc), name
    assert np.array_equal(diag, ediag), name
    arp, acol, asrc = expected_rows_A(A)
    got, rp, col, src, _ = _get(lambda *a: fetch(1, *a), m, len(acol), 0)
    assert got == len(acol), name
    assert np.array_equal(rp, arp) and np.array_equal(col, acol) and np.array_equal(src, asrc), name


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_single_qp_engine_structures(prec, ref_tests):
    lib = load(prec)
    fn = lib.lib.osqp_gb300_structure
    I = lib.I
    fn.argtypes = [C.c_void_p, I, C.POINTER(I), C.POINTER(I), C.POINTER(I), C.POINTER(I)]
    fn.restype = I
    for name, P, A in cases(ref_tests):
        s = OSQP(lib)
        assert s.setup(*_data(P, A), eps_abs=1e-3, eps_rel=1e-3) == 0, name
        check(name, P, A, lambda which, *a: fn(s._solver, which, *a))
        s.cleanup()


def test_batch_engine_structures(ref_tests):
    lib = load("f32")
    fn = lib.lib.osqp_gb300_batch_structure
    I = lib.I
    fn.argtypes = [C.c_void_p, I, I, C.POINTER(I), C.POINTER(I), C.POINTER(I), C.POINTER(I)]
    fn.restype = I
    cs = cases(ref_tests)
    b = Batch(lib)
    assert b.setup([_data(P, A) for _, P, A in cs], eps_abs=1e-3, eps_rel=1e-3) == 0
    for k, (name, P, A) in enumerate(cs):
        check(name, P, A, lambda which, *a: fn(b._h, k, which, *a))
    b.cleanup()


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_algebra_matrix_rows(prec, ref_tests):
    from osqp_gb300.algebra import AlgebraLib
    alg = AlgebraLib(prec)
    fn = alg.lib.osqp_gb300_matrix_rows
    I = alg.I
    fn.argtypes = [C.c_void_p, C.POINTER(I), C.POINTER(I), C.POINTER(I), C.POINTER(I)]
    fn.restype = I
    for name, P, A in cases(ref_tests):
        MP, MA = alg.mat(P, triu=True), alg.mat(A)
        check(name, P, A, lambda which, *a: fn(MP if which == 0 else MA, *a))
