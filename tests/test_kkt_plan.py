"""Ordering of the direct KKT solver (osqp_gb300_kkt_plan, host code of the
GB300 library; runs on CPU): a permutation whose blocks make
K = P + sigma I + A'RA block tridiagonal, the stages of an MPC QP as blocks,
and the on-chip block limit enforced."""
import numpy as np
import pytest
import scipy.sparse as sp

from osqp_gb300 import load
from osqp_gb300 import problems as pb
from osqp_gb300.api import kkt_plan


@pytest.fixture(scope="module")
def lib():
    from osqp_gb300.build import build
    build()
    return load("f32")


def kkt_pattern(P, A):
    Pu = sp.triu(sp.csc_matrix(P))
    Pf = (Pu + Pu.T).tocsr()
    Ab = sp.csc_matrix(A).copy()
    Ab.data[:] = 1.0
    K = (abs(Pf) + Ab.T @ Ab + sp.eye(P.shape[0])).tocoo()
    return K.row, K.col


def check_block_tridiagonal(P, A, bs, perm):
    n = P.shape[0]
    assert np.array_equal(np.sort(perm), np.arange(n))           # a permutation
    assert bs[0] == 0 and bs[-1] == n and np.all(np.diff(bs) > 0)
    blk = np.empty(n, np.int64)
    for k in range(len(bs) - 1):
        blk[perm[bs[k]:bs[k + 1]]] = k
    r, c = kkt_pattern(P, A)
    assert np.max(np.abs(blk[r] - blk[c])) <= 1                  # every entry in the band of blocks


@pytest.mark.parametrize("seed", [0, 1, 2, 3, 7, 11])
def test_mpc_blocks_are_stages(lib, seed):
    P, q, A, l, u = pb.mpc(np.random.default_rng([3, seed]))
    rc, bs, perm = kkt_plan(lib, P, A)
    assert rc == 0
    check_block_tridiagonal(P, A, bs, perm)
    nx = int(np.argmax(np.diff(A.tocsr().indptr) != 1))
    n = P.shape[0]
    meq = int(np.sum(np.abs(l - u) < 1e-12))
    T = meq // nx - 1
    nu = (n - (T + 1) * nx) // T
    sizes = np.diff(bs)
    # one stage (x_k, u_k) per block, up to merging of small neighbours
    assert sizes.max() <= max(nx + nu, 32), (sizes, nx, nu)
    assert len(sizes) >= (T + 1) // 2


def test_small_dense_and_limits(lib):
    P, q, A, l, u = pb.random_qp(1, n=60, m=120)
    rc, bs, perm = kkt_plan(lib, P, A)
    assert rc == 0
    check_block_tridiagonal(P, A, bs, perm)
    rc, _, _ = kkt_plan(lib, P, A, bmax_limit=10)
    assert rc == 1                                               # dense coupling: one block of 60


def test_disconnected_and_empty_rows(lib):
    # two independent chains, an unconstrained variable, an empty row of A
    n = 9
    P = sp.eye(n, format="csc")
    rows = [(0, 0), (0, 1), (1, 1), (1, 2), (2, 5), (2, 6), (3, 6), (3, 7)]
    A = sp.csc_matrix((np.ones(len(rows)), ([r for r, _ in rows], [c for _, c in rows])), shape=(5, n))
    rc, bs, perm = kkt_plan(lib, P, A)
    assert rc == 0
    check_block_tridiagonal(P, A, bs, perm)


def test_portfolio_budget_row_exceeds_limit(lib):
    P, q, A, l, u = pb.portfolio(4, n=300)
    rc, _, _ = kkt_plan(lib, P, A, bmax_limit=100)
    assert rc == 1


def test_rejects_lower_triangle(lib):
    P = sp.csc_matrix(np.array([[1.0, 0.0], [1.0, 1.0]]))
    A = sp.eye(2, format="csc")
    from osqp_gb300.api import _csc_parts
    import ctypes as C
    L, I = lib.lib, lib.I
    (n, _), pp, pi, _ = _csc_parts(P, lib.np_float, triu=False)
    (m, _), ap, ai, _ = _csc_parts(A, lib.np_float, triu=False)
    nb = I(0)
    bs = np.zeros(n + 1, np.int32)
    perm = np.zeros(n, np.int32)
    P_ = lambda a: a.ctypes.data_as(C.POINTER(I))
    rc = L.osqp_gb300_kkt_plan(n, m, P_(pp), P_(pi), P_(ap), P_(ai), 1000, C.byref(nb), P_(bs), P_(perm))
    assert rc == 2
