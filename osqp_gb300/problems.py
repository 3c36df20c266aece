"""Seeded synthetic QP workloads.

Every generator draws from ``numpy.random.Generator(PCG64(seed))`` and returns
``(P, q, A, l, u)`` with P upper-triangular CSC, A CSC, in float64.  The
shapes and value distributions are the five benchmark configurations this
package is measured on:

  random_qp      plain random QP, n=200, m=400, 15% density
  large_sparse   n=50,000 / m=100,000; P = M M' + 1e-2 I with 8 nonzeros per
                 column of M, A with 10 nonzeros per row
  mpc            linear MPC, horizon T~U{10..50}, nx~U{8..40}, nu~U{4..16},
                 stacked as in the reference's MPC example (docs/examples/mpc.rst)
  portfolio      factor-model portfolio (docs/examples/portfolio.rst),
                 n~U{100..2000}, k=n/10, F 50% dense
  svm            hinge-loss SVM (docs/examples/svm.rst), lambda = 1 mapped to
                 P = blkdiag(2*lambda*I, 0) so that 0.5 x'Px = lambda*||x||^2
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp
from numpy.random import Generator, PCG64

INF = np.inf


def _rng(seed):
    return seed if isinstance(seed, Generator) else Generator(PCG64(seed))


def _sprandn(rg, m, n, density):
    return sp.random(m, n, density=density, format="csc", random_state=rg,
                     data_rvs=rg.standard_normal)


def random_qp(seed=1, n=200, m=400, density=0.15):
    rg = _rng(seed)
    M = _sprandn(rg, n, n, density)
    P = (M @ M.T + 1e-2 * sp.eye(n)).tocsc()
    q = rg.standard_normal(n)
    A = _sprandn(rg, m, n, density)
    l = -rg.random(m)
    u = rg.random(m)
    return sp.triu(P, format="csc"), q, A, l, u


def large_sparse(seed=2, n=50_000, m=100_000, p_col_nnz=8, a_row_nnz=10):
    rg = _rng(seed)
    rows = rg.integers(0, n, size=(n, p_col_nnz)).ravel()
    cols = np.repeat(np.arange(n), p_col_nnz)
    M = sp.csc_matrix((rg.standard_normal(rows.size), (rows, cols)), shape=(n, n))
    P = (M @ M.T + 1e-2 * sp.eye(n)).tocsc()
    q = rg.standard_normal(n)
    arow = np.repeat(np.arange(m), a_row_nnz)
    acol = rg.integers(0, n, size=(m, a_row_nnz)).ravel()
    A = sp.csc_matrix((rg.standard_normal(arow.size), (arow, acol)), shape=(m, n))
    l = -rg.random(m)
    u = rg.random(m)
    return sp.triu(P, format="csc"), q, A, l, u


def mpc(seed=3, T=None, nx=None, nu=None):
    """One linear-MPC QP.  Variables (x(0..T), u(0..T-1)); dynamics as equalities."""
    rg = _rng(seed)
    T = int(rg.integers(10, 51)) if T is None else T
    nx = int(rg.integers(8, 41)) if nx is None else nx
    nu = int(rg.integers(4, 17)) if nu is None else nu
    G = rg.standard_normal((nx, nx))
    Ad = np.eye(nx) + 0.1 * G / np.sqrt(nx)
    rad = np.max(np.abs(np.linalg.eigvals(Ad)))
    if rad > 1.05:
        Ad *= 1.05 / rad
    Bd = rg.standard_normal((nx, nu))
    Q = sp.diags(rg.uniform(0.0, 10.0, nx))
    R = 0.1 * sp.eye(nu)
    x0 = rg.uniform(-1.0, 1.0, nx)
    P = sp.block_diag([sp.kron(sp.eye(T), Q), Q, sp.kron(sp.eye(T), R)], format="csc")
    q = np.zeros((T + 1) * nx + T * nu)
    Ax = sp.kron(sp.eye(T + 1), -sp.eye(nx)) + sp.kron(sp.eye(T + 1, k=-1), sp.csc_matrix(Ad))
    Bu = sp.kron(sp.vstack([sp.csc_matrix((1, T)), sp.eye(T)]), sp.csc_matrix(Bd))
    Aeq = sp.hstack([Ax, Bu])
    leq = np.hstack([-x0, np.zeros(T * nx)])
    nvar = (T + 1) * nx + T * nu
    Aineq = sp.eye(nvar)
    lineq = np.hstack([np.full((T + 1) * nx, -5.0), np.full(T * nu, -1.0)])
    uineq = -lineq
    A = sp.vstack([Aeq, Aineq], format="csc")
    l = np.hstack([leq, lineq])
    u = np.hstack([leq, uineq])
    A.eliminate_zeros()
    return sp.triu(P, format="csc"), q, A, l, u


def mpc_batch(count=4096, seed=3, start=0):
    """`count` independent MPC instances; instance i uses seed (seed, i), for
    i = start .. start + count - 1 (a contiguous share of a larger set)."""
    return [mpc(Generator(PCG64([seed, i]))) for i in range(start, start + count)]


def mpc_x0_bounds(l, u, x0):
    """Bounds of an MPC instance with its initial state replaced by x0."""
    nx = x0.size
    l2, u2 = l.copy(), u.copy()
    l2[:nx] = -x0
    u2[:nx] = -x0
    return l2, u2


def portfolio(seed=4, n=None, gamma=1.0):
    rg = _rng(seed)
    n = int(rg.integers(100, 2001)) if n is None else n
    k = max(1, n // 10)
    F = _sprandn(rg, n, k, 0.5)
    D = sp.diags(rg.uniform(0.0, np.sqrt(k), n))
    mu = rg.standard_normal(n)
    P = sp.block_diag([D, sp.eye(k)], format="csc")
    q = np.hstack([-mu / (2 * gamma), np.zeros(k)])
    A = sp.bmat([[F.T, -sp.eye(k)],
                 [sp.csc_matrix(np.ones((1, n))), None],
                 [sp.eye(n), None]], format="csc")
    l = np.hstack([np.zeros(k), 1.0, np.zeros(n)])
    u = np.hstack([np.zeros(k), 1.0, np.ones(n)])
    return sp.triu(P, format="csc"), q, A, l, u


def svm(seed=5, m=100_000, n=1_000, density=0.15, lam=1.0):
    rg = _rng(seed)
    half = m // 2
    b = np.hstack([np.ones(half), -np.ones(m - half)])
    S = sp.random(m, n, density=density, format="csr", random_state=rg)
    S.data = rg.standard_normal(S.data.size) / np.sqrt(n)
    rowsign = np.repeat(b, np.diff(S.indptr))
    S.data += rowsign / n
    Ad = S.tocsc()
    Im = sp.eye(m)
    P = sp.block_diag([2.0 * lam * sp.eye(n), sp.csc_matrix((m, m))], format="csc")
    q = np.hstack([np.zeros(n), np.ones(m)])
    A = sp.bmat([[sp.diags(b) @ Ad, -Im], [None, Im]], format="csc")
    l = np.hstack([-np.inf * np.ones(m), np.zeros(m)])
    u = np.hstack([-np.ones(m), np.inf * np.ones(m)])
    return sp.triu(P, format="csc"), q, A, l, u


def clip_inf(v, infty):
    """Replace +-inf by +-OSQP_INFTY of the library precision (1e30 FP64, 1e17 FP32)."""
    v = np.asarray(v, dtype=np.float64).copy()
    v[v > infty] = infty
    v[v < -infty] = -infty
    return v
