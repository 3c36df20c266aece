"""Algorithmic byte counts of the OSQP hot path (the roofline numerator).

Conventions: values of width w bytes (4 for FP32, 8 for FP64), int32 indices,
generic CSR; every vector operand counted once per use (ideal reuse).

  SpMV y = M x (rows x cols, nnz):  nnz*(w+4) + (rows+1)*4 + cols*w + rows*w
  PCG iteration (reduced KKT K = P + sigma I + A' R A):
      B_pcg  = B(P_full) + B(A) + B(A') + m*w + 9*n*w
      (K p needs P p, A p and A'(rho .* A p); vectors: p, Kp, x, r, M^-1 read,
       x, r, y, p written)
  ADMM iteration outside the PCG loop:
      B_admm = B(A') [right-hand side] + B(A) [z~ = A x~] + 10*n*w + 12*m*w
               + B_pcg [the PCG start-up product r = K x - rhs]
  residual / termination evaluation (every check_termination iterations):
      B_term = B(P_full) + B(A) + B(A') + 8*(n + m)*w
  block-Jacobi preconditioner (cg_precond = 2): the PCG iteration reads the
      32 x 32 blocks of M^-1, ceil(n / 32) * 1024 * w bytes, instead of the
      n*w diagonal
  direct solver (block-tridiagonal factor of F elements, gb_direct.cuh):
      ADMM iteration  B(A') + B(A) + F*w [one forward and one backward sweep
                      read each factor block once] + 2*n*4 [permutation]
                      + 10*n*w + 12*m*w
      factorisation   (set-up and every rho update) F*w written
                      + B(P_full) + 2*B(A) + B(A') read (every row of A
                      touches at most two blocks)
"""
from __future__ import annotations


def spmv_bytes(rows: int, cols: int, nnz: int, w: int) -> int:
    return nnz * (w + 4) + (rows + 1) * 4 + cols * w + rows * w


def qp_bytes(n: int, m: int, nnz_pfull: int, nnz_a: int, w: int, block_precond: bool = False):
    bp = spmv_bytes(n, n, nnz_pfull, w)
    ba = spmv_bytes(m, n, nnz_a, w)
    bat = spmv_bytes(n, m, nnz_a, w)
    pcg = bp + ba + bat + m * w + 9 * n * w
    if block_precond:
        pcg += ((n + 31) // 32) * 1024 * w - n * w
    admm = bat + ba + 10 * n * w + 12 * m * w + pcg
    term = bp + ba + bat + 8 * (n + m) * w
    return pcg, admm, term


def solve_bytes(n, m, nnz_pfull, nnz_a, w, admm_iters, pcg_iters, check_termination, block_precond=False):
    pcg, admm, term = qp_bytes(n, m, nnz_pfull, nnz_a, w, block_precond)
    checks = admm_iters // max(1, check_termination) + 1
    return pcg_iters * pcg + admm_iters * admm + checks * term


def pfull_nnz(P_triu) -> int:
    """Nonzeros of the full symmetric P with an explicit diagonal."""
    import numpy as np
    import scipy.sparse as sp
    P = sp.csc_matrix(P_triu)
    n = P.shape[0]
    has_diag = np.zeros(n, bool)
    coo = P.tocoo()
    has_diag[coo.row[coo.row == coo.col]] = True
    nd = int(has_diag.sum())
    return 2 * P.nnz - 2 * nd + n


def direct_solve_bytes(n, m, nnz_pfull, nnz_a, w, admm_iters, factor_elems, factorisations, check_termination):
    """Algorithmic bytes of one direct-solver QP solve (see the module docstring)."""
    bp = spmv_bytes(n, n, nnz_pfull, w)
    ba = spmv_bytes(m, n, nnz_a, w)
    bat = spmv_bytes(n, m, nnz_a, w)
    it = bat + ba + factor_elems * w + 2 * n * 4 + 10 * n * w + 12 * m * w
    term = bp + ba + bat + 8 * (n + m) * w
    fac = factor_elems * w + bp + 2 * ba + bat
    checks = admm_iters // max(1, check_termination) + 1
    return admm_iters * it + checks * term + factorisations * fac
