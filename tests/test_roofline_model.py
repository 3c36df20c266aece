"""The algorithmic-byte model behind bench.py's roofline (osqp_gb300/roofline.py)."""
import numpy as np
import scipy.sparse as sp

from osqp_gb300.roofline import spmv_bytes, qp_bytes, solve_bytes, pfull_nnz


def test_spmv_bytes_counts_entries_row_pointers_and_vectors():
    # nnz (value + index) + (rows+1) row pointers + x once + y once, FP32
    assert spmv_bytes(rows=3, cols=5, nnz=7, w=4) == 7 * 8 + 4 * 4 + 5 * 4 + 3 * 4


def test_pcg_iteration_bytes_of_the_large_sparse_configuration():
    # n = 50k, m = 100k, nnz(P_full) ~ 2.85M, nnz(A) ~ 1.0M: about 43 MB per PCG iteration
    pcg, admm, term = qp_bytes(50_000, 100_000, 2_850_000, 1_000_000, 4)
    assert 40e6 < pcg < 46e6
    assert admm > pcg and term > 0


def test_solve_bytes_adds_iterations_and_termination_checks():
    pcg, admm, term = qp_bytes(100, 200, 400, 300, 4)
    assert solve_bytes(100, 200, 400, 300, 4, admm_iters=10, pcg_iters=50, check_termination=5) == \
        50 * pcg + 10 * admm + 3 * term


def test_pfull_nnz_counts_the_explicit_diagonal():
    P = sp.triu(sp.csc_matrix(np.array([[2.0, 1.0, 0.0], [1.0, 0.0, 0.0], [0.0, 0.0, 3.0]])), format="csc")
    # stored triangle: (0,0) (0,1) (2,2); full with explicit diagonal: 2*3 - 2*2 + 3 = 5
    assert pfull_nnz(P) == 5


def test_block_precond_reads_the_blocks_instead_of_the_diagonal():
    # n = 100 -> 4 blocks of 32 x 32 values replace the 100-value diagonal per PCG iteration
    pcg, admm, term = qp_bytes(100, 200, 400, 300, 4)
    pcg_b, admm_b, term_b = qp_bytes(100, 200, 400, 300, 4, block_precond=True)
    assert pcg_b - pcg == 4 * 1024 * 4 - 100 * 4
    assert admm_b - admm == pcg_b - pcg and term_b == term
