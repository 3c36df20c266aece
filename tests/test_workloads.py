"""The seeded synthetic workloads stand in for the benchmark configurations:
their shapes, sizes and value distributions follow the configurations'
specifications (checked here on the CPU)."""
import numpy as np
import scipy.sparse as sp

from osqp_gb300 import problems as pb


def _is_triu(P):
    return sp.tril(P, -1).nnz == 0


def test_random_qp_shape_density_and_bounds():
    P, q, A, l, u = pb.random_qp(1)
    assert P.shape == (200, 200) and A.shape == (400, 200) and _is_triu(P)
    assert 0.10 < A.nnz / (400 * 200) < 0.20          # 15 % nonzeros drawn N(0, 1)
    assert np.all(l <= 0) and np.all(l >= -1) and np.all(u >= 0) and np.all(u <= 1)
    Pf = P + sp.triu(P, 1).T
    assert np.min(np.linalg.eigvalsh(Pf.toarray())) > 0.0   # M M' + 1e-2 I


def test_mpc_sizes_dynamics_and_bounds():
    for seed in range(6):
        rg = np.random.default_rng(seed)
        P, q, A, l, u = pb.mpc(rg)
        n, m = P.shape[0], A.shape[0]
        # n = (T+1) nx + T nu with T in 10..50, nx in 8..40, nu in 4..16
        found = [(T, nx, nu) for T in range(10, 51) for nx in range(8, 41) for nu in range(4, 17)
                 if (T + 1) * nx + T * nu == n and (T + 1) * nx + n == m]
        assert found
        # input bounds |u| <= 1, state bounds |x| <= 5 (the identity rows), x0 in [-1, 1]
        box_l = l[m - n:]
        assert set(np.round(np.unique(box_l), 6)) <= {-5.0, -1.0}
        assert np.all(np.abs(l[:found[0][1]]) <= 1.0)
        assert _is_triu(P) and np.allclose(P.diagonal()[-1], 0.1)   # R = 0.1 I


def test_mpc_batch_is_seeded_and_uneven():
    a = pb.mpc_batch(8, seed=3)
    b = pb.mpc_batch(8, seed=3)
    assert all((x[0] != y[0]).nnz == 0 for x, y in zip(a, b))
    assert len({p[0].shape[0] for p in a}) > 1


def test_portfolio_factor_model():
    P, q, A, l, u = pb.portfolio(seed=4, n=500)
    n, k = 500, 50
    assert P.shape == (n + k, n + k) and A.shape == (k + 1 + n, n + k)
    F = A[:k, :n].T
    assert 0.4 < F.nnz / (n * k) < 0.6                # F 50 % dense
    assert np.allclose(l[k], 1.0) and np.allclose(u[k], 1.0)   # budget 1'x = 1
    assert np.all(l[k + 1:] == 0) and np.all(u[k + 1:] == 1)   # 0 <= x <= 1


def test_svm_shape_and_labels():
    P, q, A, l, u = pb.svm(seed=5, m=2000, n=100)
    assert P.shape == (2100, 2100) and A.shape == (4000, 2100)
    Ad = A[:2000, :100]
    assert 0.10 < Ad.nnz / (2000 * 100) < 0.20        # 15 % density
    assert np.all(q[:100] == 0) and np.all(q[100:] == 1)
    assert np.allclose(P.diagonal()[:100], 2.0)        # lambda = 1 -> 0.5 x'Px = ||x||^2


def test_large_sparse_structure():
    P, q, A, l, u = pb.large_sparse(seed=2, n=2000, m=4000)
    assert P.shape == (2000, 2000) and A.shape == (4000, 2000)
    rows = np.diff(A.tocsr().indptr)
    assert rows.max() <= 10 and rows.mean() > 9.5     # 10 nonzeros per row at random columns
