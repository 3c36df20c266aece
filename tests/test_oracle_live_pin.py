"""The oracle against the reference itself, live: OSQP 1.0's builtin algebra
and C core compiled from the reference's sources (oracle/_ref/libosqp_ref.so,
`make -C oracle ref`) and the oracle's DIRECT mode run the same seeded
problems, settings and update sequences, and must agree on status, iteration
count, polish status and solution.  Skipped where the reference build is
absent (it is compiled from the reference tree, which only the development
machine has)."""
import os

import numpy as np
import pytest
import scipy.sparse as sp

from osqp_gb300 import problems as pb
from osqp_gb300.api import OSQP, DIRECT_SOLVER, SOLVED

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.path.join(REPO, "oracle", "_ref", "libosqp_ref.so")

pytestmark = pytest.mark.skipif(not os.path.exists(REF), reason="reference build (oracle/_ref) not present")


@pytest.fixture(scope="module")
def ref_lib():
    from osqp_gb300.api import Library
    return Library(REF, 64)


def _pair(oracle_lib, ref_lib, data, **st):
    out = []
    for lib in (oracle_lib, ref_lib):
        P, q, A, l, u = data
        s = OSQP(lib)
        assert s.setup(P, q, A, pb.clip_inf(l, 1e30), pb.clip_inf(u, 1e30), linsys_solver=DIRECT_SOLVER, **st) == 0
        out.append(s)
    return out


def _same(ro, rr, rtol=1e-7):
    assert ro.info["status_val"] == rr.info["status_val"]
    assert ro.info["iter"] == rr.info["iter"]
    assert ro.info["status_polish"] == rr.info["status_polish"]
    assert ro.info["rho_updates"] == rr.info["rho_updates"]
    if rr.info["status_val"] == SOLVED:
        scale = max(1.0, abs(rr.info["obj_val"]))
        assert abs(ro.info["obj_val"] - rr.info["obj_val"]) <= rtol * scale
        assert np.allclose(ro.x, rr.x, rtol=rtol, atol=1e-9)
        assert np.allclose(ro.y, rr.y, rtol=rtol, atol=1e-9)


SETTINGS = [
    dict(),                                                     # library defaults
    dict(rho_is_vec=0, scaling=0, check_termination=1),
    dict(rho_is_vec=1, scaling=10, polishing=1, eps_abs=1e-5, eps_rel=1e-5),
    dict(adaptive_rho=0, alpha=1.0, sigma=1e-4),
    dict(adaptive_rho=3, check_dualgap=0, scaled_termination=1),  # KKT-error adaptive rho
]


@pytest.mark.parametrize("k", range(len(SETTINGS)))
@pytest.mark.parametrize("seed", [11, 12, 13])
def test_random_qps(oracle_lib, ref_lib, k, seed):
    data = pb.random_qp(seed, n=40 + 7 * seed % 30, m=70 + 5 * seed % 40)
    so, sr = _pair(oracle_lib, ref_lib, data, **SETTINGS[k])
    _same(so.solve(), sr.solve())


@pytest.mark.parametrize("seed", [21, 22])
@pytest.mark.parametrize("k", [0, 2])
def test_mpc_and_portfolio(oracle_lib, ref_lib, seed, k):
    for data in (pb.mpc(seed), pb.portfolio(seed, n=150)):
        so, sr = _pair(oracle_lib, ref_lib, data, **SETTINGS[k])
        _same(so.solve(), sr.solve(), rtol=1e-6)


def test_update_sequences(oracle_lib, ref_lib):
    """Vector updates, warm start, cold start, matrix updates, rho and
    settings updates applied alike to both, a solve after each."""
    rng = np.random.default_rng(5)
    P, q, A, l, u = pb.random_qp(31, n=60, m=90)
    so, sr = _pair(oracle_lib, ref_lib, (P, q, A, l, u), warm_starting=1, polishing=1)
    _same(so.solve(), sr.solve())
    q2 = q * (1 + 0.1 * rng.standard_normal(q.size))
    for s in (so, sr):
        assert s.update(q=q2) == 0
    _same(so.solve(), sr.solve())
    l2 = np.where(np.isfinite(l), l - 0.05, l)
    for s in (so, sr):
        assert s.update(l=pb.clip_inf(l2, 1e30)) == 0
    _same(so.solve(), sr.solve())
    x0, y0 = rng.standard_normal(60), rng.standard_normal(90)
    for s in (so, sr):
        assert s.warm_start(x=x0, y=y0) == 0
    _same(so.solve(), sr.solve())
    for s in (so, sr):
        s.cold_start()
    _same(so.solve(), sr.solve())
    Pu = sp.triu(P, format="csc")
    Pn = Pu.data * (1 + 0.2 * rng.random(Pu.nnz))
    An = sp.csc_matrix(A).data + 0.05 * rng.standard_normal(sp.csc_matrix(A).nnz)
    idx = np.sort(rng.choice(Pu.nnz, Pu.nnz // 2, replace=False)).astype(np.int32)
    for s in (so, sr):
        assert s.update(Px=Pn[idx], Px_idx=idx, Ax=An) == 0
    _same(so.solve(), sr.solve())
    for s in (so, sr):
        assert s.update_rho(0.7) == 0
        assert s.update_settings(alpha=1.2, eps_abs=1e-4, eps_rel=1e-4, polish_refine_iter=5) == 0
    _same(so.solve(), sr.solve())
