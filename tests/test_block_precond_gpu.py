"""Block-Jacobi preconditioner (cg_precond = 2) on the GPU, through the C ABI.

Bars: the device-built blocks equal numpy's inverses of the same 32 x 32
blocks of K (FP64: 1e-9 relative; FP32: the blocks are formed and inverted
in FP64 from the FP32 data, then rounded, so 1e-5 of the block's largest
entry); solves in every execution form reach the builtin (direct) algebra's
status and an objective as close to the optimum as the FP64 oracle running
the same preconditioner (test_batch_gpu.check_against_oracles).
"""
import numpy as np
import pytest

from osqp_gb300 import load
from osqp_gb300 import problems as pb
from osqp_gb300.api import OSQP, Batch, SOLVED, BLOCK_DIAGONAL_PRECONDITIONER, objective
from test_batch_gpu import WORKLOAD, _mix, check_against_oracles
from test_block_precond import kkt_blocks

pytestmark = pytest.mark.gpu

BLOCK = dict(WORKLOAD, cg_precond=BLOCK_DIAGONAL_PRECONDITIONER)
RAW = dict(BLOCK, scaling=0, rho_is_vec=0)     # unscaled data, scalar rho: K = P + sigma I + rho A'A


def _rounded(P, A, prec):
    if prec == "f64":
        return P, A
    P, A = P.copy(), A.copy()
    P.data = P.data.astype(np.float32).astype(np.float64)
    A.data = A.data.astype(np.float32).astype(np.float64)
    return P, A


def _check_blocks(got, P, A, prec, rho, sigma=1e-6):
    P, A = _rounded(P, A, prec)
    if prec == "f32":
        rho, sigma = float(np.float32(rho)), float(np.float32(sigma))
    want = kkt_blocks(P, A, sigma, rho)
    assert got.shape == want.shape
    tol = 1e-9 if prec == "f64" else 1e-5
    for b in range(got.shape[0]):
        scale = np.max(np.abs(want[b]))
        assert np.max(np.abs(got[b] - want[b])) <= tol * scale, (b, np.max(np.abs(got[b] - want[b])), scale)


@pytest.mark.parametrize("prec", ["f32", "f64"])
@pytest.mark.parametrize("n,m", [(70, 140), (64, 100)])
def test_device_blocks_are_inverse_kkt_blocks(prec, n, m):
    P, q, A, l, u = pb.random_qp(3, n=n, m=m)
    s = OSQP(load(prec))
    assert s.setup(P, q, A, l, u, **RAW) == 0
    _check_blocks(s.precond_blocks(), P, A, prec, 0.1)
    s.cleanup()


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_blocks_follow_settings_and_rho_updates(prec):
    """Jacobi at set-up, block-Jacobi after osqp_update_settings, blocks rebuilt
    by osqp_update_rho; the solve after each change is SOLVED."""
    P, q, A, l, u = pb.random_qp(4, n=90, m=150)
    s = OSQP(load(prec))
    assert s.setup(P, q, A, l, u, **dict(RAW, cg_precond=1)) == 0
    assert s.precond_blocks().size == 0
    assert s.update_settings(cg_precond=BLOCK_DIAGONAL_PRECONDITIONER) == 0
    _check_blocks(s.precond_blocks(), P, A, prec, 0.1)
    assert s.update_rho(2.0) == 0
    _check_blocks(s.precond_blocks(), P, A, prec, 2.0)
    assert s.solve().info["status_val"] == SOLVED
    s.cleanup()


CASES = {
    "random_qp_s1": lambda: pb.random_qp(1, n=100, m=200),
    "random_qp_s7": lambda: pb.random_qp(7, n=60, m=120),
    "mpc_s1": lambda: pb.mpc(1),
    "mpc_s2": lambda: pb.mpc(2),
    "portfolio_s1": lambda: pb.portfolio(1),
}


@pytest.mark.parametrize("prec", ["f32", "f64"])
@pytest.mark.parametrize("case", sorted(CASES))
def test_engine_block_mode_matches_oracle(prec, case, oracle_lib):
    d = CASES[case]()
    s = OSQP(load(prec))
    assert s.setup(*d, **BLOCK) == 0
    r = s.solve()
    assert s.stats()["pcg_iter"] > 0
    obj = objective(d[0], d[1], r.x) if r.info["status_val"] == SOLVED else None
    check_against_oracles(oracle_lib, d, r.info["status_val"], obj, prec, settings=BLOCK)
    s.cleanup()


@pytest.mark.parametrize("mode", ["block", "grid", "cluster8"])
def test_engine_forms_agree_in_block_mode(mode, monkeypatch, oracle_lib):
    """One CTA, cooperative grid and cluster forms (the block build and the
    two-pass apply in each) against the oracle with the same preconditioner."""
    monkeypatch.setenv("OSQP_GB300_MODE", mode)
    d = pb.random_qp(5, n=150, m=300)
    s = OSQP(load("f64"))
    assert s.setup(*d, **BLOCK) == 0
    r = s.solve()
    obj = objective(d[0], d[1], r.x) if r.info["status_val"] == SOLVED else None
    check_against_oracles(oracle_lib, d, r.info["status_val"], obj, "f64", settings=BLOCK)
    s.cleanup()


@pytest.mark.parametrize("prec,cluster,split", [("f32", "0", None), ("f64", "0", None), ("f32", "8", None),
                                                ("f32", "0", "40"), ("f64", "0", "40")])
def test_batch_block_mode_matches_oracle(prec, cluster, split, oracle_lib, monkeypatch):
    """CTA form, cluster form, and a split at ADMM iteration 40 that moves every
    unfinished QP to the sliced cluster tail (slices start on block bounds)."""
    monkeypatch.setenv("OSQP_GB300_BATCH_CLUSTER", cluster)
    if split:
        monkeypatch.setenv("OSQP_GB300_BATCH_SPLIT", split)
    probs = _mix(10, seed=4)
    b = Batch(load(prec))
    assert b.setup(probs, **BLOCK) == 0 and b.solve() == 0
    sol = b.solution()
    xs = b.split(sol["x"], "n")
    for k, d in enumerate(probs):
        obj = objective(d[0], d[1], xs[k].astype(np.float64)) if sol["status"][k] == SOLVED else None
        check_against_oracles(oracle_lib, d, sol["status"][k], obj, prec, settings=BLOCK)
    b.cleanup()


def test_batch_block_mode_alone_and_in_mix_identical():
    lib = load("f32")
    probs = _mix(8, seed=6)
    big = Batch(lib)
    assert big.setup(probs, **BLOCK) == 0 and big.solve() == 0
    sb = big.solution()
    xs_big = big.split(sb["x"], "n")
    for k in (0, 3, 4):
        one = Batch(lib)
        assert one.setup([probs[k]], **BLOCK) == 0 and one.solve() == 0
        s1 = one.solution()
        assert s1["status"][0] == sb["status"][k] and s1["iter"][0] == sb["iter"][k]
        assert np.array_equal(s1["x"], xs_big[k])
