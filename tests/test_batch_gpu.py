"""Batched engine (osqp_gb300_batch_*): parity per QP with the FP64 oracle, and
the same result for a QP alone and inside a mixed batch."""
import numpy as np
import pytest

from osqp_gb300 import load
from osqp_gb300 import problems as pb
from osqp_gb300.api import OSQP, Batch, SOLVED, DIRECT_SOLVER, INDIRECT_SOLVER, objective

pytestmark = pytest.mark.gpu

WORKLOAD = dict(rho=0.1, sigma=1e-6, alpha=1.6, scaling=10, eps_abs=1e-3, eps_rel=1e-3, rho_is_vec=1,
                check_termination=5, adaptive_rho_tolerance=5.0, max_iter=4000, check_dualgap=1)


def _mix(count, seed=0):
    probs = []
    for k in range(count):
        if k % 5 == 3:
            probs.append(pb.portfolio(seed * 1000 + k, n=120 + 7 * k))
        elif k % 5 == 4:
            probs.append(pb.random_qp(seed * 1000 + k, n=40 + k, m=60 + 2 * k))
        else:
            probs.append(pb.mpc(seed * 1000 + k))
    return probs


def optimum(oracle_lib, d):
    """High-accuracy FP64 optimum (direct LDL^T, eps 1e-9, polished)."""
    s = OSQP(oracle_lib)
    assert s.setup(*d, linsys_solver=DIRECT_SOLVER, **dict(WORKLOAD, eps_abs=1e-9, eps_rel=1e-9, max_iter=100000,
                                                            polishing=1)) == 0
    r = s.solve()
    return r.info["status_val"], r.info["obj_val"]


def check_against_oracles(oracle_lib, d, status, obj_gpu, prec, settings=WORKLOAD):
    """Status of the reference's builtin (direct) algebra; trajectory of the
    same-algorithm FP64 oracle (indirect, same preconditioner); objective
    error against the true optimum no worse than 3x the direct oracle's own at
    the same eps, or eps."""
    sd = OSQP(oracle_lib)
    assert sd.setup(*d, linsys_solver=DIRECT_SOLVER, **settings) == 0
    rd = sd.solve()
    assert status == rd.info["status_val"]
    if status != SOLVED:
        return
    si = OSQP(oracle_lib)
    assert si.setup(*d, linsys_solver=INDIRECT_SOLVER, **settings) == 0
    ri = si.solve()
    st_opt, opt = optimum(oracle_lib, d)
    assert st_opt == SOLVED
    scale = max(1.0, abs(opt))
    err_gpu = abs(obj_gpu - opt) / scale
    err_direct = abs(rd.info["obj_val"] - opt) / scale
    err_indirect = abs(ri.info["obj_val"] - opt) / scale
    # eps = 1e-3 accuracy class: no further from the optimum than 3x the
    # reference's own answers (builtin direct, and the same PCG algorithm in
    # FP64), or 1e-4 (FP64) / 1e-3 (FP32) relative
    bar = max(3.0 * err_direct, 3.0 * err_indirect, 1e-4 if prec == "f64" else 1e-3)
    assert err_gpu <= bar, (err_gpu, err_direct, err_indirect)
    if prec == "f64":
        # same algorithm in FP64: the GPU stays on the oracle's PCG trajectory up
        # to reduction order (eps-class agreement)
        assert abs(obj_gpu - ri.info["obj_val"]) / scale < 1e-3, (obj_gpu, ri.info["obj_val"])


@pytest.mark.parametrize("prec,cluster", [("f32", "0"), ("f64", "0"), ("f32", "8"), ("f32", "1"), ("f64", "4")])
def test_batch_matches_oracle(prec, cluster, oracle_lib, monkeypatch):
    monkeypatch.setenv("OSQP_GB300_BATCH_CLUSTER", cluster)
    lib = load(prec)
    probs = _mix(15, seed=1)
    b = Batch(lib)
    assert b.setup(probs, **WORKLOAD) == 0
    assert b.solve() == 0
    sol = b.solution()
    xs = b.split(sol["x"], "n")
    for k, d in enumerate(probs):
        obj_gpu = objective(d[0], d[1], xs[k].astype(np.float64)) if sol["status"][k] == SOLVED else None
        check_against_oracles(oracle_lib, d, sol["status"][k], obj_gpu, prec)


@pytest.mark.parametrize("prec,cluster", [("f32", "0"), ("f64", "0"), ("f32", "4"), ("f32", "2")])
def test_alone_and_in_mix_identical(prec, cluster, monkeypatch):
    """A QP gives bit-identical results solved alone or inside a batch."""
    monkeypatch.setenv("OSQP_GB300_BATCH_CLUSTER", cluster)
    lib = load(prec)
    probs = _mix(12, seed=2)
    big = Batch(lib)
    assert big.setup(probs, **WORKLOAD) == 0 and big.solve() == 0
    sb = big.solution()
    xs_big = big.split(sb["x"], "n")
    for k in (0, 3, 4, 11):
        one = Batch(lib)
        assert one.setup([probs[k]], **WORKLOAD) == 0 and one.solve() == 0
        s1 = one.solution()
        assert s1["status"][0] == sb["status"][k]
        assert s1["iter"][0] == sb["iter"][k]
        assert np.array_equal(s1["x"], xs_big[k])


def test_batch_update_bounds_and_resolve(oracle_lib):
    """Receding-horizon step: new initial state -> new bounds for every QP."""
    lib = load("f32")
    rng = np.random.default_rng(3)
    probs = [pb.mpc(500 + k) for k in range(8)]
    b = Batch(lib)
    assert b.setup(probs, **WORKLOAD) == 0 and b.solve() == 0
    ls, us, probs2 = [], [], []
    for (P, q, A, l, u) in probs:
        # leading rows with a single nonzero are the initial-state equalities (-x0)
        rowlen = np.diff(A.tocsr().indptr)
        nx = int(np.argmax(rowlen != 1))
        l2, u2 = pb.mpc_x0_bounds(l, u, rng.uniform(-1.0, 1.0, nx))
        ls.append(l2); us.append(u2); probs2.append((P, q, A, l2, u2))
    assert b.update(l=np.concatenate(ls), u=np.concatenate(us)) == 0
    assert b.solve() == 0
    sol = b.solution()
    xs = b.split(sol["x"], "n")
    for k, d in enumerate(probs2):
        obj_gpu = objective(d[0], d[1], xs[k].astype(np.float64)) if sol["status"][k] == SOLVED else None
        check_against_oracles(oracle_lib, d, sol["status"][k], obj_gpu, "f32")
    # invalid bounds are rejected
    bad_l = np.concatenate(ls) + 100.0
    assert b.update(l=bad_l, u=np.concatenate(us)) != 0


@pytest.mark.parametrize("prec,cluster,tail", [("f32", "0", "4"), ("f64", "2", "8"), ("f32", "0", "1")])
def test_split_tail_matches_oracle(prec, cluster, tail, oracle_lib, monkeypatch):
    """QPs still running after a few ADMM iterations continue, from where they
    stopped, on larger clusters: same statuses and accuracy as the oracle, and
    the same result for a QP alone and inside the batch."""
    monkeypatch.setenv("OSQP_GB300_BATCH_CLUSTER", cluster)
    monkeypatch.setenv("OSQP_GB300_BATCH_SPLIT", "40")
    monkeypatch.setenv("OSQP_GB300_BATCH_TAIL", tail)
    lib = load(prec)
    probs = _mix(10, seed=4)
    b = Batch(lib)
    assert b.setup(probs, **WORKLOAD) == 0 and b.solve() == 0
    sol = b.solution()
    assert (sol["iter"] > 40).any() and (sol["iter"] <= 40).any()
    xs = b.split(sol["x"], "n")
    for k, d in enumerate(probs):
        obj_gpu = objective(d[0], d[1], xs[k].astype(np.float64)) if sol["status"][k] == SOLVED else None
        check_against_oracles(oracle_lib, d, sol["status"][k], obj_gpu, prec)
    for k in (0, 7):
        one = Batch(lib)
        assert one.setup([probs[k]], **WORKLOAD) == 0 and one.solve() == 0
        s1 = one.solution()
        assert s1["iter"][0] == sol["iter"][k]
        assert np.array_equal(s1["x"], xs[k])


def test_autotune_picks_a_tile_and_restores_state(monkeypatch):
    """The SpMV tile autotuner leaves every iterate as it found it: a solve after
    tuning equals a solve of a fresh batch set up with the chosen tile."""
    lib = load("f32")
    probs = _mix(12, seed=11)
    b = Batch(lib)
    assert b.setup(probs, **WORKLOAD) == 0
    tile = b.autotune(20)
    assert tile in (4, 8, 16)
    assert b.solve() == 0
    s1 = b.solution()
    monkeypatch.setenv("OSQP_GB300_LANE_TARGET", str(tile))
    c = Batch(lib)
    assert c.setup(probs, **WORKLOAD) == 0 and c.solve() == 0
    s2 = c.solution()
    assert np.array_equal(s1["iter"], s2["iter"])
    assert np.array_equal(s1["x"], s2["x"])


def test_autotune_restores_direct_factor(monkeypatch):
    """With the direct solver a probe that changes rho refactors; the tuner puts
    the factors back with the iterates, so a solve after tuning equals a solve
    of a fresh batch with the chosen tile (bitwise)."""
    lib = load("f64")
    probs = pb.mpc_batch(24, seed=3)
    st = dict(WORKLOAD, linsys_solver=DIRECT_SOLVER, rho_is_vec=1, adaptive_rho_tolerance=5.0)
    b = Batch(lib)
    assert b.setup(probs, **st) == 0
    tile = b.autotune(60)
    assert b.solve() == 0
    s1 = b.solution()
    monkeypatch.setenv("OSQP_GB300_LANE_TARGET", str(tile))
    c = Batch(lib)
    assert c.setup(probs, **st) == 0 and c.solve() == 0
    s2 = c.solution()
    assert np.array_equal(s1["iter"], s2["iter"])
    assert np.array_equal(s1["x"], s2["x"])
    b.cleanup()
    c.cleanup()
