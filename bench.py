"""Benchmark: QP solves/s of the batched GB300 OSQP engine on batched linear MPC.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--count 4096] [--precision f64|f32] [--config mpc_batch|large_sparse|svm]

Workload (default, "mpc_batch"): 4096 seeded linear-MPC QPs of uneven size
(horizon T~U{10..50}, nx~U{8..40}, nu~U{4..16}; stacked sparse OSQP form,
int32 indices).  One step is one receding-horizon round: every QP receives a
new initial state x0 (new l, u) and is solved from a cold start to eps_abs =
eps_rel = 1e-3 with the direct KKT solver.  The QP structures are set up once,
outside the timed region, as an MPC controller would.

  value   QPs solved per second with the new bounds already in HBM (device
          time of update + solve, CUDA events on the library's stream), in
          --precision: f64 (default) follows the builtin algorithm's
          trajectory; f32 runs FP32 iterates and factors with double-float
          reductions (`other_precision` reports the other one, one step)
  e2e     the same through the public C API from pinned host memory: the
          new l, u are copied in and x plus the statuses copied out inside
          the timed region (host wall clock around synchronous calls)
  roofline  algorithmic bytes of the solve kernel (osqp_gb300/roofline.py)
            over its CUDA-event time, against the measured HBM copy peak
  cpu_baseline  the FP64 CPU oracle (OSQP's builtin algebra restated; direct
            LDL^T KKT solver) on the machine's host cores, process pool, over
            every QP of the workload, through the same sequence of steps
  parity_vs_fp64_oracle  per-QP status, objective and iteration agreement
            with that oracle on the first timed step

--config large_sparse / svm run the single-QP configurations instead of the
batch (one JSON line each, not the default line): the n=50k / m=100k sparse QP
through the PCG path (ADMM / PCG iterations per second, achieved GB/s), and the
m=100k x 1000 SVM at eps 1e-5 with polish (FP32 ADMM + FP64 polish, the FP64
GPU path and the FP64 CPU oracle, objective and residual errors).

--impl reference prints the CPU reference arm (the oracle port on all host
cores) on the same workload.  With --gpus N > 1 (torchrun) every rank solves
its own contiguous share of the QP set (weak scaling) and rank 0 reports the
aggregate.
"""
from __future__ import annotations

import argparse
import json
import multiprocessing as mp
import os

# Independent launches on separate streams (the served form) must not share
# hardware queues behind long-running kernels: the default of 8 connections
# serialised concurrent launches.  Set before the CUDA context exists.
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")
import subprocess
import sys
import tempfile
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

from osqp_gb300 import problems as pb  # noqa: E402
from osqp_gb300.roofline import solve_bytes, direct_solve_bytes, pfull_nnz  # noqa: E402
from osqp_gb300.api import BLOCK_DIAGONAL_PRECONDITIONER  # noqa: E402

SETTINGS = dict(rho=0.1, sigma=1e-6, alpha=1.6, scaling=10, eps_abs=1e-3, eps_rel=1e-3, rho_is_vec=1,
                check_termination=5, adaptive_rho_tolerance=5.0, max_iter=4000, check_dualgap=1,
                warm_starting=0, polishing=0, linsys_solver=1)


def _nx_of(A):
    rowlen = np.diff(A.tocsr().indptr)
    return int(np.argmax(rowlen != 1))


def make_workload(count, steps, seed=3, share=0):
    """QPs share*count .. (share+1)*count - 1 of the seeded MPC set (a rank's
    contiguous share under --gpus N) and their bounds for `steps` steps."""
    probs = pb.mpc_batch(count, seed=seed, start=share * count)
    nxs = [_nx_of(p[2]) for p in probs]
    ls, us = [], []
    for s in range(steps):
        rg = np.random.default_rng([seed, 7919, s, share])
        lrow, urow = [], []
        for (P, q, A, l, u), nx in zip(probs, nxs):
            l2, u2 = pb.mpc_x0_bounds(l, u, rg.uniform(-1.0, 1.0, nx))
            lrow.append(l2); urow.append(u2)
        ls.append(np.concatenate(lrow)); us.append(np.concatenate(urow))
    return probs, ls, us


# DRAM bytes per algorithmic byte of the solve launch, from one ncu capture
# of a smaller batch of the same QPs (the 4096-QP launch is too long to
# capture); the launch's traffic is this ratio times its algorithmic bytes.
# Direct solver, FP64: 304 QPs, 65.54 + 2.67 GB DRAM for 108.06 GB
# algorithmic.  The PCG path and the FP32 direct path are not captured.
TRAFFIC_PER_ALGORITHMIC_BYTE = {("direct", "f64"): (65.542542 + 2.668631) / 108.057547680}
# The same for the single large sparse QP (PCG, grid form), from one ncu
# capture of each precision's timed solve: FP32 45.03 + 6.93 MB DRAM for
# 31.22 GB algorithmic (the QP stays in L2), FP64 16.09 + 4.51 GB for 19.41 GB.
TRAFFIC_SINGLE = {("large_sparse", "f32"): (45.033472e6 + 6.934528e6) / 31.22e9,
                  ("large_sparse", "f64"): (16.087259e9 + 4.507228e9) / 19.41e9}


def measured_peak():
    path = os.path.join(REPO, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self):
        self.proc = None
        # the raw samples (one CSV line per 200 ms); the JSON line carries the summary
        self.path = os.environ.get("OSQP_GB300_CLOCKS_CSV",
                                   os.path.join(tempfile.gettempdir(), "osqp_gb300_bench_clocks.csv"))

    def start(self):
        os.makedirs(os.path.dirname(self.path), exist_ok=True)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1])); mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm_, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm_)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons)}


# ---------------------------------------------------------------------------
# CPU oracle arm (the reference's builtin algorithm, FP64, direct LDL^T)
# ---------------------------------------------------------------------------
def _cpu_worker(args):
    lib_path, probs, lsteps, usteps, settings, keep = args
    from osqp_gb300.api import Library, OSQP, DIRECT_SOLVER
    lib = Library(lib_path, 64)
    solvers = []
    st = dict(settings)
    st["linsys_solver"] = DIRECT_SOLVER
    for (P, q, A, l, u) in probs:
        s = OSQP(lib)
        s.setup(P, q, A, l, u, **st)
        solvers.append(s)
    per_step, first = [], None
    for ls, us in zip(lsteps, usteps):
        objs = []
        t0 = time.perf_counter()
        for s, l, u in zip(solvers, ls, us):
            s.update(l=l, u=u)
            r = s.solve()
            objs.append((r.info["status_val"], r.info["obj_val"], r.info["iter"]))
        per_step.append(time.perf_counter() - t0)
        if len(per_step) == keep + 1:
            first = objs
    return per_step, len(solvers), first


def cpu_arm(probs, ls, us, sizes_m, steps_timed, steps_warm=0):
    """The FP64 oracle (OSQP's builtin algorithm: direct LDL' KKT solve) on all
    host cores: every QP of the workload, one process per core, each owning a
    contiguous share of the QPs (set up once, untimed).  A step updates every
    QP's bounds and solves it; the step's time is the slowest process's.
    Returns solves/s over the timed steps, the step time and, per QP, the
    first timed step's (status, objective, iterations)."""
    lib_path = os.path.join(REPO, "oracle", "_build", "liboracle.so")
    if not os.path.exists(lib_path):
        subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle"), "port"], check=True)
    cores = os.cpu_count() or 1
    moff = np.concatenate([[0], np.cumsum(sizes_m)])
    count = len(probs)
    # contiguous shares balanced by size (nonzeros of A)
    work = np.array([p[2].nnz for p in probs], dtype=np.float64)
    cuts = np.searchsorted(np.cumsum(work), np.linspace(0, work.sum(), cores + 1)[1:-1])
    chunks = [list(c) for c in np.split(np.arange(count), cuts) if len(c)]
    nsteps = steps_warm + steps_timed
    tasks = []
    for ch in chunks:
        pp = [probs[i] for i in ch]
        lst = [[ls[s][moff[i]:moff[i + 1]] for i in ch] for s in range(nsteps)]
        ust = [[us[s][moff[i]:moff[i + 1]] for i in ch] for s in range(nsteps)]
        tasks.append((lib_path, pp, lst, ust, dict(SETTINGS), steps_warm))
    ctx = mp.get_context("spawn")
    with ctx.Pool(len(tasks)) as pool:
        res = pool.map(_cpu_worker, tasks)
    step_s = [max(r[0][s] for r in res) for s in range(steps_warm, nsteps)]
    first = {}
    for ch, r in zip(chunks, res):
        for i, o in zip(ch, r[2]):
            first[i] = o
    total = float(np.sum(step_s))
    return {"value": count * steps_timed / total, "cores": len(tasks), "ms_per_step": 1e3 * total / steps_timed,
            "sample": f"all {count} MPC QPs x {steps_timed} step(s) (every QP of the step)",
            "first": first, "step_s": step_s}


# ---------------------------------------------------------------------------
# Replicas (--gpus N): one process per GPU, no data-path collective; the host
# side only synchronises the timed region and takes the slowest rank's time.
# ---------------------------------------------------------------------------
def replica_group(world):
    """torch.distributed over gloo for N > 1 replicas (None for one process)."""
    if world <= 1:
        return None
    import torch.distributed as dist
    if not dist.is_initialized():
        dist.init_process_group("gloo")
    return dist


def max_over_ranks(vals, dist):
    """Element-wise maximum of a float64 vector over all ranks."""
    vals = np.asarray(vals, dtype=np.float64)
    if dist is None:
        return vals
    import torch
    t = torch.from_numpy(vals.copy())
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return t.numpy()


def whole_job_rate(units_per_rank, world, max_seconds):
    """Units processed by all ranks over the slowest rank's time."""
    return units_per_rank * world / max_seconds


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def gpu_arm(args, probs, ls, us):
    import torch
    from osqp_gb300 import load
    from osqp_gb300.api import Batch, OSQP

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    prec = args.precision
    lib = load(prec)
    npf, tpf, w = (np.float32, torch.float32, 4) if prec == "f32" else (np.float64, torch.float64, 8)
    settings = dict(SETTINGS, device=local)
    b = Batch(lib)
    rc = b.setup(probs, **settings)
    assert rc == 0, f"batch setup failed: {rc}"
    tile = b.autotune(60)      # SpMV tile (entries per lane), timed on a sample; state restored
    count = b.count
    K, W = args.steps, args.warmup
    nsteps = K + W
    # bounds of every step resident in HBM (device path) and pinned on the host (e2e path)
    dev_l = [torch.from_numpy(ls[s].astype(npf)).to(f"cuda:{local}") for s in range(nsteps)]
    dev_u = [torch.from_numpy(us[s].astype(npf)).to(f"cuda:{local}") for s in range(nsteps)]
    pin_l = [torch.from_numpy(ls[s].astype(npf)).pin_memory() for s in range(nsteps)]
    pin_u = [torch.from_numpy(us[s].astype(npf)).pin_memory() for s in range(nsteps)]
    x_out = torch.empty(b.nsum, dtype=tpf).pin_memory()
    torch.cuda.synchronize()

    dist = replica_group(world)

    def barrier():
        if dist is not None:
            dist.barrier()

    # ---- device-resident path ----
    for s in range(W):
        b.update_ptr(l_ptr=dev_l[s].data_ptr(), u_ptr=dev_u[s].data_ptr())
        b.solve()
    clocks = ClockSampler()
    barrier(); torch.cuda.synchronize()
    clocks.start()
    step_ms, solve_ms, bytes_alg = [], [], 0.0
    first = None
    direct = SETTINGS["linsys_solver"] == 1
    felems = b.factor_elems() if direct else None
    admm_tot = pcg_tot = 0
    nnz_pf = [pfull_nnz(p[0]) for p in probs]
    launches = 0
    for s in range(W, nsteps):
        rc1 = b.update_ptr(l_ptr=dev_l[s].data_ptr(), u_ptr=dev_u[s].data_ptr())
        rc2 = b.solve()
        assert rc1 == 0 and rc2 == 0, (rc1, rc2)
        launches += 4  # bounds check, update, solve, info kernels
        step_ms.append(b.step_ms())
        st = b.stats()
        solve_ms.append(st["kernel_ms"])
        sol = b.solution()
        if first is None:   # step W: the step the CPU oracle solves
            first = {"status": sol["status"].copy(), "obj": sol["obj"].copy(), "iter": sol["iter"].copy()}
        pcg = b.pcg_iters()
        rup = b.rho_updates() if direct else None
        admm_tot += int(sol["iter"].sum()); pcg_tot += int(pcg.sum())
        for k, (P, q, A, l, u) in enumerate(probs):
            if direct:
                bytes_alg += direct_solve_bytes(P.shape[0], A.shape[0], nnz_pf[k], A.nnz, w, int(sol["iter"][k]),
                                                int(felems[k]), int(rup[k]), SETTINGS["check_termination"])
            else:
                bytes_alg += solve_bytes(P.shape[0], A.shape[0], nnz_pf[k], A.nnz, w, int(sol["iter"][k]),
                                         int(pcg[k]), SETTINGS["check_termination"],
                                         SETTINGS.get("cg_precond", 1) == BLOCK_DIAGONAL_PRECONDITIONER)
    torch.cuda.synchronize(); barrier()
    clk = clocks.stop()
    status_last = sol["status"].copy()
    obj_last = sol["obj"].copy()
    dev_total_ms = float(np.sum(step_ms))

    # ---- end-to-end path through the C API from pinned host memory ----
    barrier(); torch.cuda.synchronize()
    t0 = time.perf_counter()
    st_host = np.zeros(count, np.int32)
    for s in range(W, nsteps):
        b.update_ptr(l_ptr=pin_l[s].data_ptr(), u_ptr=pin_u[s].data_ptr())
        b.solve()
        b.solution_ptr(x_ptr=x_out.data_ptr())
        st_host = b.statuses()
    torch.cuda.synchronize(); barrier()
    e2e_s = time.perf_counter() - t0

    # ---- max over ranks; per-QP statuses of every rank's share, in order ----
    vals = max_over_ranks([dev_total_ms, e2e_s], dist)
    from osqp_gb300.router import gather_in_order
    status_last = gather_in_order({"status": status_last}, dist)["status"]
    if dist is not None:
        dist.destroy_process_group()
    dev_total_ms, e2e_s = float(vals[0]), float(vals[1])

    # ---- plain one-QP-at-a-time GPU form on a sample (the reference's usage pattern) ----
    plain = None
    if rank == 0 and args.plain_sample > 0:
        # the library picks the execution form for a single QP (CTA, cluster or grid)
        tt = 0.0
        ns = min(args.plain_sample, count)
        moff = np.concatenate([[0], np.cumsum([p[2].shape[0] for p in probs])])
        for k in range(0, count, max(1, count // ns))[:ns]:   # every (count/ns)-th QP
            s1 = OSQP(lib)
            s1.setup(*probs[k], **settings)
            s1.update(l=ls[W][moff[k]:moff[k + 1]], u=us[W][moff[k]:moff[k + 1]])
            t1 = time.perf_counter()
            s1.solve()
            tt += time.perf_counter() - t1
            s1.cleanup()
        plain = ns / tt

    solves = count * K * world
    out = dict(
        value=whole_job_rate(count * K, world, dev_total_ms * 1e-3),
        ms_per_step=dev_total_ms / K,
        e2e_value=whole_job_rate(count * K, world, e2e_s),
        h2d=2 * w * int(b.msum), d2h=w * int(b.nsum) + 40 * count,
        solve_ms=float(np.mean(solve_ms)),
        achieved_gbs=bytes_alg / K / (np.mean(solve_ms) * 1e-3) / 1e9,
        bytes_per_launch=bytes_alg / K,
        admm_per_qp=admm_tot / (count * K), pcg_per_qp=pcg_tot / (count * K),
        status_counts={int(k): int(v) for k, v in zip(*np.unique(status_last, return_counts=True))},
        first=first, launches=launches, clocks=clk, plain=plain, rank=rank, world=world, tile=tile,
        factor_bytes=float(np.sum(felems)) * w if direct else None,
    )
    b.cleanup()
    return out


def precision_leg(prec, probs, ls, us, W):
    """The batched direct solve in the other precision on the same QPs and
    step sequence: W untimed steps, then one timed step (device time)."""
    from osqp_gb300 import load
    from osqp_gb300.api import Batch
    b = Batch(load(prec))
    assert b.setup(probs, **dict(SETTINGS)) == 0
    for s in range(W):
        b.update(l=ls[s], u=us[s]); b.solve()
    b.update(l=ls[W], u=us[W]); b.solve()
    ms = b.step_ms()
    st = b.stats()
    sol = b.solution()
    b.cleanup()
    return {"precision": prec, "solves_per_s": len(probs) / (ms * 1e-3), "ms_per_step": ms,
            "admm_iters_per_qp": st["admm_iter"] / len(probs),
            "first": {"status": sol["status"].copy(), "obj": sol["obj"].copy(), "iter": sol["iter"].copy()}}


def parity(first, cpu, count):
    """Per-QP status, objective and ADMM iteration agreement with the oracle's
    results of the same step."""
    st_g, st_o = first["status"], np.array([cpu["first"][i][0] for i in range(count)])
    errs, ratio = [], []
    for i in range(count):
        if st_o[i] == 1 and st_g[i] == 1:
            oo = cpu["first"][i][1]
            errs.append(abs(float(first["obj"][i]) - oo) / max(1.0, abs(oo)))
            ratio.append(float(first["iter"][i]) / max(1, cpu["first"][i][2]))
    errs, ratio = np.array(errs), np.array(ratio)
    return {"qps": count, "status_mismatches": int(np.sum(st_g != st_o)),
            "objective_rel_err": {"max": float(errs.max()), "p99": float(np.percentile(errs, 99)),
                                  "median": float(np.median(errs)),
                                  "fraction_le_1e-4": float(np.mean(errs <= 1e-4))},
            "admm_iteration_ratio": {"median": float(np.median(ratio)),
                                     "fraction_equal": float(np.mean(ratio == 1.0)),
                                     "fraction_within_10pct": float(np.mean(np.abs(ratio - 1) <= 0.1))},
            "oracle_admm_iters_per_qp": float(np.mean([cpu["first"][i][2] for i in range(count)])),
            "against": "FP64 oracle, builtin algorithm (direct LDL' KKT solve): same QPs, same sequence of "
                       "bound updates and solves (its rho state carried from step to step as on the GPU), "
                       "the first timed step compared"}


def indirect_leg(probs, ls, us, W):
    """The PCG path (the reference CUDA backend's algorithm) on the same
    batch: one warm-up and one timed step, device time."""
    from osqp_gb300 import load
    from osqp_gb300.api import Batch
    b = Batch(load("f32"))
    assert b.setup(probs, **dict(SETTINGS, linsys_solver=2)) == 0
    b.update(l=ls[0], u=us[0]); b.solve()
    b.update(l=ls[W], u=us[W]); b.solve()
    ms = b.step_ms()
    st = b.stats()
    sol = b.solution()
    b.cleanup()
    return {"solves_per_s": len(probs) / (ms * 1e-3), "ms_per_step": ms, "admm_iters_per_qp": st["admm_iter"] / len(probs),
            "pcg_iters_per_qp": st["pcg_iter"] / len(probs),
            "status_counts": {int(k): int(v) for k, v in zip(*np.unique(sol["status"], return_counts=True))}}


# ---------------------------------------------------------------------------
# Single-QP configurations
# ---------------------------------------------------------------------------
def _host_residuals(data, x, y):
    import scipy.sparse as sp
    P, q, A, l, u = data
    Pu = P.tocsc()
    Pf = Pu + sp.triu(Pu, 1).T
    Ax = A @ x
    z = np.clip(Ax, l, u)
    prim = float(np.max(np.abs(Ax - z))) if A.shape[0] else 0.0
    dual = float(np.max(np.abs(Pf @ x + q + A.T @ y)))
    obj = float(0.5 * x @ (Pf @ x) + q @ x)
    return obj, prim, dual


def _oracle_job(args_):
    lib_path, data, settings, linsys = args_
    from osqp_gb300.api import Library, OSQP
    s = OSQP(Library(lib_path, 64))
    P, q, A, l, u = data
    s.setup(P, q, A, pb.clip_inf(l, 1e30), pb.clip_inf(u, 1e30), **dict(settings, linsys_solver=linsys))
    t = time.perf_counter()
    r = s.solve()
    return time.perf_counter() - t, r.x, r.y, r.info["status"], r.info["iter"], r.info["status_polish"]


def single_config(args):
    print(json.dumps(single_config_result(args.config, args.oracle_timeout)))


def single_config_result(which, oracle_timeout):
    """One single-QP configuration on GPU 0 (FP32 and FP64 paths) and, within
    oracle_timeout seconds, the FP64 CPU oracle."""
    import torch
    from osqp_gb300 import load
    from osqp_gb300.api import OSQP, DIRECT_SOLVER, INDIRECT_SOLVER
    torch.cuda.set_device(0)
    if which == "large_sparse":
        data = pb.large_sparse()
        st = dict(SETTINGS, warm_starting=0, polishing=0, linsys_solver=INDIRECT_SOLVER)
        oracle_linsys = INDIRECT_SOLVER
        desc = "large_sparse: n=50,000, m=100,000, P=MM'+1e-2I (8 nnz/col of M), A 10 nnz/row, eps 1e-3"
    else:
        data = pb.svm()
        st = dict(SETTINGS, eps_abs=1e-5, eps_rel=1e-5, warm_starting=0, polishing=1, max_iter=20000,
                  linsys_solver=INDIRECT_SOLVER)
        oracle_linsys = DIRECT_SOLVER
        desc = "svm: m=100,000 samples x 1,000 features, 15% density, lambda=1, eps 1e-5, polish"
    P, q, A, l, u = data
    n, m = P.shape[0], A.shape[0]
    nnz_pf = pfull_nnz(P)
    peak, peak_kind = measured_peak()
    out = {"config": {"workload": desc, "n": n, "m": m, "nnz_P_full": nnz_pf, "nnz_A": int(A.nnz)},
           "data": "synthetic (seeded)", "paths": {}}
    for prec, inf, w in (("f32", 1e17, 4), ("f64", 1e30, 8)):
        solver = OSQP(load(prec))
        assert solver.setup(P, q, A, pb.clip_inf(l, inf), pb.clip_inf(u, inf), **st) == 0
        solver.solve()                       # warm-up (cold solves: warm_starting=0)
        torch.cuda.synchronize()
        t = time.perf_counter()
        r = solver.solve()
        wall = time.perf_counter() - t
        stt = solver.stats()
        obj, prim, dual = _host_residuals(data, r.x, r.y)
        kms = stt["kernel_ms"]
        byt = solve_bytes(n, m, nnz_pf, A.nnz, w, stt["admm_iter"], stt["pcg_iter"], st["check_termination"],
                          st.get("cg_precond", 1) == BLOCK_DIAGONAL_PRECONDITIONER)
        out["paths"][prec] = {
            "status": r.info["status"], "status_polish": r.info["status_polish"], "admm_iter": stt["admm_iter"],
            "pcg_iter": stt["pcg_iter"], "solve_kernel_ms": kms, "solve_wall_ms": wall * 1e3,
            "polish_ms": r.info["polish_time"] * 1e3,
            "admm_iters_per_s": stt["admm_iter"] / (kms * 1e-3), "pcg_iters_per_s": stt["pcg_iter"] / (kms * 1e-3),
            "execution_form": {0: "cta", 1: "grid"}.get(stt["grid"], f"cluster{stt['grid']}"),
            "roofline": {"bound": "hbm", "achieved": byt / (kms * 1e-3) / 1e9, "peak": peak, "unit": "GB/s",
                         "frac": byt / (kms * 1e-3) / 1e9 / peak, "peak_source": peak_kind,
                         "traffic": (TRAFFIC_SINGLE[(which, prec)] * byt) if (which, prec) in TRAFFIC_SINGLE else None,
                         "traffic_source": ("ncu capture of this solve (dram read+write / algorithmic bytes = "
                                            f"{TRAFFIC_SINGLE[(which, prec)]:.4f})")
                         if (which, prec) in TRAFFIC_SINGLE else "not captured"},
            "obj": obj, "prim_res": prim, "dual_res": dual}
        solver.cleanup()
    if oracle_timeout > 0:
        lib_path = os.path.join(REPO, "oracle", "_build", "liboracle.so")
        if not os.path.exists(lib_path):
            subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle"), "port"], check=True)
        ctx = mp.get_context("spawn")
        with ctx.Pool(1) as pool:
            job = pool.apply_async(_oracle_job, ((lib_path, data, st, oracle_linsys),))
            try:
                secs, xo, yo, status, it, spol = job.get(timeout=oracle_timeout)
                obj, prim, dual = _host_residuals(data, xo, yo)
                out["oracle"] = {"kind": "direct LDL^T (builtin)" if oracle_linsys == DIRECT_SOLVER else
                                 "reduced-KKT PCG (FP64 restatement of the CUDA backend)", "status": status,
                                 "iter": it, "status_polish": spol, "cpu_s": secs, "cores": 1,
                                 "obj": obj, "prim_res": prim, "dual_res": dual}
                for prec, pth in out["paths"].items():
                    pth["obj_rel_err_vs_oracle"] = abs(pth["obj"] - obj) / max(1.0, abs(obj))
            except mp.TimeoutError:
                out["oracle"] = {"unavailable": f"FP64 CPU oracle did not finish within {oracle_timeout:.0f} s"}
                pool.terminate()
    ref = out["paths"]["f64"]["obj"]
    out["paths"]["f32"]["obj_rel_err_vs_f64_gpu"] = abs(out["paths"]["f32"]["obj"] - ref) / max(1.0, abs(ref))
    if oracle_timeout <= 0:
        out["oracle"] = {"unavailable": "not run in this invocation (python bench.py --config " + which +
                                        " runs it, with --oracle-timeout seconds)"}
    return out


# ---------------------------------------------------------------------------
# Served form: Poisson request stream over resident pools (continuous batching)
# ---------------------------------------------------------------------------
def serve_leg(args, rate=None, seconds=None):
    """50% MPC and 50% factor-model portfolio requests from `streams` recurring
    problems each, Poisson arrivals at `rate` req/s for `seconds`.  Each
    stream's data drift between its requests: an MPC stream's measured state
    x0 follows a random walk (step N(0, 0.05) per request, clipped to [-1, 1])
    -> new bounds; a portfolio stream's mean returns drift (x (1 + 0.02 N(0,1)))
    -> new q.  Every stream keeps its structure, scaling and warm-start iterates
    resident.  Latency = submission to results on the host."""
    import threading
    from osqp_gb300 import load
    from osqp_gb300.api import Batch, Server
    lib = load(args.precision)
    S = args.serve_streams
    mpc = pb.mpc_batch(S, seed=11)
    port = [pb.portfolio(seed=20000 + i) for i in range(S)]
    st = dict(SETTINGS, warm_starting=1)
    pools = []
    # both classes take the configured solver: MPC QPs the block-tridiagonal
    # direct solve, portfolio QPs (a budget row and factor rows over every
    # asset) its diagonal-plus-dense-rows form
    for probs, ls_ in ((mpc, SETTINGS["linsys_solver"]), (port, SETTINGS["linsys_solver"])):
        b = Batch(lib)
        assert b.setup(probs, **dict(st, linsys_solver=ls_)) == 0, "pool set-up refused"
        pools.append(b)
    srv = Server(lib, concurrency=args.serve_concurrency)
    pid = [srv.add_pool(b) for b in pools]
    nxs = [_nx_of(p[2]) for p in mpc]
    rg = np.random.default_rng([11, 3])
    rate = args.serve_rate if rate is None else rate
    seconds = args.serve_seconds if seconds is None else seconds
    n_req = int(rate * seconds)
    t_arr = np.cumsum(rg.exponential(1.0 / rate, n_req))
    kind = rg.integers(0, 2, n_req)
    which = rg.integers(0, S, n_req)
    payload = []
    x0 = [-mpc[i][3][:nxs[i]].copy() for i in range(S)]     # each MPC stream's current state
    for k, i in zip(kind, which):
        if k == 0:
            P, q, A, l, u = mpc[i]
            x0[i] = np.clip(x0[i] + 0.05 * rg.standard_normal(nxs[i]), -1.0, 1.0)
            l2, u2 = pb.mpc_x0_bounds(l, u, x0[i])
            payload.append((pid[0], int(i), None, l2, u2, P.shape[0]))
        else:
            P, q, A, l, u = port[i]
            q2 = q * (1.0 + 0.02 * rg.standard_normal(q.size))
            payload.append((pid[1], int(i), q2, None, None, P.shape[0]))
    # warm-up: one request per stream (cold start of every stream), untimed
    for j, probs in enumerate((mpc, port)):
        ts = [srv.submit(pid[j], i) for i in range(S)]
        for i, t in enumerate(ts):
            srv.wait(t, probs[i][0].shape[0])
    tickets = [None] * n_req
    t0 = time.perf_counter()

    def submitter():
        for r in range(n_req):
            dt = t0 + t_arr[r] - time.perf_counter()
            if dt > 0:
                time.sleep(dt)
            pl, i, q2, l2, u2, _ = payload[r]
            tickets[r] = srv.submit(pl, i, q2, l2, u2)

    th = threading.Thread(target=submitter)
    th.start()
    lat, stat, its = np.zeros(n_req), np.zeros(n_req, np.int32), np.zeros(n_req, np.int32)
    for r in range(n_req):
        while tickets[r] is None:
            time.sleep(1e-5)
        _, stat[r], its[r], _, lat[r] = srv.wait(tickets[r], payload[r][5])
    elapsed = time.perf_counter() - t0
    th.join()
    srv.close()
    for b in pools:
        b.cleanup()
    mk = kind == 0
    return {"rate_rps": rate, "seconds": seconds, "requests": n_req, "drained_s": elapsed,
            "streams": {"mpc": S, "portfolio": S}, "concurrency": args.serve_concurrency,
            "solves_per_s": n_req / elapsed, "p50_ms": float(np.percentile(lat, 50)),
            "p99_ms": float(np.percentile(lat, 99)), "p50_ms_mpc": float(np.percentile(lat[mk], 50)),
            "p99_ms_mpc": float(np.percentile(lat[mk], 99)),
            "p50_ms_portfolio": float(np.percentile(lat[~mk], 50)),
            "p99_ms_portfolio": float(np.percentile(lat[~mk], 99)),
            "admm_iters_mean": float(its.mean()), "admm_iters_mean_mpc": float(its[mk].mean()),
            "admm_iters_mean_portfolio": float(its[~mk].mean()),
            "status_counts": {int(k): int(v) for k, v in zip(*np.unique(stat, return_counts=True))}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--count", type=int, default=4096)
    ap.add_argument("--plain-sample", type=int, default=64)
    ap.add_argument("--serve-rate", type=float, default=50.0, help="served form: Poisson arrivals (req/s); 0 = skip")
    ap.add_argument("--serve-seconds", type=float, default=6.0)
    ap.add_argument("--serve-config-rate", type=float, default=2000.0,
                    help="served form: also one second of Poisson arrivals at this rate (0 = skip)")
    ap.add_argument("--serve-streams", type=int, default=128, help="recurring problems per class")
    ap.add_argument("--serve-concurrency", type=int, default=32, help="launches in flight")
    ap.add_argument("--config", default="mpc_batch", choices=["mpc_batch", "large_sparse", "svm"])
    ap.add_argument("--oracle-timeout", type=float, default=900.0,
                    help="single-QP configs: seconds allowed for the FP64 CPU oracle (0 = skip)")
    ap.add_argument("--max-iter", type=int, default=SETTINGS["max_iter"],
                    help="ADMM iteration cap (smaller values give short profiling cases)")
    ap.add_argument("--precond", default="diagonal", choices=["diagonal", "block"],
                    help="PCG preconditioner: OSQP's diagonal (Jacobi) one or the 32 x 32 block-Jacobi one")
    ap.add_argument("--linsys", default="direct", choices=["direct", "indirect"],
                    help="linear-system solver of the batched engine (direct: block-tridiagonal LDL'; "
                         "indirect: the reduced-KKT PCG)")
    ap.add_argument("--indirect-compare", type=int, default=1, help="also time one step of the PCG path")
    ap.add_argument("--cpu-oracle", type=int, default=1, help="FP64 CPU oracle over every QP of one step")
    ap.add_argument("--precision", default="f64", choices=["f64", "f32"],
                    help="arithmetic of the measured batched solve (f64: the builtin algorithm's trajectory; "
                         "f32: FP32 iterates and factor with double-float reductions)")
    ap.add_argument("--single-configs", type=int, default=1,
                    help="also run the large sparse QP and the SVM (single-QP configurations) as extra keys")
    ap.add_argument("--large-sparse-oracle-timeout", type=float, default=180.0,
                    help="seconds allowed for the FP64 oracle of the large sparse QP in the default run")
    ap.add_argument("--other-precision", type=int, default=1,
                    help="also time one step in the other precision, with its parity")
    args = ap.parse_args()
    SETTINGS["max_iter"] = args.max_iter
    SETTINGS["linsys_solver"] = 1 if args.linsys == "direct" else 2
    if args.precond == "block":
        SETTINGS["cg_precond"] = BLOCK_DIAGONAL_PRECONDITIONER
    if args.config != "mpc_batch":
        single_config(args)
        return
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", str(args.gpus)))
    K, W = args.steps, args.warmup
    config = {"workload": f"mpc_batch: {args.count} linear-MPC QPs (T~U{{10..50}}, nx~U{{8..40}}, nu~U{{4..16}}), "
                          "new x0 per step, cold solve to eps 1e-3",
              "qps_per_step": args.count, "eps": 1e-3, "settings": "rho_is_vec=1, check_termination=5, "
              "adaptive_rho, scaling=10, check_dualgap=1",
              "linsys_solver": args.linsys, "precision": args.precision,
              "preconditioner": ("block-Jacobi 32x32" if args.precond == "block" else "diagonal (Jacobi)") if args.linsys == "indirect" else None,
              "l2": "inputs (~3 GB of CSR data and factors) exceed the 129 MB L2",
              "parallelism": f"data-parallel x{world}: each GPU owns a contiguous share of {args.count} QPs "
                             "(weak scaling), results gathered in order"}
    metric = "QP solves/s (batched MPC, eps 1e-3)"

    if args.impl == "reference":
        if rank != 0:
            return
        probs, ls, us = make_workload(args.count, K + W)
        sizes_m = [p[2].shape[0] for p in probs]
        cpu = cpu_arm(probs, ls, us, sizes_m, steps_timed=K, steps_warm=W)
        line = dict(metric=metric, value=cpu["value"], unit="solves/s", n_gpus=args.gpus, steps=K, warmup=W,
                    ms_per_step=cpu["ms_per_step"], higher_is_better=True, scaling="weak",
                    vs_baseline=None, dtype="f64", data="synthetic (seeded)", config=config, impl="reference",
                    cpu_baseline={"value": cpu["value"], "unit": "solves/s", "cores": cpu["cores"], "kind": "port",
                                  "sample": cpu["sample"]},
                    e2e={"value": cpu["value"], "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
                    step_seconds=cpu["step_s"])
        print(json.dumps(line))
        return

    # each rank owns a contiguous share of count QPs of the whole set (weak
    # scaling: the set grows with the ranks; no data-path collective)
    probs, ls, us = make_workload(args.count, K + W, share=rank)
    g = gpu_arm(args, probs, ls, us)
    if rank != 0:
        return
    direct = SETTINGS["linsys_solver"] == 1
    indirect = indirect_leg(probs, ls, us, W) if (direct and args.indirect_compare) else None
    other = "f32" if args.precision == "f64" else "f64"
    leg2 = precision_leg(other, probs, ls, us, W) if (direct and args.other_precision) else None
    served = serve_leg(args) if args.serve_rate > 0 else None
    # the serving configuration's lowest arrival rate, one second of arrivals
    served_cfg = serve_leg(args, args.serve_config_rate, 1.0) if args.serve_config_rate > 0 else None
    # the two single-QP configurations, as extra keys of this line
    singles = {}
    if args.single_configs:
        singles["large_sparse"] = single_config_result("large_sparse", args.large_sparse_oracle_timeout)
        singles["svm"] = single_config_result("svm", 0)
    peak, peak_kind = measured_peak()
    sizes_m = [p[2].shape[0] for p in probs]
    # the FP64 oracle on the host cores: every QP, through the warm-up steps
    # and the first timed step (same update / solve sequence as the GPU run)
    cpu = cpu_arm(probs, ls[:W + 1], us[:W + 1], sizes_m, steps_timed=1, steps_warm=W) if args.cpu_oracle else None
    par = parity(g["first"], cpu, len(probs)) if cpu else None
    if leg2 is not None:
        first2 = leg2.pop("first")
        leg2["parity_vs_fp64_oracle"] = parity(first2, cpu, len(probs)) if cpu else None
    tr = TRAFFIC_PER_ALGORITHMIC_BYTE.get(("direct" if direct else "indirect", args.precision))
    line = dict(
        metric=metric, value=g["value"], unit="solves/s", n_gpus=world, steps=K, warmup=W,
        ms_per_step=g["ms_per_step"], higher_is_better=True, scaling="weak", vs_baseline=None,
        dtype=("f64" if args.precision == "f64" else "f32 (FP64-accurate double-float reductions)"),
        data="synthetic (seeded)", config=config,
        e2e={"value": g["e2e_value"], "unit": "solves/s", "h2d_bytes_per_step": g["h2d"],
             "d2h_bytes_per_step": g["d2h"]},
        roofline={"bound": "hbm", "achieved": g["achieved_gbs"], "peak": peak, "unit": "GB/s",
                  "frac": g["achieved_gbs"] / peak,
                  "traffic": (tr * g["bytes_per_launch"]) if tr else None,
                  "traffic_source": (f"ncu capture of a smaller batch (dram read+write / algorithmic bytes = {tr:.3f})"
                                     " scaled to this launch's algorithmic bytes") if tr else "not captured",
                  "kernel": "k_batch (solve)", "peak_source": peak_kind,
                  "algorithmic_bytes_per_launch": g["bytes_per_launch"], "kernel_ms": g["solve_ms"],
                  "factor_bytes": g["factor_bytes"]},
        cpu_baseline=None if not cpu else {"value": cpu["value"], "unit": "solves/s", "cores": cpu["cores"],
                                           "kind": "port", "sample": cpu["sample"]},
        clocks=g["clocks"], gpu_launches=g["launches"],
        linsys_solver="direct (block-tridiagonal LDL')" if direct else "indirect (reduced-KKT PCG)",
        arithmetic=("FP64; the direct solver factors in FP64 and runs its block solve in double-float "
                    "(hi + lo floats, 48 significant bits) on the FP32 pipe"
                    if direct and args.precision == "f64" else
                    "FP64" if args.precision == "f64" else
                    "FP32 iterates and factors, double-float reductions, FP64 scalars"),
        plain_gpu_solves_per_s=g["plain"],
        batched_over_plain=(g["value"] / g["plain"]) if g["plain"] else None,
        admm_iters_per_qp=g["admm_per_qp"], pcg_iters_per_qp=g["pcg_per_qp"],
        status_counts=g["status_counts"], parity_vs_fp64_oracle=par,
        other_precision=leg2,
        indirect=indirect,
        spmv_tile_entries_per_lane=g["tile"],
        served=served, served_at_config_rate=served_cfg,
        **singles,
    )
    print(json.dumps(line))


if __name__ == "__main__":
    main()
