"""Regenerate the committed golden fixtures in tests/golden/.

Run in the development container only (it reads the reference tree):

    make -C oracle ref
    python tests/golden/make_golden.py /root/reference

Two kinds of fixtures are written:

  ref_tests.npz   problem data and expected answers of the reference's own
                  test generators (tests/*/generate_problem.py).  The
                  generators are imported from a scratch copy with
                  utils.codegen_utils replaced by a capturing stub, so the
                  numbers are exactly the ones the reference's C++ tests use.
  ref_outputs.npz outputs of the reference itself (oracle/_ref/libosqp_ref.so:
                  the reference's builtin FP64 algebra and C core compiled from
                  its sources) on the reference test problems and on seeded
                  instances of the benchmark workloads, with their problem data.
"""
from __future__ import annotations

import os
import shutil
import sys
import tempfile
import types

import numpy as np
import scipy.sparse as sp

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from osqp_gb300.api import Library, OSQP  # noqa: E402
from osqp_gb300 import problems as pb  # noqa: E402

GENERATORS = ["basic_qp", "basic_qp2", "basic_lp", "unconstrained", "no_active_set",
              "primal_infeasibility", "primal_dual_infeasibility", "non_cvx",
              "solve_linsys", "update_matrices", "lin_alg"]


def _flatten(prefix, value, out):
    if sp.issparse(value):
        M = sp.csc_matrix(value)
        out[prefix + "/indptr"] = M.indptr.astype(np.int64)
        out[prefix + "/indices"] = M.indices.astype(np.int64)
        out[prefix + "/data"] = M.data.astype(np.float64)
        out[prefix + "/shape"] = np.array(M.shape, dtype=np.int64)
    elif isinstance(value, str):
        out[prefix + "/str"] = np.array(value)
    elif isinstance(value, dict):
        for k, v in value.items():
            _flatten(prefix + "/" + str(k), v, out)
    elif isinstance(value, (list, tuple)):
        out[prefix + "/list"] = np.asarray(value)
    else:
        out[prefix] = np.asarray(value)


def capture_reference_tests(ref_root):
    captured = {}
    tmp = tempfile.mkdtemp(prefix="osqp_golden_")
    try:
        for g in GENERATORS:
            os.makedirs(os.path.join(tmp, g))
            shutil.copy(os.path.join(ref_root, "tests", g, "generate_problem.py"),
                        os.path.join(tmp, g, "generate_problem.py"))
        utils = types.ModuleType("utils")
        cu = types.ModuleType("utils.codegen_utils")

        def generate_problem_data(P, q, A, l, u, problem_name, sols_data={}):
            captured[problem_name] = {"P": P, "q": q, "A": A, "l": l, "u": u, "sols": dict(sols_data)}

        def generate_data(problem_name, sols_data):
            captured[problem_name] = {"data": dict(sols_data)}

        cu.generate_problem_data = generate_problem_data
        cu.generate_data = generate_data
        utils.codegen_utils = cu
        sys.modules["utils"] = utils
        sys.modules["utils.codegen_utils"] = cu
        sys.path.insert(0, tmp)
        cwd = os.getcwd()
        for g in GENERATORS:
            os.chdir(os.path.join(tmp, g))
            src = open("generate_problem.py").read()
            exec(compile(src, f"{g}/generate_problem.py", "exec"), {"__name__": f"gen_{g}"})
        os.chdir(cwd)
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    out = {}
    for name, d in captured.items():
        _flatten(name, d, out)
    return out


def ref_settings(**kw):
    base = dict(verbose=0)
    base.update(kw)
    return base


def solve_ref(lib, P, q, A, l, u, settings):
    s = OSQP(lib)
    rc = s.setup(P, q, A, l, u, **settings)
    if rc:
        return {"setup_rc": rc}
    r = s.solve()
    return {"setup_rc": 0, "x": r.x, "y": r.y, "prim_inf_cert": r.prim_inf_cert,
            "dual_inf_cert": r.dual_inf_cert, "status_val": r.info["status_val"],
            "iter": r.info["iter"], "obj_val": r.info["obj_val"],
            "prim_res": r.info["prim_res"], "dual_res": r.info["dual_res"],
            "status_polish": r.info["status_polish"]}


def main(ref_root):
    tests = capture_reference_tests(ref_root)
    np.savez_compressed(os.path.join(HERE, "ref_tests.npz"), **tests)

    lib = Library(os.path.join(REPO, "oracle", "_ref", "libosqp_ref.so"), 64)
    outputs = {}

    # Reference test problems with the reference test-fixture settings
    # (tests/osqp_tester.h:66-80: rho 0.1, alpha 1.6, max_iter 2000, scaling 1,
    # eps 1e-5) for polish off/on.
    names = ["basic_qp", "basic_qp2", "basic_lp", "unconstrained", "no_active_set",
             "primal_infeasibility"]
    for name in names:
        P = sp.csc_matrix((tests[f"{name}/P/data"], tests[f"{name}/P/indices"], tests[f"{name}/P/indptr"]),
                          shape=tuple(tests[f"{name}/P/shape"]))
        A = sp.csc_matrix((tests[f"{name}/A/data"], tests[f"{name}/A/indices"], tests[f"{name}/A/indptr"]),
                          shape=tuple(tests[f"{name}/A/shape"]))
        q, l, u = tests[f"{name}/q"], tests[f"{name}/l"], tests[f"{name}/u"]
        l = pb.clip_inf(l, 1e30)
        u = pb.clip_inf(u, 1e30)
        for pol in (0, 1):
            st = ref_settings(rho=0.1, alpha=1.6, max_iter=2000, scaling=1, eps_abs=1e-5,
                              eps_rel=1e-5, polishing=pol)
            res = solve_ref(lib, P, q, A, l, u, st)
            _flatten(f"{name}/pol{pol}", res, outputs)

    # Seeded benchmark-shaped problems; the settings pin every default that
    # differs between the reference's CPU and CUDA builds.
    pinned = dict(rho=0.1, sigma=1e-6, alpha=1.6, scaling=10, eps_abs=1e-3, eps_rel=1e-3,
                  rho_is_vec=1, check_termination=25, adaptive_rho_tolerance=5.0,
                  max_iter=4000, polishing=0)
    cases = {
        "random_qp_s1": pb.random_qp(1),
        "random_qp_s7": pb.random_qp(7),
        "mpc_s0": pb.mpc(0),
        "mpc_s2": pb.mpc(2),
        "portfolio_s1": pb.portfolio(1, n=150),
    }
    for name, (P, q, A, l, u) in cases.items():
        _flatten(f"{name}/data", {"P": P, "q": q, "A": A, "l": l, "u": u}, outputs)
        for pol in (0, 1):
            st = dict(pinned, polishing=pol)
            _flatten(f"{name}/pol{pol}", solve_ref(lib, P, q, A, l, u, st), outputs)
    np.savez_compressed(os.path.join(HERE, "ref_outputs.npz"), **outputs)
    print("wrote", len(tests), "test arrays and", len(outputs), "reference-output arrays")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
