"""Build the GB300 shared libraries in-tree (nvcc, sm_103a only).

    python -m osqp_gb300.build            # both precisions, in parallel

Outputs (git-ignored, next to this file):
    osqp_gb300/lib/libosqp_gb300.so                OSQP public API + batch engine, OSQPFloat = float
    osqp_gb300/lib/libosqp_gb300_f64.so            the same with OSQPFloat = double
    osqp_gb300/lib/libosqp_gb300_algebra.so        algebra / linear-system ABI (drop-in for the
                                                   reference's algebra/cuda), OSQPFloat = float
    osqp_gb300/lib/libosqp_gb300_algebra_f64.so    the same with OSQPFloat = double
Each translation unit is compiled once per precision; all compilations run
concurrently and are skipped when the object is newer than its sources.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "lib")
INCLUDE = os.path.join(REPO, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-std=c++17", "-O3", "-lineinfo", "--extended-lambda", "-Xcompiler", "-fPIC",
           "-I" + INCLUDE, "-I" + CSRC]

VARIANTS = {
    "f32": {"defines": ["-DOSQP_USE_FLOAT"]},
    "f64": {"defines": []},
}
# library -> (precision variant, translation units)
TARGETS = {
    "libosqp_gb300.so": ("f32", ["engine.cu", "polish.cu", "batch.cu"]),
    "libosqp_gb300_f64.so": ("f64", ["engine.cu", "polish.cu", "batch.cu"]),
    "libosqp_gb300_algebra.so": ("f32", ["algebra.cu"]),
    "libosqp_gb300_algebra_f64.so": ("f64", ["algebra.cu"]),
}
SOURCES = sorted({s for _, srcs in TARGETS.values() for s in srcs})


def nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _deps():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _compile(src, variant):
    obj = os.path.join(OBJ, variant, os.path.splitext(src)[0] + ".o")
    os.makedirs(os.path.dirname(obj), exist_ok=True)
    if not _stale(obj, _deps()):
        return obj, ""
    cmd = [nvcc()] + ARCH + NVFLAGS + VARIANTS[variant]["defines"] + ["-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src} [{variant}]:\n{r.stderr[-6000:]}")
    return obj, r.stderr


def build(verbose: bool = False) -> dict:
    os.makedirs(LIB, exist_ok=True)
    jobs = sorted({(src, v) for v, srcs in TARGETS.values() for src in srcs})
    objs = {}
    with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
        futs = {ex.submit(_compile, s, v): (s, v) for s, v in jobs}
        for f in cf.as_completed(futs):
            key = futs[f]
            obj, log = f.result()
            objs[key] = obj
            if verbose and log:
                print(log)
    out = {}
    for name, (v, srcs) in TARGETS.items():
        lib = os.path.join(LIB, name)
        deps = [objs[(s, v)] for s in srcs]
        if _stale(lib, deps):
            cmd = [nvcc()] + ARCH + ["-shared", "-Xlinker", "-Bsymbolic", "-o", lib] + deps + ["-lcudart"]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"link failed for {lib}:\n{r.stderr[-4000:]}")
        out[name] = lib
    return out


if __name__ == "__main__":
    libs = build(verbose="-v" in sys.argv)
    for k, v in libs.items():
        print(k, v)
