"""Build the GB300 shared libraries in-tree (nvcc, sm_103a only).

    python -m osqp_gb300.build            # both precisions, in parallel

Outputs (git-ignored, next to this file):
    osqp_gb300/lib/libosqp_gb300.so        OSQPFloat = float  (the reference CUDA default)
    osqp_gb300/lib/libosqp_gb300_f64.so    OSQPFloat = double
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

# translation units of each library
SOURCES = ["engine.cu", "polish.cu", "batch.cu", "algebra.cu"]

VARIANTS = {
    "f32": {"defines": ["-DOSQP_USE_FLOAT"], "lib": "libosqp_gb300.so"},
    "f64": {"defines": [], "lib": "libosqp_gb300_f64.so"},
}


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


def build(verbose: bool = False, sources=None) -> dict:
    sources = [s for s in (sources or SOURCES) if os.path.exists(os.path.join(CSRC, s))]
    os.makedirs(LIB, exist_ok=True)
    jobs = [(s, v) for v in VARIANTS for s in sources]
    objs = {v: [] for v in VARIANTS}
    with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
        futs = {ex.submit(_compile, s, v): (s, v) for s, v in jobs}
        for f in cf.as_completed(futs):
            s, v = futs[f]
            obj, log = f.result()
            objs[v].append(obj)
            if verbose and log:
                print(log)
    out = {}
    for v, spec in VARIANTS.items():
        lib = os.path.join(LIB, spec["lib"])
        if _stale(lib, objs[v]):
            cmd = [nvcc()] + ARCH + ["-shared", "-Xlinker", "-Bsymbolic", "-o", lib] + sorted(objs[v]) + ["-lcudart"]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"link failed for {lib}:\n{r.stderr[-4000:]}")
        out[v] = lib
    return out


if __name__ == "__main__":
    libs = build(verbose="-v" in sys.argv)
    for k, v in libs.items():
        print(k, v)
