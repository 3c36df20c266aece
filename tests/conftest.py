"""Shared fixtures.  `-m gpu` tests need a CUDA device; everything else runs on CPU."""
import os
import subprocess
import sys

import numpy as np
import pytest
import scipy.sparse as sp

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, REPO)
GOLDEN = os.path.join(REPO, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


@pytest.fixture(scope="session")
def oracle_lib():
    """FP64 CPU oracle (test infrastructure), built from oracle/ if needed."""
    from osqp_gb300.api import Library
    path = os.path.join(REPO, "oracle", "_build", "liboracle.so")
    src = os.path.join(REPO, "oracle", "osqp_oracle.c")
    if not os.path.exists(path) or os.path.getmtime(path) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle"), "port"], check=True)
    return Library(path, 64)


def reference_dir():
    """Location of the reference sources as oracle/Makefile resolves it
    (OSQP_REFERENCE_DIR overrides), or "" when they are absent."""
    r = subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle"), "refdir"], capture_output=True, text=True)
    return r.stdout.strip() if r.returncode == 0 else ""


@pytest.fixture(scope="session")
def ref_tests():
    return np.load(os.path.join(GOLDEN, "ref_tests.npz"))


@pytest.fixture(scope="session")
def ref_outputs():
    return np.load(os.path.join(GOLDEN, "ref_outputs.npz"))


def csc_from(d, prefix):
    return sp.csc_matrix((d[prefix + "/data"], d[prefix + "/indices"], d[prefix + "/indptr"]),
                         shape=tuple(d[prefix + "/shape"]))


def problem_from(d, name, data_prefix=None):
    pre = data_prefix or name
    P = csc_from(d, f"{pre}/P")
    A = csc_from(d, f"{pre}/A")
    return P, np.asarray(d[f"{pre}/q"]), A, np.asarray(d[f"{pre}/l"]), np.asarray(d[f"{pre}/u"])


@pytest.fixture(scope="session")
def gpu_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
