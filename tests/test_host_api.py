"""Host-only parts of the public API on a machine without a GPU: the CSC
helpers (tests/csc_api/test_csc_api.cpp:7-290) and the settings defaults
(tests/settings/test_settings.cpp:7-30), for both builds of the GB300 library."""
import ctypes as C
import os

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBS = {"f32": ("libosqp_gb300.so", 32), "f64": ("libosqp_gb300_f64.so", 64)}


@pytest.fixture(scope="module", params=sorted(LIBS))
def L(request):
    from osqp_gb300.api import Library
    name, bits = LIBS[request.param]
    path = os.path.join(REPO, "osqp_gb300", "lib", name)
    if not os.path.exists(path):
        pytest.skip(f"{name} not built")
    lib = Library(path, bits)
    P = C.POINTER(lib.CscMatrix)
    f = lib.lib
    f.OSQPCscMatrix_zeros.argtypes = [lib.I, lib.I]
    f.OSQPCscMatrix_zeros.restype = P
    f.OSQPCscMatrix_diag_scalar.argtypes = [lib.I, lib.I, lib.F]
    f.OSQPCscMatrix_diag_scalar.restype = P
    f.OSQPCscMatrix_diag_vec.argtypes = [lib.I, lib.I, C.POINTER(lib.F)]
    f.OSQPCscMatrix_diag_vec.restype = P
    f.OSQPCscMatrix_identity.argtypes = [lib.I]
    f.OSQPCscMatrix_identity.restype = P
    f.OSQPCscMatrix_free.argtypes = [P]
    f.OSQPCscMatrix_free.restype = None
    return lib


def _check(M, m, n, diag):
    """Size, ownership and the arrays of an m x n matrix whose first
    min(m, n) diagonal entries are `diag` (None: no entries at all)."""
    c = M.contents
    assert (c.m, c.n, c.owned) == (m, n, 1)
    k = min(m, n)
    p = [c.p[j] for j in range(n + 1)]
    if diag is None:
        assert p == [0] * (n + 1)
        assert not bool(c.x) and not bool(c.i)
        return
    assert p == [min(j, k) for j in range(n + 1)]
    assert [c.i[j] for j in range(k)] == list(range(k))
    assert [c.x[j] for j in range(k)] == list(diag)


@pytest.mark.parametrize("m,n", [(5, 5), (3, 5), (7, 5)])
def test_csc_zeros(L, m, n):
    M = L.lib.OSQPCscMatrix_zeros(m, n)
    _check(M, m, n, None)
    L.lib.OSQPCscMatrix_free(M)


@pytest.mark.parametrize("m,n", [(5, 5), (4, 7), (5, 4)])
def test_csc_diag_scalar(L, m, n):
    M = L.lib.OSQPCscMatrix_diag_scalar(m, n, 3.0)
    _check(M, m, n, [3.0] * min(m, n))
    L.lib.OSQPCscMatrix_free(M)


@pytest.mark.parametrize("m,n", [(5, 5), (4, 7), (5, 4)])
def test_csc_diag_vec(L, m, n):
    vals = np.arange(1.0, min(m, n) + 1.0).astype(L.np_float)
    M = L.lib.OSQPCscMatrix_diag_vec(m, n, vals.ctypes.data_as(C.POINTER(L.F)))
    _check(M, m, n, list(vals))
    L.lib.OSQPCscMatrix_free(M)


def test_csc_identity(L):
    M = L.lib.OSQPCscMatrix_identity(5)
    _check(M, 5, 5, [1.0] * 5)
    L.lib.OSQPCscMatrix_free(M)


def test_default_settings_fill_every_field(L):
    """Every field is written: a sentinel in each 32-bit word (FP32 build, where
    every field is 4 bytes) or in each field (FP64 build) is gone afterwards."""
    st = L.Settings()
    raw = (C.c_uint32 * (C.sizeof(st) // 4)).from_buffer(st)
    for k in range(len(raw)):
        raw[k] = 0xDEADBEEF
    before = {name: getattr(st, name) for name, _ in st._fields_}
    L.lib.osqp_set_default_settings(C.byref(st))
    if L.float_bits == 32:
        assert all(w != 0xDEADBEEF for w in raw)
    for name, _ in st._fields_:
        if name == "device":   # default device 0
            continue
        v = getattr(st, name)
        assert v != before[name] or v == 0, name
