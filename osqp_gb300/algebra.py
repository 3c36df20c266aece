"""ctypes binding for the algebra / linear-system ABI (include/osqp_gb300_algebra.h).

This is the interface OSQP's C core links against (libosqp_gb300_algebra.so,
FP32; libosqp_gb300_algebra_f64.so, FP64).  The wrapper exposes it to Python
for conformance tests and for callers that drive the algebra directly.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np
import scipy.sparse as sp

from .api import _struct_types

HERE = os.path.dirname(os.path.abspath(__file__))
NAMES = {"f32": "libosqp_gb300_algebra.so", "f64": "libosqp_gb300_algebra_f64.so"}


def _linsys_type(F, I):
    """struct linsys_solver (include/private/types.h:243-279) for one OSQPFloat width."""
    class LinSysSolver(C.Structure):
        pass
    LS = C.POINTER(LinSysSolver)
    V = C.c_void_p
    LinSysSolver._fields_ = [
        ("type", C.c_int), ("name", C.CFUNCTYPE(C.c_char_p, LS)),
        ("solve", C.CFUNCTYPE(I, LS, V, I)), ("update_settings", C.CFUNCTYPE(None, LS, V)),
        ("warm_start", C.CFUNCTYPE(None, LS, V)), ("adjoint_derivative", C.CFUNCTYPE(I, LS)),
        ("free", C.CFUNCTYPE(None, LS)),
        ("update_matrices", C.CFUNCTYPE(I, LS, V, C.POINTER(I), I, V, C.POINTER(I), I)),
        ("update_rho_vec", C.CFUNCTYPE(I, LS, V, F)), ("nthreads", I),
    ]
    return LinSysSolver


class AlgebraLib:
    def __init__(self, precision: str = "f32", path: str | None = None):
        self.precision = precision
        bits = 32 if precision == "f32" else 64
        (self.F, self.I, self.CscMatrix, self.Settings, self.Info, self.Solution,
         self.Solver) = _struct_types(bits)
        self.np_float = np.float32 if bits == 32 else np.float64
        path = path or os.path.join(HERE, "lib", NAMES[precision])
        if not os.path.exists(path):
            raise RuntimeError(f"{path} is missing: build it with `python -m osqp_gb300.build`")
        self.lib = L = C.CDLL(path)
        F, I, V = self.F, self.I, C.c_void_p
        PF, PI = C.POINTER(F), C.POINTER(I)
        self.LinSysSolver = _linsys_type(F, I)
        LS = C.POINTER(self.LinSysSolver)
        sig = {
            "OSQPVectorf_new": (V, [PF, I]), "OSQPVectorf_malloc": (V, [I]), "OSQPVectorf_calloc": (V, [I]),
            "OSQPVectori_new": (V, [PI, I]), "OSQPVectori_calloc": (V, [I]),
            "OSQPVectorf_free": (None, [V]), "OSQPVectori_free": (None, [V]),
            "OSQPVectorf_to_raw": (None, [PF, V]), "OSQPVectori_to_raw": (None, [PI, V]),
            "OSQPVectorf_from_raw": (None, [V, PF]), "OSQPVectorf_copy": (None, [V, V]),
            "OSQPVectorf_length": (I, [V]), "OSQPVectorf_view": (V, [V, I, I]), "OSQPVectorf_view_free": (None, [V]),
            "OSQPVectorf_concat": (V, [V, V]), "OSQPVectorf_subvector_byrows": (V, [V, V]),
            "OSQPVectorf_subvector_assign": (None, [V, PF, I, I, F]),
            "OSQPVectorf_subvector_assign_scalar": (None, [V, F, I, I]),
            "OSQPVectorf_set_scalar": (None, [V, F]),
            "OSQPVectorf_set_scalar_conditional": (None, [V, V, F, F, F]),
            "OSQPVectorf_round_to_zero": (None, [V, F]), "OSQPVectorf_mult_scalar": (None, [V, F]),
            "OSQPVectorf_plus": (None, [V, V, V]), "OSQPVectorf_minus": (None, [V, V, V]),
            "OSQPVectorf_add_scaled": (None, [V, F, V, F, V]),
            "OSQPVectorf_add_scaled3": (None, [V, F, V, F, V, F, V]),
            "OSQPVectorf_norm_inf": (F, [V]), "OSQPVectorf_scaled_norm_inf": (F, [V, V]),
            "OSQPVectorf_norm_inf_diff": (F, [V, V]), "OSQPVectorf_norm_2": (F, [V]),
            "OSQPVectorf_norm_1": (F, [V]), "OSQPVectorf_dot_prod": (F, [V, V]),
            "OSQPVectorf_dot_prod_signed": (F, [V, V, I]), "OSQPVectorf_ew_prod": (None, [V, V, V]),
            "OSQPVectorf_all_leq": (I, [V, V]), "OSQPVectorf_ew_bound_vec": (None, [V, V, V, V]),
            "OSQPVectorf_project_polar_reccone": (None, [V, V, V, F]),
            "OSQPVectorf_in_reccone": (I, [V, V, V, F, F]), "OSQPVectorf_ew_reciprocal": (None, [V, V]),
            "OSQPVectorf_ew_sqrt": (None, [V]), "OSQPVectorf_ew_max_vec": (None, [V, V, V]),
            "OSQPVectorf_ew_min_vec": (None, [V, V, V]), "OSQPVectorf_ew_bounds_type": (I, [V, V, V, F, F]),
            "OSQPVectorf_set_scalar_if_lt": (None, [V, V, F, F]),
            "OSQPVectorf_set_scalar_if_gt": (None, [V, V, F, F]), "OSQPVectorf_is_eq": (I, [V, V, F]),
            "OSQPMatrix_new_from_csc": (V, [C.POINTER(self.CscMatrix), I]), "OSQPMatrix_free": (None, [V]),
            "OSQPMatrix_get_m": (I, [V]), "OSQPMatrix_get_n": (I, [V]), "OSQPMatrix_get_nz": (I, [V]),
            "OSQPMatrix_mult_scalar": (None, [V, F]), "OSQPMatrix_lmult_diag": (None, [V, V]),
            "OSQPMatrix_rmult_diag": (None, [V, V]), "OSQPMatrix_Axpy": (None, [V, V, V, F, F]),
            "OSQPMatrix_Atxpy": (None, [V, V, V, F, F]), "OSQPMatrix_col_norm_inf": (None, [V, V]),
            "OSQPMatrix_row_norm_inf": (None, [V, V]), "OSQPMatrix_submatrix_byrows": (V, [V, V]),
            "OSQPMatrix_update_values": (None, [V, PF, PI, I]), "OSQPMatrix_extract_diag": (None, [V, V]),
            "OSQPMatrix_AtDA_extract_diag": (None, [V, V, V]), "OSQPMatrix_is_eq": (I, [V, V, F]),
            "osqp_algebra_init_libs": (I, [I]), "osqp_algebra_free_libs": (None, []),
            "osqp_algebra_linsys_supported": (I, []), "osqp_algebra_default_linsys": (C.c_int, []),
            "osqp_algebra_name": (I, [C.c_char_p, I]), "osqp_algebra_device_name": (I, [C.c_char_p, I]),
            "osqp_algebra_init_linsys_solver": (I, [C.POINTER(LS), V, V, V, C.POINTER(self.Settings), PF, PF, I]),
            "osqp_set_default_settings": None,
        }
        for name, s in sig.items():
            if s is None or not hasattr(L, name):
                continue
            fn = getattr(L, name)
            fn.restype, fn.argtypes = s[0], s[1]
        assert L.osqp_algebra_init_libs(0) == 0

    # helpers -------------------------------------------------------------
    def vec(self, a):
        a = np.ascontiguousarray(a, dtype=self.np_float)
        return self.lib.OSQPVectorf_new(a.ctypes.data_as(C.POINTER(self.F)), len(a))

    def ivec(self, a):
        a = np.ascontiguousarray(a, dtype=np.int32)
        return self.lib.OSQPVectori_new(a.ctypes.data_as(C.POINTER(self.I)), len(a))

    def get(self, v):
        n = self.lib.OSQPVectorf_length(v)
        out = np.zeros(n, self.np_float)
        if n:
            self.lib.OSQPVectorf_to_raw(out.ctypes.data_as(C.POINTER(self.F)), v)
        return out.astype(np.float64)

    def mat(self, M, triu=False):
        M = sp.csc_matrix(M)
        if triu:
            M = sp.triu(M, format="csc")
        M.sort_indices()
        p = np.ascontiguousarray(M.indptr, np.int32)
        i = np.ascontiguousarray(M.indices if M.nnz else np.zeros(1), np.int32)
        x = np.ascontiguousarray(M.data if M.nnz else np.zeros(1), self.np_float)
        c = self.CscMatrix(M.shape[0], M.shape[1], p.ctypes.data_as(C.POINTER(self.I)),
                           i.ctypes.data_as(C.POINTER(self.I)), x.ctypes.data_as(C.POINTER(self.F)),
                           M.nnz, -1, 0)
        return self.lib.OSQPMatrix_new_from_csc(C.byref(c), 1 if triu else 0)

    def default_settings(self):
        st = self.Settings()
        st.rho, st.sigma, st.delta = 0.1, 1e-6, 1e-6
        st.cg_max_iter, st.cg_tol_reduction, st.cg_tol_fraction, st.cg_precond = 20, 10, 0.15, 1
        st.linsys_solver = 2
        return st
