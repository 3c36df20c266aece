"""ctypes binding for OSQP's public C API (include/public/osqp_api_functions.h).

One binding drives every library that exports that API with the reference's
struct layouts (include/public/osqp_api_types.h:37-187): the GB300 library
(libosqp_gb300.so, FP32; libosqp_gb300_f64.so, FP64), and, in the test suite
only, the FP64 CPU checkers.  The wrapper class mirrors the shape of OSQP's
Python interface: ``setup(P, q, A, l, u, **settings)``, ``solve()``,
``update(q=, l=, u=, Px=, Ax=)``, ``warm_start(x=, y=)``, ``update_settings``.

No torch import here: the binding is plain ctypes + numpy so that the CPU test
suite can use it without a GPU.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import Any, Dict, Optional

import numpy as np
import scipy.sparse as sp

# Status values: include/public/osqp_api_constants.h:28-40
SOLVED = 1
SOLVED_INACCURATE = 2
PRIMAL_INFEASIBLE = 3
PRIMAL_INFEASIBLE_INACCURATE = 4
DUAL_INFEASIBLE = 5
DUAL_INFEASIBLE_INACCURATE = 6
MAX_ITER_REACHED = 7
TIME_LIMIT_REACHED = 8
NON_CVX = 9
SIGINT = 10
UNSOLVED = 11

DIRECT_SOLVER = 1
INDIRECT_SOLVER = 2
# cg_precond values: OSQP's none / diagonal, and the GB300 block-Jacobi option
NO_PRECONDITIONER = 0
DIAGONAL_PRECONDITIONER = 1
BLOCK_DIAGONAL_PRECONDITIONER = 2

STATUS_NAMES = {
    1: "solved", 2: "solved inaccurate", 3: "primal infeasible",
    4: "primal infeasible inaccurate", 5: "dual infeasible",
    6: "dual infeasible inaccurate", 7: "maximum iterations reached",
    8: "run time limit reached", 9: "problem non convex", 10: "interrupted",
    11: "unsolved",
}


def _struct_types(float_bits: int):
    """Struct layouts of osqp_api_types.h for OSQPFloat = float or double, OSQPInt = int32."""
    F = C.c_double if float_bits == 64 else C.c_float
    I = C.c_int32

    class CscMatrix(C.Structure):
        _fields_ = [("m", I), ("n", I), ("p", C.POINTER(I)), ("i", C.POINTER(I)),
                    ("x", C.POINTER(F)), ("nzmax", I), ("nz", I), ("owned", I)]

    class Settings(C.Structure):
        _fields_ = [
            ("device", I), ("linsys_solver", C.c_int), ("allocate_solution", I),
            ("verbose", I), ("profiler_level", I), ("warm_starting", I),
            ("scaling", I), ("polishing", I),
            ("rho", F), ("rho_is_vec", I), ("sigma", F), ("alpha", F),
            ("cg_max_iter", I), ("cg_tol_reduction", I), ("cg_tol_fraction", F),
            ("cg_precond", C.c_int),
            ("adaptive_rho", I), ("adaptive_rho_interval", I),
            ("adaptive_rho_fraction", F), ("adaptive_rho_tolerance", F),
            ("max_iter", I), ("eps_abs", F), ("eps_rel", F), ("eps_prim_inf", F),
            ("eps_dual_inf", F), ("scaled_termination", I), ("check_termination", I),
            ("check_dualgap", I), ("time_limit", F), ("delta", F),
            ("polish_refine_iter", I),
        ]

    class Info(C.Structure):
        _fields_ = [
            ("status", C.c_char * 32), ("status_val", I), ("status_polish", I),
            ("obj_val", F), ("dual_obj_val", F), ("prim_res", F), ("dual_res", F),
            ("duality_gap", F), ("iter", I), ("rho_updates", I), ("rho_estimate", F),
            ("setup_time", F), ("solve_time", F), ("update_time", F),
            ("polish_time", F), ("run_time", F), ("primdual_int", F),
            ("rel_kkt_error", F),
        ]

    class Solution(C.Structure):
        _fields_ = [("x", C.POINTER(F)), ("y", C.POINTER(F)),
                    ("prim_inf_cert", C.POINTER(F)), ("dual_inf_cert", C.POINTER(F))]

    class Solver(C.Structure):
        _fields_ = [("settings", C.POINTER(Settings)), ("solution", C.POINTER(Solution)),
                    ("info", C.POINTER(Info)), ("work", C.c_void_p)]

    return F, I, CscMatrix, Settings, Info, Solution, Solver


class Library:
    """A loaded shared library exporting the OSQP public API."""

    def __init__(self, path: str, float_bits: int = 64, handle: Optional[C.CDLL] = None):
        self.path = path
        self.float_bits = float_bits
        self.np_float = np.float64 if float_bits == 64 else np.float32
        (self.F, self.I, self.CscMatrix, self.Settings, self.Info, self.Solution,
         self.Solver) = _struct_types(float_bits)
        self.lib = handle if handle is not None else C.CDLL(path)
        L, F, I = self.lib, self.F, self.I
        PSolver = C.POINTER(self.Solver)
        L.osqp_set_default_settings.argtypes = [C.POINTER(self.Settings)]
        L.osqp_set_default_settings.restype = None
        L.osqp_setup.argtypes = [C.POINTER(PSolver), C.POINTER(self.CscMatrix), C.POINTER(F),
                                 C.POINTER(self.CscMatrix), C.POINTER(F), C.POINTER(F),
                                 I, I, C.POINTER(self.Settings)]
        L.osqp_setup.restype = I
        L.osqp_solve.argtypes = [PSolver]
        L.osqp_solve.restype = I
        L.osqp_cleanup.argtypes = [PSolver]
        L.osqp_cleanup.restype = I
        L.osqp_update_data_vec.argtypes = [PSolver, C.POINTER(F), C.POINTER(F), C.POINTER(F)]
        L.osqp_update_data_vec.restype = I
        L.osqp_update_data_mat.argtypes = [PSolver, C.POINTER(F), C.POINTER(I), I,
                                           C.POINTER(F), C.POINTER(I), I]
        L.osqp_update_data_mat.restype = I
        L.osqp_warm_start.argtypes = [PSolver, C.POINTER(F), C.POINTER(F)]
        L.osqp_warm_start.restype = I
        L.osqp_cold_start.argtypes = [PSolver]
        L.osqp_cold_start.restype = None
        L.osqp_update_rho.argtypes = [PSolver, F]
        L.osqp_update_rho.restype = I
        L.osqp_update_settings.argtypes = [PSolver, C.POINTER(self.Settings)]
        L.osqp_update_settings.restype = I
        L.osqp_get_solution.argtypes = [PSolver, C.POINTER(self.Solution)]
        L.osqp_get_solution.restype = I
        if hasattr(L, "osqp_version"):
            L.osqp_version.restype = C.c_char_p
        if hasattr(L, "osqp_gb300_solve_stats"):
            L.osqp_gb300_solve_stats.argtypes = [PSolver, C.POINTER(I), C.POINTER(C.c_longlong),
                                                 C.POINTER(C.c_double), C.POINTER(I)]
            L.osqp_gb300_solve_stats.restype = I
        if hasattr(L, "osqp_gb300_precond_blocks"):
            L.osqp_gb300_precond_blocks.argtypes = [PSolver, C.POINTER(F)]
            L.osqp_gb300_precond_blocks.restype = I

    def default_settings(self):
        s = self.Settings()
        self.lib.osqp_set_default_settings(C.byref(s))
        return s

    def version(self) -> str:
        return self.lib.osqp_version().decode()


@dataclass
class Result:
    x: np.ndarray
    y: np.ndarray
    prim_inf_cert: np.ndarray
    dual_inf_cert: np.ndarray
    info: Dict[str, Any] = field(default_factory=dict)


def _csc_parts(M: sp.spmatrix, float_dtype, triu: bool):
    M = sp.csc_matrix(M)
    if triu:
        M = sp.triu(M, format="csc")
    M = sp.csc_matrix(M)
    M.sort_indices()
    p = np.ascontiguousarray(M.indptr, dtype=np.int32)
    i = np.ascontiguousarray(M.indices, dtype=np.int32)
    x = np.ascontiguousarray(M.data, dtype=float_dtype)
    return M.shape, p, i, x


def _ptr(a: Optional[np.ndarray], ctype):
    if a is None:
        return None
    return a.ctypes.data_as(C.POINTER(ctype))


class OSQP:
    """OSQP solver object over any library exporting the OSQP C API."""

    def __init__(self, library: Library):
        self.L = library
        self._solver = C.POINTER(library.Solver)()
        self._keep = []
        self.n = self.m = 0

    # -- life cycle ---------------------------------------------------------
    def setup(self, P, q, A, l, u, **settings) -> int:
        L = self.L
        fdt = L.np_float
        n = int(np.asarray(q).shape[0])
        if A is None:
            A = sp.csc_matrix((0, n))
        (pn, _), Pp, Pi, Px = _csc_parts(P, fdt, triu=True)
        (am, an), Ap, Ai, Ax = _csc_parts(A, fdt, triu=False)
        self.n, self.m = n, am
        q = np.ascontiguousarray(q, dtype=fdt)
        l = np.ascontiguousarray(l if l is not None else np.zeros(am), dtype=fdt)
        u = np.ascontiguousarray(u if u is not None else np.zeros(am), dtype=fdt)
        Pc = L.CscMatrix(pn, pn, _ptr(Pp, L.I), _ptr(Pi, L.I), _ptr(Px, L.F), len(Px), -1, 0)
        Ac = L.CscMatrix(am, an, _ptr(Ap, L.I), _ptr(Ai, L.I), _ptr(Ax, L.F), len(Ax), -1, 0)
        st = L.default_settings()
        st.verbose = 0
        for k, v in settings.items():
            setattr(st, k, v)
        self._keep = [Pp, Pi, Px, Ap, Ai, Ax, q, l, u]
        self.nnzP, self.nnzA = len(Px), len(Ax)
        rc = L.lib.osqp_setup(C.byref(self._solver), C.byref(Pc), _ptr(q, L.F), C.byref(Ac),
                              _ptr(l, L.F), _ptr(u, L.F), am, n, C.byref(st))
        self.setup_rc = int(rc)
        return int(rc)

    def solve(self) -> Result:
        L = self.L
        rc = L.lib.osqp_solve(self._solver)
        # 1 with status "interrupted": the solve was interrupted (Ctrl-C or interrupt())
        if rc != 0 and not (rc == 1 and self._solver.contents.info.contents.status_val == SIGINT):
            raise RuntimeError(f"osqp_solve returned {rc}")
        return self.result()

    def interrupt(self) -> int:
        """Stop the solve running on this solver (call from another thread)."""
        f = self.L.lib.osqp_gb300_interrupt
        f.argtypes = [C.POINTER(self.L.Solver)]
        f.restype = self.L.I
        return int(f(self._solver))

    def result(self) -> Result:
        s = self._solver.contents
        info = s.info.contents
        sol = s.solution.contents
        n, m = self.n, self.m
        x = np.ctypeslib.as_array(sol.x, shape=(n,)).copy() if n else np.zeros(0)
        y = np.ctypeslib.as_array(sol.y, shape=(m,)).copy() if m else np.zeros(0)
        pc = np.ctypeslib.as_array(sol.prim_inf_cert, shape=(m,)).copy() if m else np.zeros(0)
        dc = np.ctypeslib.as_array(sol.dual_inf_cert, shape=(n,)).copy() if n else np.zeros(0)
        d = {name: getattr(info, name) for name, _ in info._fields_}
        d["status"] = info.status.decode()
        return Result(x=x.astype(np.float64), y=y.astype(np.float64),
                      prim_inf_cert=pc.astype(np.float64), dual_inf_cert=dc.astype(np.float64), info=d)

    def info(self) -> Dict[str, Any]:
        info = self._solver.contents.info.contents
        d = {name: getattr(info, name) for name, _ in info._fields_}
        d["status"] = info.status.decode()
        return d

    def stats(self) -> Dict[str, Any]:
        """Device statistics of the last solve (GB300 library only)."""
        it, form = self.L.I(), self.L.I()
        pcg = C.c_longlong()
        ms = C.c_double()
        self.L.lib.osqp_gb300_solve_stats(self._solver, C.byref(it), C.byref(pcg), C.byref(ms), C.byref(form))
        return {"admm_iter": it.value, "pcg_iter": pcg.value, "kernel_ms": ms.value, "grid": form.value}

    def precond_blocks(self) -> np.ndarray:
        """Block-Jacobi blocks of M^-1 (cg_precond = 2) as an array of shape
        (ceil(n / 32), 32, 32); empty when the solver has none."""
        L = self.L
        cnt = int(L.lib.osqp_gb300_precond_blocks(self._solver, None))
        out = np.zeros(cnt, dtype=L.np_float)
        if cnt:
            got = int(L.lib.osqp_gb300_precond_blocks(self._solver, _ptr(out, L.F)))
            if got != cnt:
                raise RuntimeError("osqp_gb300_precond_blocks failed")
        return out.reshape(-1, 32, 32)

    def settings(self):
        return self._solver.contents.settings.contents

    def cleanup(self):
        if self._solver:
            self.L.lib.osqp_cleanup(self._solver)
            self._solver = C.POINTER(self.L.Solver)()

    def __del__(self):
        try:
            self.cleanup()
        except Exception:
            pass

    # -- updates ------------------------------------------------------------
    def update(self, q=None, l=None, u=None, Px=None, Px_idx=None, Ax=None, Ax_idx=None) -> int:
        L = self.L
        fdt = L.np_float
        rc = 0
        if q is not None or l is not None or u is not None:
            qa = None if q is None else np.ascontiguousarray(q, dtype=fdt)
            la = None if l is None else np.ascontiguousarray(l, dtype=fdt)
            ua = None if u is None else np.ascontiguousarray(u, dtype=fdt)
            rc = L.lib.osqp_update_data_vec(self._solver, _ptr(qa, L.F), _ptr(la, L.F), _ptr(ua, L.F))
            if rc:
                return int(rc)
        if Px is not None or Ax is not None:
            pa = None if Px is None else np.ascontiguousarray(Px, dtype=fdt)
            pi = None if Px_idx is None else np.ascontiguousarray(Px_idx, dtype=np.int32)
            aa = None if Ax is None else np.ascontiguousarray(Ax, dtype=fdt)
            ai = None if Ax_idx is None else np.ascontiguousarray(Ax_idx, dtype=np.int32)
            pn = 0 if pa is None else (len(pi) if pi is not None else len(pa))
            an = 0 if aa is None else (len(ai) if ai is not None else len(aa))
            rc = L.lib.osqp_update_data_mat(self._solver, _ptr(pa, L.F), _ptr(pi, L.I), pn,
                                            _ptr(aa, L.F), _ptr(ai, L.I), an)
        return int(rc)

    def warm_start(self, x=None, y=None) -> int:
        L = self.L
        fdt = L.np_float
        xa = None if x is None else np.ascontiguousarray(x, dtype=fdt)
        ya = None if y is None else np.ascontiguousarray(y, dtype=fdt)
        return int(L.lib.osqp_warm_start(self._solver, _ptr(xa, L.F), _ptr(ya, L.F)))

    def cold_start(self):
        self.L.lib.osqp_cold_start(self._solver)

    def update_rho(self, rho: float) -> int:
        return int(self.L.lib.osqp_update_rho(self._solver, rho))

    def update_settings(self, **kw) -> int:
        st = self.L.Settings()
        C.memmove(C.byref(st), self._solver.contents.settings, C.sizeof(st))
        for k, v in kw.items():
            setattr(st, k, v)
        return int(self.L.lib.osqp_update_settings(self._solver, C.byref(st)))


class Batch:
    """Many QPs solved in one persistent launch (osqp_gb300_batch_* in osqp_gb300_ext.h)."""

    def __init__(self, library: Library):
        self.L = library
        L, F, I = library.lib, library.F, library.I
        self._h = C.c_void_p()
        PI, PF = C.POINTER(I), C.POINTER(F)
        L.osqp_gb300_batch_setup.argtypes = [C.POINTER(C.c_void_p), I, PI, PI, PI, PI, PF, PI, PI, PF,
                                             PF, PF, PF, C.POINTER(library.Settings)]
        L.osqp_gb300_batch_setup.restype = I
        L.osqp_gb300_batch_update_data_vec.argtypes = [C.c_void_p, PF, PF, PF]
        L.osqp_gb300_batch_update_data_vec.restype = I
        L.osqp_gb300_batch_update_data_mat.argtypes = [C.c_void_p, I, PF, PI, I, PF, PI, I]
        L.osqp_gb300_batch_update_data_mat.restype = I
        L.osqp_gb300_batch_solve.argtypes = [C.c_void_p]
        L.osqp_gb300_batch_solve.restype = I
        L.osqp_gb300_batch_get_solution.argtypes = [C.c_void_p, PF, PF, PI, PI, PF, PF, PF]
        L.osqp_gb300_batch_get_solution.restype = I
        L.osqp_gb300_batch_stats.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_longlong),
                                             C.POINTER(C.c_longlong)]
        L.osqp_gb300_batch_stats.restype = I
        L.osqp_gb300_batch_step_ms.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
        L.osqp_gb300_batch_step_ms.restype = I
        L.osqp_gb300_batch_pcg_iters.argtypes = [C.c_void_p, C.POINTER(C.c_longlong)]
        L.osqp_gb300_batch_pcg_iters.restype = I
        L.osqp_gb300_batch_cleanup.argtypes = [C.c_void_p]
        L.osqp_gb300_batch_cleanup.restype = I
        L.osqp_gb300_batch_autotune.argtypes = [C.c_void_p, I, C.POINTER(I)]
        L.osqp_gb300_batch_autotune.restype = I
        L.osqp_gb300_batch_qp_seconds.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
        L.osqp_gb300_batch_qp_seconds.restype = I
        L.osqp_gb300_batch_rho_updates.argtypes = [C.c_void_p, PI]
        L.osqp_gb300_batch_rho_updates.restype = I
        L.osqp_gb300_batch_factor_elems.argtypes = [C.c_void_p, C.POINTER(C.c_longlong)]
        L.osqp_gb300_batch_factor_elems.restype = I
        L.osqp_gb300_batch_phase_cycles.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
        L.osqp_gb300_batch_phase_cycles.restype = I

    @staticmethod
    def pack(problems, float_dtype):
        """Pack [(P, q, A, l, u), ...] into the batch input arrays."""
        n, m, Pp, Pi, Px, Ap, Ai, Ax, q, l, u = [], [], [], [], [], [], [], [], [], [], []
        for (P, qq, A, ll, uu) in problems:
            (pn, _), pp, pi, px = _csc_parts(P, float_dtype, triu=True)
            (am, an), ap, ai, ax = _csc_parts(A, float_dtype, triu=False)
            n.append(pn); m.append(am)
            Pp.append(pp); Pi.append(pi); Px.append(px); Ap.append(ap); Ai.append(ai); Ax.append(ax)
            q.append(np.asarray(qq)); l.append(np.asarray(ll)); u.append(np.asarray(uu))
        cat = lambda xs, dt: np.ascontiguousarray(np.concatenate(xs) if xs else np.zeros(0), dtype=dt)
        return dict(n=np.array(n, np.int32), m=np.array(m, np.int32),
                    Pp=cat(Pp, np.int32), Pi=cat(Pi, np.int32), Px=cat(Px, float_dtype),
                    Ap=cat(Ap, np.int32), Ai=cat(Ai, np.int32), Ax=cat(Ax, float_dtype),
                    q=cat(q, float_dtype), l=cat(l, float_dtype), u=cat(u, float_dtype))

    def setup(self, problems=None, packed=None, **settings) -> int:
        L = self.L
        pk = packed if packed is not None else self.pack(problems, L.np_float)
        self.packed = pk
        self.count = len(pk["n"])
        self.nsum, self.msum = int(pk["n"].sum()), int(pk["m"].sum())
        st = L.default_settings()
        st.verbose = 0
        for k, v in settings.items():
            setattr(st, k, v)
        F, I = L.F, L.I
        rc = L.lib.osqp_gb300_batch_setup(C.byref(self._h), self.count, _ptr(pk["n"], I), _ptr(pk["m"], I),
                                          _ptr(pk["Pp"], I), _ptr(pk["Pi"], I), _ptr(pk["Px"], F),
                                          _ptr(pk["Ap"], I), _ptr(pk["Ai"], I), _ptr(pk["Ax"], F),
                                          _ptr(pk["q"], F), _ptr(pk["l"], F), _ptr(pk["u"], F), C.byref(st))
        return int(rc)

    def update(self, q=None, l=None, u=None) -> int:
        F = self.L.F
        fdt = self.L.np_float
        conv = lambda v: None if v is None else np.ascontiguousarray(v, dtype=fdt)
        qa, la, ua = conv(q), conv(l), conv(u)
        return int(self.L.lib.osqp_gb300_batch_update_data_vec(self._h, _ptr(qa, F), _ptr(la, F), _ptr(ua, F)))

    def update_mat(self, k: int, Px=None, Px_idx=None, Ax=None, Ax_idx=None) -> int:
        """New P (upper triangle) / A values of QP k, as osqp_update_data_mat
        (src/osqp_api.c:1309-1409): values in the entry order of set-up, or at
        the given entry indices."""
        L = self.L
        fdt, idt = L.np_float, np.int64 if C.sizeof(L.I) == 8 else np.int32
        conv = lambda v, t: None if v is None else np.ascontiguousarray(v, dtype=t)
        pa, pi, aa, ai = conv(Px, fdt), conv(Px_idx, idt), conv(Ax, fdt), conv(Ax_idx, idt)
        pn = 0 if pa is None else (pi.size if pi is not None else pa.size)
        an = 0 if aa is None else (ai.size if ai is not None else aa.size)
        return int(L.lib.osqp_gb300_batch_update_data_mat(self._h, int(k), _ptr(pa, L.F), _ptr(pi, L.I), pn,
                                                          _ptr(aa, L.F), _ptr(ai, L.I), an))

    def solve(self) -> int:
        return int(self.L.lib.osqp_gb300_batch_solve(self._h))

    def solution(self):
        L, F, I = self.L, self.L.F, self.L.I
        x = np.zeros(self.nsum, L.np_float)
        y = np.zeros(max(self.msum, 1), L.np_float)
        status = np.zeros(self.count, np.int32)
        it = np.zeros(self.count, np.int32)
        obj = np.zeros(self.count, L.np_float)
        pr = np.zeros(self.count, L.np_float)
        du = np.zeros(self.count, L.np_float)
        rc = L.lib.osqp_gb300_batch_get_solution(self._h, _ptr(x, F), _ptr(y, F), _ptr(status, I), _ptr(it, I),
                                                 _ptr(obj, F), _ptr(pr, F), _ptr(du, F))
        assert rc == 0, rc
        return dict(x=x, y=y[:self.msum], status=status, iter=it, obj=obj, prim_res=pr, dual_res=du)

    def split(self, v, which):
        sizes = self.packed["n"] if which == "n" else self.packed["m"]
        return np.split(v, np.cumsum(sizes)[:-1])

    def statuses(self):
        I = self.L.I
        status = np.zeros(self.count, np.int32)
        rc = self.L.lib.osqp_gb300_batch_get_solution(self._h, None, None, _ptr(status, I), None, None, None, None)
        assert rc == 0, rc
        return status

    def step_ms(self) -> float:
        v = C.c_double()
        self.L.lib.osqp_gb300_batch_step_ms(self._h, C.byref(v))
        return v.value

    def update_ptr(self, l_ptr=0, u_ptr=0, q_ptr=0) -> int:
        """update() from raw (host or device) addresses, e.g. torch tensors' data_ptr()."""
        PF = C.POINTER(self.L.F)
        cast = lambda a: C.cast(C.c_void_p(a), PF) if a else None
        return int(self.L.lib.osqp_gb300_batch_update_data_vec(self._h, cast(q_ptr), cast(l_ptr), cast(u_ptr)))

    def solution_ptr(self, x_ptr=0, y_ptr=0) -> int:
        """Copy packed x / y to raw (host or device) addresses."""
        PF = C.POINTER(self.L.F)
        cast = lambda a: C.cast(C.c_void_p(a), PF) if a else None
        return int(self.L.lib.osqp_gb300_batch_get_solution(self._h, cast(x_ptr), cast(y_ptr), None, None,
                                                            None, None, None))

    def qp_seconds(self):
        """Device time of every QP's last solve (seconds)."""
        out = np.zeros(self.count, np.float64)
        self.L.lib.osqp_gb300_batch_qp_seconds(self._h, out.ctypes.data_as(C.POINTER(C.c_double)))
        return out

    def pcg_iters(self):
        out = np.zeros(self.count, np.int64)
        self.L.lib.osqp_gb300_batch_pcg_iters(self._h, out.ctypes.data_as(C.POINTER(C.c_longlong)))
        return out

    def rho_updates(self):
        out = np.zeros(self.count, np.int32)
        self.L.lib.osqp_gb300_batch_rho_updates(self._h, out.ctypes.data_as(C.POINTER(self.L.I)))
        return out

    def phase_cycles(self):
        """SM cycles of the last solve per ADMM phase, summed over QPs (needs OSQP_GB300_PROFILE=1 at set-up)."""
        out = np.zeros(16, np.float64)
        self.L.lib.osqp_gb300_batch_phase_cycles(self._h, out.ctypes.data_as(C.POINTER(C.c_double)))
        return dict(zip(["rhs", "linsys", "updates", "termination", "refactor", "linsys_wait", "linsys_barrier",
                         "linsys_forward", "linsys_backward", "rhs_spmv", "updates_spmv", "linsys_issue",
                         "direct_solves", "direct_solves_ring", "direct_solves_global", "linsys_dot"],
                        out.tolist()))

    def dense_rows(self, k: int):
        """Dense-row form of QP k (osqp_gb300_batch_dense_rows): (rows, C^-1, Dg^-1),
        or None when QP k does not use that form."""
        L, I, F = self.L.lib, self.L.I, self.L.F
        r = I()
        rc = L.osqp_gb300_batch_dense_rows(self._h, k, C.byref(r), None, None, None)
        if rc:
            raise RuntimeError(f"osqp_gb300_batch_dense_rows failed: {rc}")
        if r.value == 0:
            return None
        n = int(self.packed["n"][k])
        rows = np.zeros(r.value, np.int32)
        cinv = np.zeros(r.value * r.value, self.L.np_float)
        dginv = np.zeros(n, self.L.np_float)
        rc = L.osqp_gb300_batch_dense_rows(self._h, k, C.byref(r), _ptr(rows, I), _ptr(cinv, F), _ptr(dginv, F))
        if rc:
            raise RuntimeError(f"osqp_gb300_batch_dense_rows failed: {rc}")
        return rows, cinv.reshape(r.value, r.value), dginv

    def factor_elems(self):
        """Elements of each QP's direct-solver factor (0 with the indirect solver)."""
        out = np.zeros(self.count, np.int64)
        self.L.lib.osqp_gb300_batch_factor_elems(self._h, out.ctypes.data_as(C.POINTER(C.c_longlong)))
        return out

    def stats(self):
        ms, a, p = C.c_double(), C.c_longlong(), C.c_longlong()
        self.L.lib.osqp_gb300_batch_stats(self._h, C.byref(ms), C.byref(a), C.byref(p))
        return {"kernel_ms": ms.value, "admm_iter": a.value, "pcg_iter": p.value}

    def autotune(self, probe_iter: int = 30) -> int:
        """Pick the SpMV tile (entries per lane) by timing; returns it."""
        v = self.L.I()
        rc = self.L.lib.osqp_gb300_batch_autotune(self._h, probe_iter, C.byref(v))
        if rc:
            raise RuntimeError(f"osqp_gb300_batch_autotune failed: {rc}")
        return int(v.value)

    def cleanup(self):
        if self._h:
            self.L.lib.osqp_gb300_batch_cleanup(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.cleanup()
        except Exception:
            pass


class Server:
    """Request serving with continuous batching (osqp_gb300_server_* in osqp_gb300_ext.h).

    Pools are Batch objects whose QPs stay resident on the device; submit()
    queues a solve of one QP of a pool with optional new q / l / u and returns
    a ticket; wait() returns (x, status, iter, obj, latency_ms)."""

    def __init__(self, library: Library, concurrency: int = 4):
        self.L = library
        L, F, I = library.lib, library.F, library.I
        PF = C.POINTER(F)
        L.osqp_gb300_server_create.argtypes = [C.POINTER(C.c_void_p), I]
        L.osqp_gb300_server_create.restype = I
        L.osqp_gb300_server_add_pool.argtypes = [C.c_void_p, C.c_void_p, C.POINTER(I)]
        L.osqp_gb300_server_add_pool.restype = I
        L.osqp_gb300_server_submit.argtypes = [C.c_void_p, I, I, PF, PF, PF, C.POINTER(C.c_longlong)]
        L.osqp_gb300_server_submit.restype = I
        L.osqp_gb300_server_wait.argtypes = [C.c_void_p, C.c_longlong, PF, C.POINTER(I), C.POINTER(I), PF,
                                             C.POINTER(C.c_double)]
        L.osqp_gb300_server_wait.restype = I
        L.osqp_gb300_server_destroy.argtypes = [C.c_void_p]
        L.osqp_gb300_server_destroy.restype = I
        self._h = C.c_void_p()
        rc = L.osqp_gb300_server_create(C.byref(self._h), concurrency)
        if rc:
            raise RuntimeError(f"osqp_gb300_server_create failed: {rc}")
        self.pools = []

    def add_pool(self, batch: "Batch") -> int:
        pid = self.L.I()
        rc = self.L.lib.osqp_gb300_server_add_pool(self._h, batch._h, C.byref(pid))
        if rc:
            raise RuntimeError(f"osqp_gb300_server_add_pool failed: {rc}")
        self.pools.append(batch)
        return int(pid.value)

    def submit(self, pool: int, qp: int, q=None, l=None, u=None) -> int:
        F = self.L.F
        fdt = self.L.np_float
        conv = lambda v: None if v is None else np.ascontiguousarray(v, dtype=fdt)
        qa, la, ua = conv(q), conv(l), conv(u)
        t = C.c_longlong()
        rc = self.L.lib.osqp_gb300_server_submit(self._h, pool, qp, _ptr(qa, F), _ptr(la, F), _ptr(ua, F),
                                                 C.byref(t))
        if rc:
            raise ValueError(f"osqp_gb300_server_submit failed: {rc}")
        return int(t.value)

    def wait(self, ticket: int, n: int):
        L, F, I = self.L, self.L.F, self.L.I
        x = np.zeros(n, L.np_float)
        st, it, ob, lat = I(), I(), F(), C.c_double()
        rc = L.lib.osqp_gb300_server_wait(self._h, ticket, _ptr(x, F), C.byref(st), C.byref(it), C.byref(ob),
                                          C.byref(lat))
        if rc:
            raise RuntimeError(f"osqp_gb300_server_wait failed: {rc}")
        return x, int(st.value), int(it.value), float(ob.value), float(lat.value)

    def close(self):
        if self._h:
            self.L.lib.osqp_gb300_server_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def objective(P, q, x) -> float:
    """0.5 x'Px + q'x with P given full or upper-triangular (symmetrised here)."""
    P = sp.csc_matrix(P)
    Pu = sp.triu(P)
    Pf = Pu + sp.triu(Pu, 1).T
    return float(0.5 * x @ (Pf @ x) + q @ x)


def kkt_plan(library: Library, P, A, bmax_limit: int = 1 << 30):
    """Ordering of the direct KKT solver for one QP (osqp_gb300_kkt_plan; host
    work only).  Returns (rc, block_start, perm): rc 0 on success, 1 when a
    block exceeds bmax_limit, 2 on inconsistent input; block_start has
    nblocks + 1 entries and perm maps permuted positions to variables."""
    L, I = library.lib, library.I
    fn = L.osqp_gb300_kkt_plan
    fn.argtypes = [I, I, C.POINTER(I), C.POINTER(I), C.POINTER(I), C.POINTER(I), I, C.POINTER(I), C.POINTER(I),
                   C.POINTER(I)]
    fn.restype = I
    (n, _), pp, pi, _ = _csc_parts(P, library.np_float, triu=True)
    (m, _), ap, ai, _ = _csc_parts(A, library.np_float, triu=False)
    nb = I(0)
    bs = np.zeros(n + 1, np.int32)
    perm = np.zeros(n, np.int32)
    rc = fn(n, m, _ptr(pp, I), _ptr(pi, I), _ptr(ap, I), _ptr(ai, I), bmax_limit, C.byref(nb), _ptr(bs, I),
            _ptr(perm, I))
    return int(rc), bs[:nb.value + 1].copy(), perm
