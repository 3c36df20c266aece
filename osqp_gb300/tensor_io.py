"""Zero-copy tensor inputs and outputs for the OSQP and batched solvers.

The libraries read every caller array through its address with
cudaMemcpyDefault, so device tensors (and host tensors) are passed as they
are: no staging copy in Python.  These helpers check each tensor (dtype of
the library's OSQPFloat / int32 indices, contiguous, length), order the
caller's pending device work before the library reads the memory, and hand
the addresses to the C entry points:

    from osqp_gb300 import load
    from osqp_gb300.tensor_io import setup_tensors, solution_into
    s = setup_tensors(load("f32"), P_csc, q, A_csc, l, u, eps_abs=1e-3)   # P_csc = (indptr, indices, data)
    s.solve()
    solution_into(s, x_out, y_out)          # writes the solution into the tensors

Batched solver: `update_tensors(batch, q=..., l=..., u=...)` and
`batch_solution_into(batch, x_out, y_out)` (packed vectors, as
`osqp_gb300_batch_update_data_vec` / `osqp_gb300_batch_get_solution`).

PyTorch is used only for the tensors' memory (it is imported lazily).
"""
from __future__ import annotations

import ctypes as C
from typing import Optional, Sequence

from .api import OSQP, Batch, Library

__all__ = ["setup_tensors", "solution_into", "update_tensors", "batch_solution_into"]


def _torch():
    import torch
    return torch


def _float_dtype(lib: Library):
    torch = _torch()
    return torch.float32 if lib.float_bits == 32 else torch.float64


def _check(t, name: str, dtype, length: Optional[int]):
    torch = _torch()
    if not isinstance(t, torch.Tensor):
        raise TypeError(f"{name}: expected a torch.Tensor, got {type(t).__name__}")
    if t.dtype != dtype:
        raise TypeError(f"{name}: dtype {t.dtype}, the library needs {dtype}")
    if t.dim() != 1 or not t.is_contiguous():
        raise ValueError(f"{name}: expected a contiguous 1-D tensor")
    if length is not None and t.numel() != length:
        raise ValueError(f"{name}: {t.numel()} values, expected {length}")
    return t


def _ptr(t, T):
    return None if t is None else C.cast(C.c_void_p(t.data_ptr()), C.POINTER(T))


def _order_device_work(tensors: Sequence):
    """The library works on its own streams: finish the producers' work on the
    tensors' current streams before it reads them."""
    torch = _torch()
    seen = set()
    for t in tensors:
        if t is not None and t.is_cuda and t.device not in seen:
            seen.add(t.device)
            torch.cuda.current_stream(t.device).synchronize()


def setup_tensors(lib: Library, P: Sequence, q, A: Sequence, l, u, **settings) -> OSQP:
    """osqp_setup from tensors: P = (indptr, indices, data) of the upper
    triangle in CSC, A = (indptr, indices, data) in CSC with A's row count
    taken from len(l).  Returns an OSQP object (solve / update / stats as usual)."""
    torch = _torch()
    fdt = _float_dtype(lib)
    n = int(q.numel())
    m = int(l.numel()) if l is not None else 0
    Pp, Pi, Px = P
    Ap, Ai, Ax = A
    _check(q, "q", fdt, n)
    _check(Pp, "P indptr", torch.int32, n + 1)
    _check(Ap, "A indptr", torch.int32, n + 1)
    nnzP = int(Pp[-1].item())
    nnzA = int(Ap[-1].item())
    _check(Pi, "P indices", torch.int32, None)
    _check(Px, "P data", fdt, None)
    _check(Ai, "A indices", torch.int32, None)
    _check(Ax, "A data", fdt, None)
    if Pi.numel() < nnzP or Px.numel() < nnzP or Ai.numel() < nnzA or Ax.numel() < nnzA:
        raise ValueError("CSC indices / data shorter than indptr[-1]")
    if m:
        _check(l, "l", fdt, m)
        _check(u, "u", fdt, m)
    _order_device_work([Pp, Pi, Px, Ap, Ai, Ax, q, l, u])
    Pc = lib.CscMatrix(n, n, _ptr(Pp, lib.I), _ptr(Pi, lib.I), _ptr(Px, lib.F), nnzP, -1, 0)
    Ac = lib.CscMatrix(m, n, _ptr(Ap, lib.I), _ptr(Ai, lib.I), _ptr(Ax, lib.F), nnzA, -1, 0)
    st = lib.default_settings()
    st.verbose = 0
    for k, v in settings.items():
        setattr(st, k, v)
    s = OSQP(lib)
    s.n, s.m = n, m
    s.nnzP, s.nnzA = nnzP, nnzA
    s._keep = [Pp, Pi, Px, Ap, Ai, Ax, q, l, u]
    rc = lib.lib.osqp_setup(C.byref(s._solver), C.byref(Pc), _ptr(q, lib.F), C.byref(Ac),
                            _ptr(l if m else None, lib.F), _ptr(u if m else None, lib.F), m, n, C.byref(st))
    s.setup_rc = int(rc)
    if rc:
        raise RuntimeError(f"osqp_setup returned {rc}")
    return s


def solution_into(s: OSQP, x=None, y=None, prim_inf_cert=None, dual_inf_cert=None) -> None:
    """osqp_get_solution into tensors.  OSQP's get_solution writes all four
    arrays (src/auxil.c store_solution), so the ones passed as None get
    scratch tensors on the device of the given ones."""
    torch = _torch()
    L = s.L
    fdt = _float_dtype(L)
    given = [t for t in (x, y, prim_inf_cert, dual_inf_cert) if t is not None]
    dev = given[0].device if given else torch.device("cpu")
    out = []
    for t, name, length in ((x, "x", s.n), (y, "y", s.m), (prim_inf_cert, "prim_inf_cert", s.m),
                            (dual_inf_cert, "dual_inf_cert", s.n)):
        if t is None:
            t = torch.empty(max(length, 1), dtype=fdt, device=dev)
        else:
            _check(t, name, fdt, length)
        out.append(t)
    x, y, prim_inf_cert, dual_inf_cert = out
    _order_device_work(out)
    sol = L.Solution(_ptr(x, L.F), _ptr(y, L.F), _ptr(prim_inf_cert, L.F), _ptr(dual_inf_cert, L.F))
    rc = L.lib.osqp_get_solution(s._solver, C.byref(sol))
    if rc:
        raise RuntimeError(f"osqp_get_solution returned {rc}")


def update_tensors(target, q=None, l=None, u=None) -> None:
    """osqp_update_data_vec (OSQP) or osqp_gb300_batch_update_data_vec (Batch,
    packed vectors of all QPs) from tensors."""
    L = target.L
    fdt = _float_dtype(L)
    if isinstance(target, Batch):
        n, m = target.nsum, target.msum
    else:
        n, m = target.n, target.m
    for t, name, length in ((q, "q", n), (l, "l", m), (u, "u", m)):
        if t is not None:
            _check(t, name, fdt, length)
    _order_device_work([q, l, u])
    if isinstance(target, Batch):
        rc = L.lib.osqp_gb300_batch_update_data_vec(target._h, _ptr(q, L.F), _ptr(l, L.F), _ptr(u, L.F))
    else:
        rc = L.lib.osqp_update_data_vec(target._solver, _ptr(q, L.F), _ptr(l, L.F), _ptr(u, L.F))
    if rc:
        raise RuntimeError(f"update returned {rc}")


def batch_solution_into(b: Batch, x=None, y=None) -> None:
    """Packed x / y of every QP of the batch into tensors."""
    fdt = _float_dtype(b.L)
    if x is not None:
        _check(x, "x", fdt, b.nsum)
    if y is not None:
        _check(y, "y", fdt, b.msum)
    _order_device_work([x, y])
    rc = b.L.lib.osqp_gb300_batch_get_solution(b._h, _ptr(x, b.L.F), _ptr(y, b.L.F), None, None, None, None, None)
    if rc:
        raise RuntimeError(f"osqp_gb300_batch_get_solution returned {rc}")
