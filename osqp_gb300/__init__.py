"""GB300-native OSQP: the OSQP 1.0 C API on hand-written sm_103a CUDA kernels.

    from osqp_gb300 import load
    lib = load("f32")            # or "f64"
    from osqp_gb300.api import OSQP
    s = OSQP(lib); s.setup(P, q, A, l, u, eps_abs=1e-3); res = s.solve()

`load` opens the in-tree shared library built by `osqp_gb300.build`; it raises
if the library has not been built -- there is no CPU fallback.
"""
from __future__ import annotations

import os

from .api import Library, OSQP  # noqa: F401

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_DIR = os.path.join(HERE, "lib")
LIB_NAMES = {"f32": "libosqp_gb300.so", "f64": "libosqp_gb300_f64.so"}

_loaded = {}


def lib_path(precision: str = "f32") -> str:
    return os.path.join(LIB_DIR, LIB_NAMES[precision])


def load(precision: str = "f32") -> Library:
    if precision not in _loaded:
        path = lib_path(precision)
        if not os.path.exists(path):
            raise RuntimeError(f"{path} is missing: build it with `python -m osqp_gb300.build` "
                               "(the GB300 solver has no CPU fallback)")
        _loaded[precision] = Library(path, 32 if precision == "f32" else 64)
    return _loaded[precision]
