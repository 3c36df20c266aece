"""Write tests/golden/large_qp.npz from the reference's large_qp fixture.

Run in the development container only (it reads the reference tree):

    python tests/golden/make_large_qp.py /root/reference

tests/large_qp/large_qp_data.c is a C source written by OSQP's code
generator (prob1: n = 160, m = 270, expected objective 0.106081, checked by
tests/large_qp/test_large_qp.cpp:10-37).  It is read here as text: each
array initialiser `<type> prob1_data_<name>[<len>] = { ... };` becomes one
array of the fixture, and the expected objective `prob1_obj_val` a scalar.
"""
from __future__ import annotations

import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ARRAYS = {"P_csc_p": np.int32, "P_csc_i": np.int32, "P_csc_x": np.float64,
          "A_csc_p": np.int32, "A_csc_i": np.int32, "A_csc_x": np.float64,
          "q_val": np.float64, "l_val": np.float64, "u_val": np.float64}


def parse(text: str) -> dict:
    out = {}
    for name, dtype in ARRAYS.items():
        m = re.search(r"prob1_data_%s\[(\d+)\]\s*=\s*\{(.*?)\};" % name, text, re.S)
        if not m:
            raise ValueError(f"prob1_data_{name} not found")
        items = [t.strip() for t in m.group(2).split(",") if t.strip()]
        vals = [float(t.replace("(OSQPFloat)", "").replace("OSQP_INFTY", "inf")) for t in items]
        arr = np.asarray(vals, dtype=np.float64).astype(dtype)
        if arr.size != int(m.group(1)):
            raise ValueError(f"prob1_data_{name}: {arr.size} values, declared {m.group(1)}")
        out[name] = arr
    for name in ("n", "m"):
        out[name] = np.int32(int(re.search(r"prob1_data_%s\s*=\s*(\d+);" % name, text).group(1)))
    out["obj_val"] = np.float64(float(re.search(r"prob1_obj_val\s*=\s*([-0-9.eE+]+);", text).group(1)))
    return out


def main(ref_root: str) -> None:
    with open(os.path.join(ref_root, "tests", "large_qp", "large_qp_data.c")) as f:
        data = parse(f.read())
    np.savez_compressed(os.path.join(HERE, "large_qp.npz"), **data)
    print({k: (v.shape if np.ndim(v) else float(v)) for k, v in data.items()})


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
