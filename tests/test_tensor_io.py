"""Zero-copy tensor front-end (osqp_gb300/tensor_io.py) on CPU: host tensors
through the FP64 oracle library (which reads host addresses like the GPU
libraries do) give the same bits as the NumPy front-end, and malformed
tensors are rejected before any C call."""
import numpy as np
import pytest
import scipy.sparse as sp

from osqp_gb300 import problems as pb
from osqp_gb300.api import OSQP, DIRECT_SOLVER
from osqp_gb300.tensor_io import setup_tensors, solution_into, update_tensors

torch = pytest.importorskip("torch")

ST = dict(linsys_solver=DIRECT_SOLVER, eps_abs=1e-4, eps_rel=1e-4, polishing=1)


def _csc_tensors(M, dtype, triu=False):
    M = sp.triu(M, format="csc") if triu else sp.csc_matrix(M)
    M.sort_indices()
    return (torch.tensor(M.indptr, dtype=torch.int32), torch.tensor(M.indices, dtype=torch.int32),
            torch.tensor(M.data, dtype=dtype))


def _tensors(data, dtype=torch.float64):
    P, q, A, l, u = data
    return (_csc_tensors(P, dtype, triu=True), torch.tensor(q, dtype=dtype), _csc_tensors(A, dtype),
            torch.tensor(pb.clip_inf(l, 1e30), dtype=dtype), torch.tensor(pb.clip_inf(u, 1e30), dtype=dtype))


def test_same_bits_as_numpy_front_end(oracle_lib):
    data = pb.random_qp(41, n=50, m=80)
    P, q, A, l, u = data
    ref = OSQP(oracle_lib)
    assert ref.setup(P, q, A, pb.clip_inf(l, 1e30), pb.clip_inf(u, 1e30), **ST) == 0
    r = ref.solve()
    Pt, qt, At, lt, ut = _tensors(data)
    s = setup_tensors(oracle_lib, Pt, qt, At, lt, ut, **ST)
    r2 = s.solve()
    assert r2.info["iter"] == r.info["iter"] and r2.info["obj_val"] == r.info["obj_val"]
    x, y = torch.empty(50, dtype=torch.float64), torch.empty(80, dtype=torch.float64)
    solution_into(s, x, y)
    assert np.array_equal(x.numpy(), r.x) and np.array_equal(y.numpy(), r.y)
    # vector update from tensors == NumPy update
    q2 = q * 1.1
    assert ref.update(q=q2) == 0
    update_tensors(s, q=torch.tensor(q2, dtype=torch.float64))
    r, r2 = ref.solve(), s.solve()
    assert np.array_equal(r.x, r2.x) and r.info["iter"] == r2.info["iter"]


def test_rejects_malformed_tensors(oracle_lib):
    data = pb.random_qp(42, n=20, m=30)
    Pt, qt, At, lt, ut = _tensors(data)
    with pytest.raises(TypeError):       # FP32 values for the FP64 library
        setup_tensors(oracle_lib, Pt, qt.float(), At, lt, ut, **ST)
    with pytest.raises(ValueError):      # l of the wrong length
        setup_tensors(oracle_lib, Pt, qt, At, lt[:-1], ut, **ST)
    with pytest.raises(TypeError):       # int64 indices
        setup_tensors(oracle_lib, (Pt[0].long(), Pt[1], Pt[2]), qt, At, lt, ut, **ST)
    with pytest.raises(ValueError):      # non-contiguous
        setup_tensors(oracle_lib, Pt, torch.stack([qt, qt], 1)[:, 0], At, lt, ut, **ST)
    s = setup_tensors(oracle_lib, Pt, qt, At, lt, ut, **ST)
    s.solve()
    with pytest.raises(ValueError):
        solution_into(s, torch.empty(19, dtype=torch.float64))
    with pytest.raises(TypeError):
        update_tensors(s, q=qt.numpy())
