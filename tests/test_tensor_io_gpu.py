"""Zero-copy tensor front-end (osqp_gb300/tensor_io.py) with CUDA tensors: the
GPU libraries read the device tensors in place and give the same bits as the
NumPy front-end on the same data."""
import numpy as np
import pytest

from osqp_gb300 import load
from osqp_gb300 import problems as pb
from osqp_gb300.api import OSQP, Batch
from osqp_gb300.tensor_io import setup_tensors, solution_into, update_tensors, batch_solution_into
from test_tensor_io import _tensors

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

INF = {"f32": 1e17, "f64": 1e30}
ST = dict(eps_abs=1e-3, eps_rel=1e-3, rho_is_vec=1, check_termination=5, adaptive_rho_tolerance=5.0)


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_device_tensors_same_bits_as_numpy(prec):
    lib = load(prec)
    dt = torch.float32 if prec == "f32" else torch.float64
    data = pb.random_qp(43, n=70, m=110)
    P, q, A, l, u = data
    ref = OSQP(lib)
    assert ref.setup(P, q, A, pb.clip_inf(l, INF[prec]), pb.clip_inf(u, INF[prec]), **ST) == 0
    r = ref.solve()
    (Pp, Pi, Px), qt, (Ap, Ai, Ax), lt, ut = _tensors(data, dt)
    cuda = lambda t: t.cuda()
    s = setup_tensors(lib, tuple(map(cuda, (Pp, Pi, Px))), qt.cuda(), tuple(map(cuda, (Ap, Ai, Ax))),
                      lt.clamp(-INF[prec], INF[prec]).cuda(), ut.clamp(-INF[prec], INF[prec]).cuda(), **ST)
    r2 = s.solve()
    assert r2.info["iter"] == r.info["iter"]
    x = torch.empty(70, dtype=dt, device="cuda")
    y = torch.empty(110, dtype=dt, device="cuda")
    solution_into(s, x, y)
    assert np.array_equal(x.cpu().numpy(), r.x.astype(lib.np_float))
    assert np.array_equal(y.cpu().numpy(), r.y.astype(lib.np_float))
    q2 = (q * 1.05).astype(lib.np_float)
    assert ref.update(q=q2) == 0
    update_tensors(s, q=torch.tensor(q2, device="cuda"))
    r, r2 = ref.solve(), s.solve()
    assert r2.info["iter"] == r.info["iter"] and np.array_equal(r.x, r2.x)
    ref.cleanup(); s.cleanup()


def test_batch_tensors_same_bits_as_host_arrays():
    lib = load("f32")
    probs = [pb.mpc(950 + k) for k in range(3)]
    rg = np.random.default_rng(12)
    ls, us = [], []
    for (P, q, A, l, u) in probs:
        rowlen = np.diff(A.tocsr().indptr)
        nx = int(np.argmax(rowlen != 1))
        l2, u2 = pb.mpc_x0_bounds(l, u, rg.uniform(-1.0, 1.0, nx))
        ls.append(l2); us.append(u2)
    l_all = pb.clip_inf(np.concatenate(ls), 1e17).astype(np.float32)
    u_all = pb.clip_inf(np.concatenate(us), 1e17).astype(np.float32)
    st = dict(ST, rho=0.1, sigma=1e-6, alpha=1.6, scaling=10, max_iter=4000)
    host, dev = Batch(lib), Batch(lib)
    assert host.setup(probs, **st) == 0 and dev.setup(probs, **st) == 0
    assert host.update(l=l_all, u=u_all) == 0 and host.solve() == 0
    sol = host.solution()
    update_tensors(dev, l=torch.tensor(l_all, device="cuda"), u=torch.tensor(u_all, device="cuda"))
    assert dev.solve() == 0
    x = torch.empty(sol["x"].size, dtype=torch.float32, device="cuda")
    y = torch.empty(sol["y"].size, dtype=torch.float32, device="cuda")
    batch_solution_into(dev, x, y)
    assert np.array_equal(x.cpu().numpy(), sol["x"]) and np.array_equal(y.cpu().numpy(), sol["y"])
    host.cleanup(); dev.cleanup()
