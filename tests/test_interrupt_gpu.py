"""Interrupting a running solve (osqp_api.c:728-737, src/interrupt_unix.c):
from another thread through osqp_gb300_interrupt, and by SIGINT while
osqp_solve runs.  Either way the solve stops with status OSQP_SIGINT well
before its iteration limit, and osqp_solve returns 1.  The solves are bounded
by max_iter should an interrupt not arrive."""
import os
import signal
import threading

import pytest

from osqp_gb300 import load
from osqp_gb300 import problems as pb
from osqp_gb300.api import OSQP, SIGINT, SOLVED

pytestmark = pytest.mark.gpu

MAX_ITER = 100_000
# no termination checks and tiny tolerances: the solve runs until stopped
LONG = dict(eps_abs=1e-12, eps_rel=1e-12, max_iter=MAX_ITER, check_termination=0, adaptive_rho=0)


def _long_solver(prec):
    P, q, A, l, u = pb.random_qp(7, n=300, m=600)
    s = OSQP(load(prec))
    inf = 1e17 if prec == "f32" else 1e30
    assert s.setup(P, q, A, pb.clip_inf(l, inf), pb.clip_inf(u, inf), **LONG) == 0
    return s


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_interrupt_from_another_thread(prec):
    s = _long_solver(prec)
    out = {}
    th = threading.Thread(target=lambda: out.setdefault("r", s.solve()))
    th.start()
    stop = threading.Event()
    stop.wait(0.1)
    assert s.interrupt() == 0
    th.join(timeout=120)
    assert not th.is_alive()
    r = out["r"]
    assert r.info["status_val"] == SIGINT and 0 < r.info["iter"] < MAX_ITER
    # the next solve is not affected by the earlier request
    assert s.update_settings(eps_abs=1e-3, eps_rel=1e-3, check_termination=5, max_iter=4000) == 0
    assert s.solve().info["status_val"] == SOLVED
    s.cleanup()


def test_sigint_interrupts_the_solve():
    """A SIGINT during osqp_solve becomes an interrupt; the caller's handler
    is back in place afterwards (a SIGINT outside the solve would reach it,
    never Python's default KeyboardInterrupt)."""
    got = []
    old = signal.signal(signal.SIGINT, lambda *a: got.append(1))
    try:
        s = _long_solver("f32")
        timer = threading.Timer(0.1, lambda: os.kill(os.getpid(), signal.SIGINT))
        timer.start()
        r = s.solve()
        timer.join()
        assert r.info["status_val"] == SIGINT and 0 < r.info["iter"] < MAX_ITER
        assert not got
        assert signal.getsignal(signal.SIGINT) is not signal.default_int_handler
        s.cleanup()
    finally:
        signal.signal(signal.SIGINT, old)
