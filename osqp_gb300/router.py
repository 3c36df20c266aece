"""Spread independent QPs over several GPUs and gather the results in order.

Batched and served QPs are independent, so a batch or a request stream
partitions with no data-path collective: each device owns a share of the QPs
as its own resident batch (structures, factors, iterates) and solves it in one
persistent launch; only the per-QP results travel back, once per solve.

Two ways to drive it:

* one process, several devices -- ``DeviceRouter(problems, devices, **settings)``
  sets up one ``Batch`` per device (settings ``device=k``) and solves them from
  one host thread per device;
* one process per device (torch.distributed, e.g. launched by torchrun) --
  every rank calls ``partition(weights, world)`` for its share, solves it,
  and ``gather_in_order`` collects the shares on every rank over the process
  group (gloo or nccl; host objects, one collective per solve).

The partition is contiguous and balanced by a per-QP cost (nonzeros of P and
A by default), so results come back in the caller's order by concatenation.
"""
from __future__ import annotations

import threading
from typing import Dict, List, Sequence

import numpy as np


def qp_cost(problem) -> float:
    """Work estimate of one QP: stored entries of P and A plus its dimensions."""
    P, q, A, l, u = problem
    return float(P.nnz + 2 * A.nnz + P.shape[0] + A.shape[0])


def partition(weights: Sequence[float], parts: int) -> List[range]:
    """Contiguous index ranges, one per part, of roughly equal total weight
    (every part non-empty while there are at least `parts` items)."""
    w = np.asarray(weights, dtype=np.float64)
    count = len(w)
    if parts <= 0:
        raise ValueError("parts must be positive")
    if count == 0:
        return [range(0, 0) for _ in range(parts)]
    cum = np.concatenate([[0.0], np.cumsum(w)])
    cuts = [0]
    for p in range(1, parts):
        target = cum[-1] * p / parts
        c = int(np.searchsorted(cum, target, side="left"))
        lo = cuts[-1] + (1 if count - cuts[-1] > parts - p else 0)   # keep later parts non-empty
        hi = count - (parts - p)
        cuts.append(int(min(max(c, lo), max(hi, lo))))
    cuts.append(count)
    return [range(cuts[p], cuts[p + 1]) for p in range(parts)]


def gather_in_order(local: Dict[str, np.ndarray], dist=None) -> Dict[str, np.ndarray]:
    """Concatenate every rank's per-QP result arrays in rank order (the
    caller's order for a contiguous partition).  Without a process group the
    local arrays are returned."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return {k: np.asarray(v) for k, v in local.items()}
    world = dist.get_world_size()
    out: List[Dict[str, np.ndarray]] = [None] * world
    dist.all_gather_object(out, {k: np.asarray(v) for k, v in local.items()})
    return {k: np.concatenate([o[k] for o in out]) for k in local}


class DeviceRouter:
    """One resident batch per device over a contiguous, cost-balanced split."""

    def __init__(self, library, problems, devices: Sequence[int], weights=None, **settings):
        from .api import Batch
        self.devices = list(devices)
        self.count = len(problems)
        w = [qp_cost(p) for p in problems] if weights is None else weights
        self.parts = partition(w, len(self.devices))
        self.batches = []
        for dev, rg in zip(self.devices, self.parts):
            b = Batch(library)
            rc = b.setup([problems[i] for i in rg], **dict(settings, device=dev))
            if rc:
                self.cleanup()
                raise RuntimeError(f"batch set-up on device {dev} failed: {rc}")
            self.batches.append(b)
        self.nsplit = [np.cumsum([0] + [problems[i][0].shape[0] for i in rg]) for rg in self.parts]
        self.msplit = [np.cumsum([0] + [problems[i][2].shape[0] for i in rg]) for rg in self.parts]

    def _each(self, fn):
        errs = []

        def run(b):
            try:
                fn(b)
            except Exception as e:   # re-raised on the calling thread
                errs.append(e)

        ts = [threading.Thread(target=run, args=(b,)) for b in self.batches]
        for t in ts:
            t.start()
        for t in ts:
            t.join()
        if errs:
            raise errs[0]

    def update(self, l=None, u=None, q=None):
        """New bounds / linear costs packed in the caller's order."""
        offs_m = np.cumsum([0] + [int(s[-1]) for s in self.msplit])
        offs_n = np.cumsum([0] + [int(s[-1]) for s in self.nsplit])
        jobs = []
        for k, b in enumerate(self.batches):
            jobs.append((b, None if l is None else l[offs_m[k]:offs_m[k + 1]],
                         None if u is None else u[offs_m[k]:offs_m[k + 1]],
                         None if q is None else q[offs_n[k]:offs_n[k + 1]]))
        rcs = {}

        def upd(b):
            for bb, ll, uu, qq in jobs:
                if bb is b:
                    rcs[id(b)] = b.update(l=ll, u=uu, q=qq)

        self._each(upd)
        return max(rcs.values()) if rcs else 0

    def solve(self) -> Dict[str, np.ndarray]:
        """Solve every device's share concurrently; results in the caller's order."""
        sols = {}

        def run(b):
            rc = b.solve()
            if rc:
                raise RuntimeError(f"batch solve failed: {rc}")
            sols[id(b)] = b.solution()

        self._each(run)
        parts = [sols[id(b)] for b in self.batches]
        return {k: np.concatenate([p[k] for p in parts]) for k in parts[0]}

    def cleanup(self):
        for b in self.batches:
            b.cleanup()
        self.batches = []
