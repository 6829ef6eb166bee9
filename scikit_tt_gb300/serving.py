"""Batched and served ALS requests (linear systems and eigenproblems).

``solve_batch`` runs a list of requests in one launch (one CTA per request).
``Server`` is the continuous-batching loop: requests are admitted as they
arrive, grouped into jobs launched on their own streams while earlier jobs
still run (so their work overlaps on the device), and admitted only while
the device-memory budget holds; each request's latency is measured from its
arrival to its completion.  Admission is per CTA slot in effect: a job's CTA
exits once its job has no request left, and the hardware scheduler gives its
SM to the CTAs of the jobs launched after it.
"""

from __future__ import annotations

import ctypes as C
import time
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

from . import _lib
from .tensor_train import TT

_PREC = {'fp64': _lib.PREC_FP64, 'mixed': _lib.PREC_MIXED}


@dataclass
class Request:
    """One ALS problem.  kind 'sle': ``op @ x = rhs`` (sle.py:10); kind 'evp':
    eigenpair of the symmetric ``op`` (evp.py:17); kind 'gevp': eigenpair of
    ``op x = lambda rhs x`` with ``rhs`` the symmetric positive definite
    ``operator_gevp`` (evp.py:17 with operator_gevp)."""
    kind: str
    op: List[np.ndarray]
    x0: List[np.ndarray]
    rhs: Optional[List[np.ndarray]] = None
    repeats: int = 1
    solver: str = None
    sigma: float = 1.0
    conv_eps: float = 1e-10
    arrival: float = 0.0
    # filled on completion
    solution: Optional[TT] = None
    value: Optional[float] = None
    iterations: Optional[int] = None
    local_residual: Optional[float] = None   # worst final relative residual of its local solves
    done: float = 0.0
    _keep: list = field(default_factory=list, repr=False)

    def _descriptor(self):
        lib = _lib.load()
        op, x0 = _lib.Packed(self.op), _lib.Packed(self.x0)
        rhs = _lib.Packed(self.rhs) if self.kind in ('sle', 'gevp') else x0
        dims = np.array([c.shape[1] for c in self.op], dtype=np.int64)
        ranks = np.zeros(len(dims) + 1, dtype=np.int64)
        _lib.check(lib.ttals_als_ranks(len(dims), _lib.i64ptr(dims), _lib.i64ptr(x0.ranks), _lib.i64ptr(ranks)))
        out = np.empty(max(1, int(sum(ranks[i] * dims[i] * ranks[i + 1] for i in range(len(dims))))))
        val = np.zeros(1)
        its = np.zeros(1, dtype=np.int32)
        r = _lib.Request()
        r.kind = {'sle': _lib.REQ_SLE, 'evp': _lib.REQ_EVP, 'gevp': _lib.REQ_GEVP}[self.kind]
        r.op, r.x0, r.rhs = op.desc, x0.desc, rhs.desc
        r.repeats = int(self.repeats)
        solver = self.solver or ('solve' if self.kind == 'sle' else 'eig')
        r.solver = (_lib.SLE_SOLVERS if self.kind == 'sle' else _lib.EVP_SOLVERS)[solver]
        r.sigma = float(self.sigma)
        r.conv_eps = float(self.conv_eps)
        r.out_data = _lib.dptr(out)
        r.out_value = _lib.dptr(val)
        r.out_iterations = its.ctypes.data_as(C.POINTER(C.c_int32))
        self._keep = [op, x0, rhs, out, val, its, ranks, dims]
        return r

    def work_estimate(self) -> float:
        """Relative device work: flops of the local-operator application at
        every site (ranks of the initial guess, operator ranks, mode sizes),
        times the sweeps; an eigenproblem counts 4x (FP64 Lanczos with full
        reorthogonalisation, against the mixed-precision GMRES of a system)."""
        r = [c.shape[0] for c in self.x0] + [1]
        R = [c.shape[0] for c in self.op] + [1]
        w = 0.0
        for i, c in enumerate(self.op):
            n, a, s, R0, R1 = c.shape[1], r[i], r[i + 1], R[i], R[i + 1]
            w += a * a * R0 * n * s + a * s * n * n * R0 * R1 + a * n * s * s * R1
        return w * max(1, int(self.repeats)) * (1.0 if self.kind == 'sle' else 4.0)

    def _complete(self):
        _, _, _, out, val, its, ranks, dims = self._keep
        self.solution = TT(_lib.unpack(out, dims, [1] * len(dims), ranks))
        if self.kind != 'sle':
            self.value = float(val[0])
            self.iterations = int(its[0])
        self._keep = []


def solve_batch(requests: List[Request], precision: str = 'mixed', tol: float = 0.0):
    """Solve all requests in one launch; returns the engine statistics."""
    arr = (_lib.Request * len(requests))(*[r._descriptor() for r in requests])
    st = _lib.Stats()
    _lib.check(_lib.load().ttals_solve_batch(_lib.context(), len(requests), arr, _PREC[precision], float(tol), 0, st))
    for r in requests:
        r._complete()
    return st.as_dict()


class Server:
    """Continuous batching over the asynchronous job API (ttals_submit)."""

    def __init__(self, precision: str = 'mixed', tol: float = 0.0, max_batch: int = 608, max_jobs: int = 64):
        self.prec = _PREC[precision]
        self.tol = float(tol)
        self.max_batch = max_batch
        self.max_jobs = max_jobs
        self.queue: List[Request] = []
        self.jobs = []       # (handle, requests, descriptor array)
        self.finished: List[Request] = []
        self.stats = []

    def submit(self, req: Request):
        self.queue.append(req)

    def _launch(self, clock):
        lib, ctx = _lib.load(), _lib.context()
        # first come, first served across jobs; inside a job the largest
        # requests first (the job's CTAs take requests in index order, so the
        # longest ones start at once instead of extending the job's tail)
        take = sorted(self.queue[:self.max_batch], key=lambda r: r.work_estimate(), reverse=True)
        arr = (_lib.Request * len(take))(*[r._descriptor() for r in take])
        h = C.c_void_p()
        st = lib.ttals_submit(ctx, len(take), arr, self.prec, self.tol, C.byref(h))
        if st == _lib.ERR_NOMEM:
            return False         # budget held by running jobs: admit later
        _lib.check(st)
        self.queue = self.queue[len(take):]
        self.jobs.append({'h': h, 'reqs': take, 'arr': arr, 'fetched': set(),
                          'flags': (C.c_int32 * len(take))()})
        return True

    def pump(self, clock, launch: bool = True) -> int:
        """Complete finished jobs and (if ``launch``) launch queued requests;
        returns the number of requests completed by this call."""
        lib = _lib.load()
        completed = 0
        still = []
        for job in self.jobs:
            h, reqs, fetched, flags = job['h'], job['reqs'], job['fetched'], job['flags']
            # requests complete one by one: a slow request does not hold the others back
            _lib.check(lib.ttals_job_poll_each(h, flags))
            for i in range(len(reqs)):
                if flags[i] and i not in fetched:
                    _lib.check(lib.ttals_job_fetch(h, i))
                    rep = np.zeros(4)
                    _lib.check(lib.ttals_job_report(h, i, _lib.dptr(rep), 4))
                    reqs[i].local_residual = float(rep[0])
                    reqs[i]._complete()
                    reqs[i].done = clock()
                    fetched.add(i)
                    self.finished.append(reqs[i])
                    completed += 1
            if len(fetched) == len(reqs):
                st = _lib.Stats()
                _lib.check(lib.ttals_job_finish(h, C.byref(st)))
                self.stats.append(st.as_dict())
            else:
                still.append(job)
        self.jobs = still
        while launch and self.queue and len(self.jobs) < self.max_jobs:
            if not self._launch(clock):
                break
        return completed

    def drain(self, clock, timeout: float = 600.0):
        t0 = time.perf_counter()
        while (self.queue or self.jobs) and time.perf_counter() - t0 < timeout:
            if self.pump(clock) == 0:
                time.sleep(0.0005)


def run_stream(stream, duration_cap: float, precision='mixed', max_batch=608, max_jobs=64, batch_window=0.005):
    """Replay ``(arrival_s, kind, instance)`` items against a Server in real
    time.  Requests are admitted when they arrive; a job is launched when the
    queue holds ``max_batch`` requests or the oldest has waited
    ``batch_window`` seconds.  Returns the finished requests and wall time."""
    srv = Server(precision=precision, max_batch=max_batch, max_jobs=max_jobs)
    items = list(stream)
    t0 = time.perf_counter()
    clock = lambda: time.perf_counter() - t0  # noqa: E731
    k = 0
    while k < len(items) or srv.queue or srv.jobs:
        now = clock()
        while k < len(items) and items[k][0] <= now:
            t, kind, inst = items[k]
            if kind == 'sle':
                r = Request('sle', inst.op, inst.x0, inst.rhs, repeats=inst.repeats, arrival=t)
            else:
                r = Request('evp', inst.op, inst.x0, repeats=inst.repeats, sigma=inst.sigma, arrival=t)
            srv.queue.append(r)
            k += 1
        ready = bool(srv.queue) and (len(srv.queue) >= max_batch or now - srv.queue[0].arrival >= batch_window
                                     or k >= len(items))
        if srv.pump(clock, launch=ready) == 0 and not ready:
            time.sleep(0.0005)
        if now > duration_cap + 600:
            break
    return srv.finished, clock(), srv.stats
