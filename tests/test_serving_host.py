"""Host logic of the continuous-batching server on CPU, against a fake of the
asynchronous job API (ttals_submit / ttals_job_poll_each / ttals_job_fetch /
ttals_job_finish): requests are grouped first come first served (largest
first inside a job), a job the
memory budget cannot hold (TTALS_ERR_NOMEM) waits until running jobs release
theirs, at most ``max_jobs`` jobs run at once, and each request completes on
its own, in the order its CTA finishes.  The rank rule comes from the real
library (host-only entry point); nothing touches a GPU."""

import ctypes as C

import pytest

from scikit_tt_gb300 import _lib, serving
from scikit_tt_gb300 import workloads as wl


class FakeJobs:
    """Each job completes one request per poll, last request first."""

    def __init__(self, real, budget, per_request):
        self.ttals_als_ranks = real.ttals_als_ranks
        self.budget, self.per_request = budget, per_request
        self.in_use = self.peak = self.nomem = 0
        self.jobs, self.members, self.running_max = {}, [], 0

    def ttals_submit(self, ctx, n, arr, prec, tol, hp):
        need = n * self.per_request
        if self.in_use + need > self.budget:
            self.nomem += 1
            return _lib.ERR_NOMEM
        self.in_use += need
        self.peak = max(self.peak, self.in_use)
        jid = len(self.members) + 1
        self.jobs[jid] = {'arr': arr, 'n': n, 'todo': list(range(n - 1, -1, -1)), 'need': need}
        self.members.append([arr[i].out_data for i in range(n)])
        self.running_max = max(self.running_max, len(self.jobs))
        hp._obj.value = jid
        return _lib.OK

    def ttals_job_poll_each(self, h, flags):
        job = self.jobs[h.value]
        if job['todo']:
            flags[job['todo'].pop(0)] = 1
        return _lib.OK

    def ttals_job_fetch(self, h, i):
        r = self.jobs[h.value]['arr'][i]
        r.out_data[0] = 1000.0 * h.value + i
        r.out_value[0] = -float(i)
        r.out_iterations[0] = i + 1
        return _lib.OK

    def ttals_job_report(self, h, i, out, cap):
        out[0] = 1e-12 * (i + 1)
        return _lib.OK

    def ttals_job_finish(self, h, st):
        job = self.jobs.pop(h.value)
        self.in_use -= job['need']
        st._obj.local_solves = job['n']
        return _lib.OK


@pytest.fixture
def fake(monkeypatch):
    from scikit_tt_gb300 import build_ext
    build_ext.build()
    real = _lib.load()

    def make(budget, per_request):
        f = FakeJobs(real, budget, per_request)
        monkeypatch.setattr(_lib, 'load', lambda: f)
        monkeypatch.setattr(_lib, 'context', lambda: C.c_void_p(1))
        return f
    return make


def _requests(k):
    out = []
    for j in range(k):
        if j % 3 == 2:
            w = wl.ising_evp(d=4, x_rank=2, repeats=1)
            out.append(serving.Request('evp', w.op, w.x0, repeats=1, sigma=w.sigma))
        else:
            w = wl.laplace_sle(d=4, n=2, rhs_rank=2, x_rank=2, repeats=1, seed=j)
            out.append(serving.Request('sle', w.op, w.x0, w.rhs, repeats=1))
    return out


def test_budget_admission_and_per_request_completion(fake):
    f = fake(budget=4, per_request=1)           # one job of three requests fits, not two; 3 + 1 does
    srv = serving.Server(max_batch=3, max_jobs=8)
    reqs = _requests(7)
    for r in reqs:
        srv.submit(r)
    clock = iter(range(1, 10 ** 6)).__next__
    srv.drain(lambda: float(clock()), timeout=60)
    assert not srv.queue and not srv.jobs
    assert f.nomem > 0 and f.peak == 4 and f.running_max == 2
    assert len(srv.finished) == 7 and len(srv.stats) == 3
    assert sorted(s['local_solves'] for s in srv.stats) == [1, 3, 3]   # in the order jobs finish
    # first come, first served across jobs: requests 0-2 in job 1, 3-5 in job 2, 6 in job 3;
    # inside a job the largest request first (the eigenproblem of each three here)
    for job in range(3):
        members = reqs[3 * job:3 * job + 3]
        order = sorted(members, key=lambda r: r.work_estimate(), reverse=True)
        assert order[0].kind == 'evp' or len(members) == 1
        for idx, r in enumerate(order):
            assert r.solution.cores[0].reshape(-1)[0] == 1000.0 * (job + 1) + idx
            if r.kind == 'evp':
                assert r.value == -float(idx) and r.iterations == idx + 1
    # within a job, requests complete in the order their CTAs finish (last first here)
    first = sorted(reqs[:3], key=lambda r: r.work_estimate(), reverse=True)
    assert [id(r) for r in srv.finished[:3]] == [id(r) for r in first[::-1]]
    assert all(r.done > 0 for r in reqs)


def test_max_jobs_caps_concurrency(fake):
    f = fake(budget=10 ** 9, per_request=1)
    srv = serving.Server(max_batch=2, max_jobs=2)
    for r in _requests(9):
        srv.submit(r)
    srv.pump(lambda: 0.0)
    assert len(srv.jobs) == 2 and len(srv.queue) == 5
    clock = iter(range(1, 10 ** 6)).__next__
    srv.drain(lambda: float(clock()), timeout=60)
    assert len(srv.finished) == 9 and f.running_max == 2 and f.nomem == 0


def test_run_stream_groups_arrivals(fake):
    fake(budget=10 ** 9, per_request=1)
    items = [(0.0, 'sle', wl.laplace_sle(d=4, n=2, rhs_rank=2, x_rank=2, repeats=1, seed=j)) for j in range(5)]
    done, wall, stats = serving.run_stream(items, duration_cap=1.0, max_batch=2, batch_window=0.001)
    assert len(done) == 5 and sum(s['local_solves'] for s in stats) == 5
    assert all(r.done >= r.arrival for r in done)


def test_request_kinds_map_to_the_abi():
    """Served request kinds and their descriptors (host only): a generalised
    eigenproblem travels as TTALS_REQ_GEVP with operator_gevp in the rhs slot,
    and it weighs like an eigenproblem in the largest-first order of a job."""
    from scikit_tt_gb300 import build_ext
    build_ext.build()
    d = 4
    A = wl.ising_op(d, 1.0, 1.2)
    B = wl.laplace_op(d, 2, h=1.0, shift=1.0)
    x0 = wl.gaussian_tt(__import__('numpy').random.default_rng(0), d, 2, 2)
    rg = serving.Request('gevp', A, x0, B, repeats=2, solver='eigh')
    re_ = serving.Request('evp', A, x0, repeats=2)
    dg, de = rg._descriptor(), re_._descriptor()
    assert dg.kind == _lib.REQ_GEVP and de.kind == _lib.REQ_EVP
    assert dg.rhs.order == d and dg.rhs.ranks[1] == B[0].shape[3]
    assert dg.solver == _lib.EVP_SOLVERS['eigh']
    assert rg.work_estimate() == re_.work_estimate() > 0
