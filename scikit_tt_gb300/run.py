"""Run one seeded ALS workload on the GPU and print the engine statistics.

    python -m scikit_tt_gb300.run coupled --precision mixed --repeats 1
    python -m scikit_tt_gb300.run ising --repeats 2
    python -m scikit_tt_gb300.run tdvp --d 8 --count 1

Used for profiling (one warm-up solve, then ``--count`` measured solves).
"""

from __future__ import annotations

import argparse
import json

from . import workloads as wl
from .solvers import evp, sle
from .tensor_train import TT


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('workload', choices=['laplace', 'coupled', 'ising', 'tdvp'])
    ap.add_argument('--precision', default='fp64', choices=['fp64', 'mixed'])
    ap.add_argument('--repeats', type=int, default=None)
    ap.add_argument('--d', type=int, default=None)
    ap.add_argument('--rank', type=int, default=None)
    ap.add_argument('--count', type=int, default=1)
    ap.add_argument('--tol', type=float, default=0.0)
    ap.add_argument('--batch', type=int, default=0, help='solve this many seeded instances in one batch launch')
    ap.add_argument('--variant', type=int, default=-1,
                    help='launch variant of batched calls (ttals_set_batch_variant; -1: autotuned)')
    a = ap.parse_args()
    kw = {}
    if a.d:
        kw['d'] = a.d
    if a.rank:
        kw['x_rank'] = a.rank
    if a.workload == 'tdvp':
        # two-site imaginary-time TDVP on the Ising chain (Krylov exponentials, Jacobi SVD splits)
        from .solvers import ode
        w = wl.tdvp_ising(**({'d': a.d} if a.d else {}), **({'max_rank': a.rank} if a.rank else {}))
        for k in range(a.count + 1):
            ode.tdvp2site(TT([c.copy() for c in w.op]), TT([c.copy() for c in w.x0]), w.step_size, w.steps,
                          max_rank=w.max_rank, normalize=2)
        print(json.dumps(ode.last_stats))
        return
    if a.workload == 'ising':
        w = wl.ising_evp(**kw)
        rep = a.repeats or w.repeats
        for k in range(a.count + 1):
            val, _, its = evp.als(TT([c.copy() for c in w.op]), TT([c.copy() for c in w.x0]), repeats=rep,
                                  sigma=w.sigma)
        print(json.dumps({'eigenvalue': float(val), 'iterations': its, **evp.last_stats}))
        return
    w = wl.laplace_sle(**kw) if a.workload == 'laplace' else wl.coupled_sle(**kw)
    rep = a.repeats or w.repeats
    if a.batch:
        from . import _lib
        _lib.check(_lib.load().ttals_set_batch_variant(_lib.context(), a.variant))
        build = wl.laplace_sle if a.workload == 'laplace' else wl.coupled_sle
        probs = []
        for j in range(a.batch):
            wj = build(seed=j, **kw)
            probs.append((TT([c.copy() for c in wj.op]), TT([c.copy() for c in wj.x0]),
                          TT([c.copy() for c in wj.rhs])))
        for k in range(a.count + 1):
            _, st = sle.als_batch(probs, repeats=rep, precision=a.precision, tol=a.tol)
        print(json.dumps(st))
        return
    for k in range(a.count + 1):
        _, st = sle.als_ex(TT([c.copy() for c in w.op]), TT([c.copy() for c in w.x0]),
                           TT([c.copy() for c in w.rhs]), repeats=rep, precision=a.precision, tol=a.tol)
    print(json.dumps(st))


if __name__ == '__main__':
    main()
