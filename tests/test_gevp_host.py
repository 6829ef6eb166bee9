"""Host side of generalised eigenproblems (evp.py:17 with operator_gevp): the
drop-in routes a symmetric operator with a symmetric positive definite
operator_gevp to the batch engine as one TTALS_REQ_GEVP request (operator_gevp
in the request's rhs slot, FP64) and unpacks the eigenvalue, the eigentensor
in the rank schedule of ttals_als_ranks and the sweep count.  The library is
the real one for the host-only rank rule and a fake for the batch call, so
nothing touches a GPU."""

import ctypes as C

import numpy as np

from scikit_tt_gb300 import _lib
from scikit_tt_gb300 import workloads as wl
from scikit_tt_gb300.solvers import evp
from scikit_tt_gb300.tensor_train import TT


class FakeBatch:
    def __init__(self, real):
        self.ttals_als_ranks = real.ttals_als_ranks
        self.calls = []

    def ttals_solve_batch(self, ctx, count, arr, prec, tol, out_on_device, st):
        r = arr[0]
        self.calls.append({'count': count, 'kind': r.kind, 'prec': prec, 'solver': r.solver,
                           'gevp_order': r.rhs.order, 'gevp_rank1': r.rhs.ranks[1], 'repeats': r.repeats,
                           'sigma': r.sigma, 'on_device': out_on_device})
        r.out_value[0] = -1.25
        r.out_iterations[0] = 3
        for k in range(self.size):   # the output buffer the caller sized: sum of the output cores
            r.out_data[k] = float(k)
        st.local_solves = 7
        return _lib.OK


def test_gevp_goes_to_the_batch_engine(monkeypatch):
    from scikit_tt_gb300 import build_ext
    build_ext.build()
    real = _lib.load()
    fake = FakeBatch(real)
    d = 4
    A = TT(wl.ising_op(d, 1.0, 1.2))
    B = TT(wl.laplace_op(d, 2, h=1.0, shift=1.0))
    x0 = TT(wl.gaussian_tt(np.random.default_rng(1), d, 2, 2))
    dims = np.array(A.row_dims, dtype=np.int64)
    ranks = np.zeros(d + 1, dtype=np.int64)
    xr = np.array(x0.ranks, dtype=np.int64)
    _lib.check(real.ttals_als_ranks(d, _lib.i64ptr(dims), _lib.i64ptr(xr), _lib.i64ptr(ranks)))
    fake.size = int(sum(ranks[i] * dims[i] * ranks[i + 1] for i in range(d)))
    monkeypatch.setattr(_lib, 'load', lambda: fake)
    monkeypatch.setattr(_lib, 'context', lambda: C.c_void_p(1))
    val, vec, its = evp.als(A, x0, operator_gevp=B, repeats=3, solver='eigh', sigma=0.5)
    assert len(fake.calls) == 1
    call = fake.calls[0]
    assert call['count'] == 1 and call['kind'] == _lib.REQ_GEVP and call['prec'] == _lib.PREC_FP64
    assert call['solver'] == _lib.EVP_SOLVERS['eigh'] and call['repeats'] == 3 and call['sigma'] == 0.5
    assert call['gevp_order'] == d and call['gevp_rank1'] == B.cores[0].shape[3] and call['on_device'] == 0
    assert val == -1.25 and its == 3
    assert [c.shape[0] for c in vec.cores] + [1] == list(ranks)
    assert np.array_equal(np.concatenate([c.ravel() for c in vec.cores]), np.arange(fake.size, dtype=float))
    assert evp.last_stats['local_solves'] == 7
