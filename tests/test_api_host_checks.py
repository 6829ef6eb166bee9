"""The drop-in's argument checks run on the host before any device work, with
the exception types the reference's callers expect: unknown solver strings
and precisions raise ValueError (the reference silently skips the local
solve, sle.py:505-509: a documented deviation); features outside the device
path raise NotImplementedError.  The library is replaced by a stub that fails
if anything reaches it."""

import numpy as np
import pytest

from scikit_tt_gb300 import _lib, models
from scikit_tt_gb300 import workloads as wl
from scikit_tt_gb300.solvers import evp, sle
from scikit_tt_gb300.tensor_train import TT


@pytest.fixture(autouse=True)
def no_device(monkeypatch):
    def touched():
        raise AssertionError('the device library was reached before the argument check')
    monkeypatch.setattr(_lib, 'load', touched)
    monkeypatch.setattr(_lib, 'context', touched)


def _sle():
    w = wl.laplace_sle(d=4, n=2, rhs_rank=2, x_rank=2, repeats=1)
    return TT([c.copy() for c in w.op]), TT([c.copy() for c in w.x0]), TT([c.copy() for c in w.rhs])


def test_sle_checks():
    A, x0, b = _sle()
    with pytest.raises(ValueError):
        sle.als(A, x0, b, solver='cg')
    with pytest.raises(ValueError):
        sle.als_ex(A, x0, b, precision='bf16')
    with pytest.raises(ValueError):
        sle.mals(A, x0, b, solver='qr')
    with pytest.raises(NotImplementedError):
        sle.mals(TT([A.cores[0][:, :, :, :1]]), TT([x0.cores[0][:, :, :, :1]]), TT([b.cores[0][:, :, :, :1]]))
    xc = TT([c.astype(complex) for c in x0.cores])
    with pytest.raises(NotImplementedError):
        sle.als(A, xc, b)


def test_evp_checks():
    H = models.ising(4, 1.0, 0.7)
    x0 = TT([np.ones((1, 2, 1, 2)), np.ones((2, 2, 1, 2)), np.ones((2, 2, 1, 2)), np.ones((2, 2, 1, 1))])
    with pytest.raises(ValueError):
        evp.als(H, x0, solver='lobpcg')
    M = 2.0 * TT([np.eye(2).reshape(1, 2, 2, 1) for _ in range(4)])
    # generalised problems run with number_ev == 1, no deflation, symmetric operators
    with pytest.raises(NotImplementedError):
        evp.als(H, x0, operator_gevp=M, number_ev=2)
    with pytest.raises(NotImplementedError):
        evp.als(H, x0, previous=[x0], operator_gevp=M)
    with pytest.raises(NotImplementedError):
        evp.als(H, x0, number_ev=9)
    rng = np.random.default_rng(0)
    N = TT([rng.standard_normal((1, 2, 2, 1)) for _ in range(4)])
    with pytest.raises(NotImplementedError):
        evp.als(N, x0, solver='eigh')
    with pytest.raises(NotImplementedError):
        evp.als(H, x0, operator_gevp=N)
    with pytest.raises(ValueError):
        evp.als(H, x0, operator_gevp=TT([2 * np.eye(3).reshape(1, 3, 3, 1) for _ in range(4)]))


def test_identity_gevp_is_accepted():
    """operator_gevp = identity is the plain problem (evp.py:337-383 with M = I)."""
    assert evp._is_identity(None)
    assert evp._is_identity(TT([np.eye(3).reshape(1, 3, 3, 1) for _ in range(3)]))
    assert not evp._is_identity(TT([2 * np.eye(3).reshape(1, 3, 3, 1) for _ in range(3)]))
    assert evp._is_symmetric(models.ising(5, 1.0, 1.3))
