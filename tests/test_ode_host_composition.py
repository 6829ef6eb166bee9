"""Host logic of the integrators that are compositions of device operations
(``ode.hod``, ``ode.explicit_euler``): the device primitives they call --
``TT.__matmul__``, the truncated ``ortho_left``/``ortho_right`` and the 2-norm,
each checked on the GPU by its own tests -- are replaced here by the oracle's
versions (pinned to the reference), so the composition itself is checked
against the reference's results on CPU."""

import numpy as np
import pytest

from oracle import tt_oracle as O
from scikit_tt_gb300.solvers import ode
from scikit_tt_gb300.tensor_train import TT


@pytest.fixture
def oracle_primitives(monkeypatch):
    def matmul(self, other):
        prod = TT(O.tt_matmul(self.cores, other.cores))
        if np.prod(prod.row_dims) == 1 and np.prod(prod.col_dims) == 1:
            return prod.element([0] * prod.order * 2)
        return prod

    def ortho_trunc(self, direction, first, last, threshold, caps):
        assert (first, last) == ((0, self.order - 2) if direction == 0 else (self.order - 1, 1))
        inner = [m for m in caps[1:-1] if m != np.inf]
        cap = max(inner) if inner else np.inf
        self.cores = (O.ortho_left if direction == 0 else O.ortho_right)(self.cores, threshold, cap)
        self.ranks = [c.shape[0] for c in self.cores] + [1]
        return self

    plain_norm = TT.norm

    def norm(self, p=2):
        return O.norm2(self.cores) if p == 2 else plain_norm(self, p)

    def untruncated(self, *a, **k):
        raise AssertionError('these integrators always truncate (threshold > 0)')

    monkeypatch.setattr(TT, '__matmul__', matmul)
    monkeypatch.setattr(TT, '_ortho_trunc', ortho_trunc)
    monkeypatch.setattr(TT, '_ortho', untruncated)
    monkeypatch.setattr(TT, 'norm', norm)


def _same(z, prefix, sol):
    assert len(sol) == int(z[prefix + '_n'])
    for k, s in enumerate(sol):
        r = z[f'{prefix}_{k}']
        assert np.linalg.norm(s.full().reshape(-1) - r) / np.linalg.norm(r) < 1e-12


@pytest.mark.parametrize('prefix,step,steps,order,prev,normalize',
                         [('o2', 0.1, 4, 2, False, 1), ('o4', 0.1, 4, 3, False, 1), ('o2p', 0.05, 3, 2, True, 2)])
def test_hod_composition(golden, oracle_primitives, prefix, step, steps, order, prev, normalize):
    z, cores = golden('ode_hod')
    sol = ode.hod(TT(cores('op')), TT(cores('x0')), step, steps, order=order,
                  previous_value=TT(cores('prev')) if prev else None, normalize=normalize, progress=False)
    _same(z, prefix, sol)


def test_explicit_euler_composition(golden, oracle_primitives):
    z, cores = golden('ode_markov')
    op, x0 = TT(cores('op')), TT(cores('x0'))
    sol = ode.explicit_euler(op, x0, [0.05, 0.05, 0.05], progress=False)
    _same(z, 'expl', sol)
    np.testing.assert_allclose(ode.errors_expl_euler(op, sol, [0.05] * 3), z['expl_err'], atol=1e-14)
