"""Alternating ridge regression (regression.arr) on the device against the reference's outputs."""

import numpy as np
import pytest

from oracle import tt_oracle as O
from tests.test_oracle_golden import ARR_CASES, arr_inputs, kuramoto_basis, three_mode_basis

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize('name', ARR_CASES)
def test_arr_matches_reference(golden, name):
    """Every fitted train against the reference's (full tensors, relative 1e-10):
    the least-squares fits follow gelss (QR, then the SVD of R with the same
    relative cut)."""
    from scikit_tt_gb300.data_driven import regression
    from scikit_tt_gb300.tensor_train import TT
    z, _ = golden(name)
    _, x0, refs = arr_inputs(z)
    basis = kuramoto_basis() if name.startswith('arr_kuramoto') else three_mode_basis()
    sols = regression.arr(z['x'], z['y'], basis, TT([c.copy() for c in x0]), repeats=int(z['repeats']),
                          rcond=float(z['rcond']), progress=False)
    assert len(sols) == len(refs)
    for s, r in zip(sols, refs):
        assert [c.shape for c in s.cores] == [c.shape for c in r]
        v = O.full_vector(r)
        assert np.linalg.norm(O.full_vector(s.cores) - v) / np.linalg.norm(v) < 1e-10


def test_arr_kuramoto_coefficients():
    """The reference's own ARR test (tests/test_regression.py:116-137): ten sweeps
    with rcond 1e-12 recover the exact coefficient tensor of the Kuramoto model
    to 1e-5; a list of initial guesses is updated in place."""
    from scikit_tt_gb300 import tensor_train as tt
    from scikit_tt_gb300.data_driven import regression
    z = np.load(__import__('os').path.join(__import__('os').path.dirname(__file__), 'golden',
                                           'arr_kuramoto_rcond12.npz'))
    guesses = [tt.ones([11, 11], [1, 1], 11) for _ in range(10)]
    xi = regression.arr(z['x'], z['y'], kuramoto_basis(), guesses, repeats=10, rcond=1e-12, progress=False)
    assert xi is guesses
    full = np.stack([O.full_vector(t.cores).reshape(11, 11) for t in xi], axis=2)
    exact = z['xi_exact_full']
    assert np.linalg.norm(full.reshape(-1) - exact) / np.linalg.norm(exact) < 1e-5


def test_arr_single_mode_matches_oracle():
    """One basis list (a one-core train): the fit is a single least-squares solve."""
    from scikit_tt_gb300.data_driven import regression, transform as tdt
    from scikit_tt_gb300.tensor_train import TT
    rng = np.random.default_rng(4)
    x = rng.uniform(-2, 2, (1, 300))
    y = np.vstack([np.exp(-x[0] ** 2), np.sin(3 * x[0])])
    basis = [[tdt.ConstantFunction(0), tdt.Identity(0), tdt.Monomial(0, 2), tdt.GaussFunction(0, 0.0, 0.3),
              tdt.Sin(0, 3), tdt.Cos(0, 3)]]
    g = [rng.standard_normal((1, 6, 1, 1))]
    sols = regression.arr(x, y, basis, TT([c.copy() for c in g]), repeats=2, rcond=1e-8)
    refs = O.arr(regression.evaluate_basis(x, basis), y, [g, g], repeats=2, rcond=1e-8)
    for s, r in zip(sols, refs):
        v = O.full_vector(r)
        assert np.linalg.norm(O.full_vector(s.cores) - v) / np.linalg.norm(v) < 1e-10
