"""Linear-ODE integrators built on the device ALS against the reference's outputs."""

import numpy as np
import pytest

from oracle import tt_oracle as O

pytestmark = pytest.mark.gpu


def _tt(cores):
    from scikit_tt_gb300.tensor_train import TT
    return TT([np.array(c) for c in cores])


def _series(z, prefix):
    return [z[f'{prefix}_{k}'] for k in range(int(z[prefix + '_n']))]


def _close(sol, ref, tol):
    assert len(sol) == len(ref)
    for t, r in zip(sol, ref):
        v = O.full_vector(t.cores)
        assert np.linalg.norm(v - r) / np.linalg.norm(r) < tol


def test_implicit_euler_and_trapezoidal_match_reference(golden):
    from scikit_tt_gb300.solvers import ode
    z, cores = golden('ode_markov')
    op, x0, guess, steps = _tt(cores('op')), _tt(cores('x0')), _tt(cores('guess')), list(z['steps'])
    sol = ode.implicit_euler(op, x0, guess, steps, progress=False)
    _close(sol, _series(z, 'impl'), 1e-9)
    assert np.allclose(ode.errors_impl_euler(op, sol, steps), z['impl_err'], rtol=1e-6, atol=1e-13)
    sol = ode.trapezoidal_rule(op, x0, guess, steps, progress=False)
    _close(sol, _series(z, 'trap'), 1e-9)
    assert np.allclose(ode.errors_trapezoidal(op, sol, steps), z['trap_err'], rtol=1e-6, atol=1e-13)


def test_explicit_euler_matches_reference(golden):
    from scikit_tt_gb300.solvers import ode
    z, cores = golden('ode_markov')
    op, x0 = _tt(cores('op')), _tt(cores('x0'))
    sol = ode.explicit_euler(op, x0, [0.05, 0.05, 0.05], progress=False)
    _close(sol, _series(z, 'expl'), 1e-10)
    assert np.allclose(ode.errors_expl_euler(op, sol, [0.05, 0.05, 0.05]), z['expl_err'], rtol=1e-4, atol=1e-13)


def test_adaptive_step_size_matches_reference(golden):
    from scikit_tt_gb300.solvers import ode
    z, cores = golden('ode_markov')
    op, x0, guess = _tt(cores('op')), _tt(cores('x0')), _tt(cores('guess'))
    sol, times = ode.adaptive_step_size(op, x0, guess, 2.0, step_size_first=0.05, progress=False)
    assert np.allclose(times, z['adapt_times'], rtol=1e-9, atol=1e-12)
    _close(sol, _series(z, 'adapt'), 1e-9)
