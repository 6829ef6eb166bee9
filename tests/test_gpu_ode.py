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


TDVP_CASES = ['tdvp1_ising_d5_krylov', 'tdvp1_ising_d5_exact', 'tdvp2_ising_d5_krylov', 'tdvp2_ising_d6_exact_r3',
              'tdvp1_ising_d6_krylov4']


@pytest.mark.parametrize('name', TDVP_CASES)
def test_tdvp_matches_reference(golden, name):
    """Every state of the device TDVP run against the reference's (full tensors,
    relative 1e-10; the local exponentials are converged Krylov approximations
    in place of scipy's expm_multiply, or the same fixed-dimension recurrence)."""
    from scikit_tt_gb300.solvers import ode
    z, cores = golden(name)
    steps = int(z['steps'])
    h = 1j * float(z['step_im'])
    kdim = int(z['krylov_dim'])
    solver = {'method': 'exact'} if kdim == 0 else {'method': 'krylov', 'dimension': kdim}
    norm = int(z['normalize']) if 'normalize' in z else 0
    if name.startswith('tdvp1'):
        sol = ode.tdvp1site(_tt(cores('op')), _tt(cores('x0')), h, steps, local_solver=solver, normalize=norm)
    else:
        mr = int(z['max_rank']) if 'max_rank' in z else 50
        thr = float(z['threshold']) if 'threshold' in z else 1e-12
        sol = ode.tdvp2site(_tt(cores('op')), _tt(cores('x0')), h, steps, local_solver=solver, threshold=thr,
                            max_rank=mr, normalize=norm)
    assert len(sol) == int(z['n_states'])
    for k, t in enumerate(sol):
        assert list(t.ranks) == list(z[f'ranks_{k}'])
        ref = z[f'full_{k}']
        assert np.linalg.norm(O.full_vector(t.cores) - ref) / np.linalg.norm(ref) < 1e-10


def test_tdvp_adaptive_matches_oracle():
    """The adaptive one-/two-site TDVP against the oracle's restatement (the
    reference's own function cannot run: it omits an argument)."""
    from scikit_tt_gb300 import workloads as wl
    from scikit_tt_gb300 import models
    from scikit_tt_gb300.solvers import ode
    rng = np.random.default_rng(5)
    op = models.ising(6, 1.0, 0.9)
    x0 = wl.gaussian_tt(rng, 6, 2, 1)
    x0 = [c / np.linalg.norm(c) for c in x0]
    sol = ode.tdvp(op, _tt(x0), -0.05j, 6, threshold=1e-12, max_rank=3, normalize=2)
    ref = O.tdvp_adaptive([np.array(c) for c in op.cores], x0, -0.05, 6, threshold=1e-12, max_rank=3, normalize=2)
    assert len(sol) == len(ref)
    for t, r in zip(sol, ref):
        assert [c.shape for c in t.cores] == [c.shape for c in r]
        v = O.full_vector(r)
        assert np.linalg.norm(O.full_vector(t.cores) - v) / np.linalg.norm(v) < 1e-10


def test_tdvp_ground_state_energy():
    """The reference's own TDVP test (tests/test_ode.py:135-158): 500 imaginary-time
    steps of tdvp1site / tdvp2site with the local Krylov method reach the Ising
    ground-state energy that the ALS eigensolver finds, to 1e-8."""
    from scikit_tt_gb300 import models
    from scikit_tt_gb300 import tensor_train as tt
    from scikit_tt_gb300.solvers import evp, ode
    N = 5
    operator = models.ising(N, J=1.0, h=1.2)
    init = tt.uniform(N * [2], ranks=15).ortho()
    init = (1 / init.norm()) * init
    eigval, _, _ = evp.als(operator, init, number_ev=1, repeats=10, conv_eps=1e-6, sigma=-100)
    for fn in (ode.tdvp1site, ode.tdvp2site):
        sol = fn(operator, init, -1j * 0.02, 500, local_solver={'method': 'local_krylov'}, normalize=2)
        energy = sol[-1].transpose(conjugate=True) @ operator @ sol[-1]
        assert abs(energy - eigval) < 1e-8
    assert abs(eigval - O.ising_exact_e0(N, 1.0, 1.2)) < 1e-8


def test_tdvp_manhattan_normalisation_and_zero_steps():
    """normalize=1 (the sum of all entries, tensor_train.py:1334-1420) on a positive
    state -- exp(-tau H) of the transverse-field Ising chain is entrywise positive --
    against the oracle; number_of_steps=0 returns the initial value alone."""
    from scikit_tt_gb300 import models
    from scikit_tt_gb300.solvers import ode
    rng = np.random.default_rng(9)
    op = models.ising(5, 1.0, 0.8)
    x0 = [rng.uniform(0.2, 1.0, (r0, 2, 1, r1)) for r0, r1 in zip([1, 2, 2, 2, 2], [2, 2, 2, 2, 1])]
    sol = ode.tdvp1site(op, _tt(x0), -0.03j, 4, local_solver={'method': 'exact'}, normalize=1)
    ref = O.tdvp1site([np.array(c) for c in op.cores], x0, -0.03, 4, kdim=0, normalize=1)
    for t, r in zip(sol, ref):
        v = O.full_vector(r)
        assert np.linalg.norm(O.full_vector(t.cores) - v) / np.linalg.norm(v) < 1e-10
    assert abs(np.sum(O.full_vector(sol[-1].cores)) - 1.0) < 1e-12
    assert len(ode.tdvp2site(op, _tt(x0), -0.03j, 0)) == 1


@pytest.mark.parametrize('prefix,step,steps,order,prev,normalize',
                         [('o2', 0.1, 4, 2, False, 1), ('o4', 0.1, 4, 3, False, 1), ('o2p', 0.05, 3, 2, True, 2)])
def test_hod_matches_reference(golden, prefix, step, steps, order, prev, normalize):
    """Higher-order differencing (ode.py:117-247) on the device: operator products
    (A^3 at order 4), truncated orthonormalisation of operator and vector trains."""
    from scikit_tt_gb300.solvers import ode
    z, cores = golden('ode_hod')
    sol = ode.hod(_tt(cores('op')), _tt(cores('x0')), step, steps, order=order,
                  previous_value=_tt(cores('prev')) if prev else None, normalize=normalize, progress=False)
    _close(sol, _series(z, prefix), 1e-10)
