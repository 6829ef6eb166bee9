"""The CPU oracle against outputs of the reference itself (tests/golden)."""

import numpy as np
import pytest
import scipy.linalg as sla

from oracle import tt_oracle as O
from scikit_tt_gb300 import workloads as wl


@pytest.mark.parametrize('name', ['sle_laplace_d10', 'sle_laplace_d10_lu', 'sle_laplace_d10_r8', 'sle_coupled_d8'])
def test_oracle_sle_matches_reference(golden, name):
    z, cores = golden(name)
    sol = O.sle_als(cores('op'), cores('x0'), cores('rhs'), repeats=int(z['repeats']), solver=str(z['solver']))
    ref = cores('sol')
    assert [c.shape for c in sol] == [c.shape for c in ref]
    assert O.stable_rel_diff(sol, ref) < 1e-12


@pytest.mark.parametrize('solver', ['solve', 'lu'])
def test_oracle_sle_toeplitz_known_answer(golden, solver):
    """The reference's ALS known answer (tests/test_sle.py:37-59), both local solvers."""
    z, cores = golden('sle_toeplitz')
    mat = sla.toeplitz(np.arange(1, 2 ** 10 + 1), np.arange(1, 2 ** 10 + 1)).astype(float)
    from scikit_tt_gb300.tensor_train import _hosvd
    op = _hosvd(mat.reshape([2] * 20), 0, np.inf)
    sol = O.sle_als(op, cores('x0'), cores('rhs'), repeats=1, solver=solver)
    exact = np.linalg.solve(mat, np.ones(1024))
    got = O.full_vector(sol)
    ref = O.full_vector(cores('sol'))
    assert np.linalg.norm(got - exact) / np.linalg.norm(exact) < 1e-7      # test_sle.py:53-59 tolerance
    # cond(Toeplitz) is large: both solutions sit within the reference tolerance of
    # the exact one and within 1e-6 of each other (operator TT gauges differ)
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-6


@pytest.mark.parametrize('name', ['evp_ising_d12_eig', 'evp_ising_d12_eigh'])
def test_oracle_evp_matches_reference(golden, name):
    z, cores = golden(name)
    val, vec, its = O.evp_als(cores('op'), cores('x0'), repeats=int(z['repeats']), solver=str(z['solver']),
                              sigma=float(z['sigma']), conv_eps=float(z['conv_eps']))
    assert abs(val - float(z['val'])) < 1e-10
    assert its == int(z['its'])
    # eigenvectors agree up to sign
    v, r = O.full_vector(vec), O.full_vector(cores('vec'))
    assert min(np.linalg.norm(v - r), np.linalg.norm(v + r)) / np.linalg.norm(r) < 1e-7


@pytest.mark.parametrize('name', ['evp_gevp_ising_d6_eig', 'evp_gevp_ising_d6_eigh'])
def test_oracle_gevp_matches_reference(golden, name):
    """Generalised problem (operator_gevp = SPD mass operator): the oracle's
    stacks and dense local pencil solve against the reference's result, and
    the eigenvalue against the dense pencil's extreme eigenvalue."""
    z, cores = golden(name)
    val, vec, its = O.evp_als(cores('op'), cores('x0'), op_gevp=cores('gevp'), repeats=int(z['repeats']),
                              solver=str(z['solver']), sigma=float(z['sigma']), conv_eps=float(z['conv_eps']))
    assert abs(val - float(z['val'])) < 1e-10
    assert its == int(z['its'])
    want = z['pencil_vals'][0] if str(z['solver']) == 'eig' else z['pencil_vals'][-1]
    assert abs(val - want) < 1e-7      # rank-4 ALS after four sweeps
    v, r = O.full_vector(vec), O.full_vector(cores('vec'))
    assert min(np.linalg.norm(v - r), np.linalg.norm(v + r)) / np.linalg.norm(r) < 1e-7


def test_oracle_ising_free_fermion():
    # E0 of the d=12 chain from free fermions vs the dense spectrum
    op = wl.ising_op(8, 1.0, 1.0)
    H = O.full_matrix(op)
    assert abs(np.linalg.eigvalsh(H)[0] - O.ising_exact_e0(8, 1.0, 1.0)) < 1e-10


def test_oracle_helpers_match_reference(golden):
    z, _ = golden('helpers')
    left = O.stack_left_op(z['Lp'], z['x0c'][:, :, 0, :], z['A0'])
    right = O.stack_right_op(z['Rn'], z['x1c'][:, :, 0, :], z['A1'])
    micro = O.micro_matrix(z['Ls'], z['A0'], z['Rs'])
    np.testing.assert_allclose(left, z['left'], rtol=1e-13, atol=1e-13 * np.abs(z['left']).max())
    np.testing.assert_allclose(right, z['right'], rtol=1e-13, atol=1e-13 * np.abs(z['right']).max())
    np.testing.assert_allclose(micro, z['micro'], rtol=1e-13, atol=1e-13 * np.abs(z['micro']).max())


def test_oracle_tt_ops_match_reference(golden):
    z, cores = golden('ttops')
    t, A = cores('t'), cores('A')
    assert abs(O.norm2(t) - float(z['norm'])) < 1e-12 * float(z['norm'])
    assert abs(O.norm2(A) - float(z['opnorm'])) < 1e-12 * float(z['opnorm'])
    np.testing.assert_allclose(O.full_vector(O.tt_matmul(A, t)), z['prod_full'], rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(O.full_vector(O.ortho_left(t)), z['left_full'], rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(O.full_vector(O.ortho_right(t)), z['right_full'], rtol=1e-12, atol=1e-12)
    assert abs(O.stable_norm(t) - float(z['norm'])) < 1e-12 * float(z['norm'])


BLOCK_CASES = ['evp_markov_eig_k1', 'evp_markov_eig_k3', 'evp_markov_eigs_k3', 'evp_ising_d8_eigh_k3',
               'evp_ising_d8_eig_k3']


def _up_to_sign(v, r):
    return min(np.linalg.norm(v - r), np.linalg.norm(v + r)) / np.linalg.norm(r)


@pytest.mark.parametrize('name', BLOCK_CASES)
def test_oracle_evp_blocks_match_reference(golden, name):
    # nonsymmetric operators and number_ev > 1 (evp.py:386-495 with eig / eigs / eigh)
    z, cores = golden(name)
    k = int(z['number_ev'])
    vals, vecs, its = O.evp_als(cores('op'), cores('x0'), number_ev=k, repeats=int(z['repeats']),
                                solver=str(z['solver']), sigma=float(z['sigma']), conv_eps=float(z['conv_eps']))
    assert its == int(z['its'])
    vals = np.atleast_1d(np.real(vals))
    assert np.max(np.abs(vals - z['vals'])) < 1e-10
    vecs = [vecs] if k == 1 else vecs
    for e in range(k):
        v = O.full_vector(vecs[e])
        v = v * np.exp(-1j * np.angle(v[np.argmax(np.abs(v))]))
        assert _up_to_sign(np.real(v), z[f'vec{e}']) < 1e-8


TDVP_CASES = ['tdvp1_ising_d5_krylov', 'tdvp1_ising_d5_exact', 'tdvp2_ising_d5_krylov', 'tdvp2_ising_d6_exact_r3',
              'tdvp1_ising_d6_krylov4']


def tdvp_args(z):
    """Keyword arguments of one golden TDVP run (tau = -1j * step_size is real)."""
    kw = {'kdim': int(z['krylov_dim'])}
    for key in ('normalize', 'threshold', 'max_rank'):
        if key in z:
            kw[key] = float(z[key]) if key == 'threshold' else int(z[key])
    return float(z['step_im']), int(z['steps']), kw


@pytest.mark.parametrize('name', TDVP_CASES)
def test_oracle_tdvp_matches_reference(golden, name):
    z, cores = golden(name)
    tau, steps, kw = tdvp_args(z)
    fn = O.tdvp1site if name.startswith('tdvp1') else O.tdvp2site
    states = fn(cores('op'), cores('x0'), tau, steps, **kw)
    assert len(states) == int(z['n_states'])
    for k, s in enumerate(states):
        assert [c.shape[0] for c in s] + [1] == list(z[f'ranks_{k}'])
        ref = z[f'full_{k}']
        assert np.linalg.norm(O.full_vector(s) - ref) / np.linalg.norm(ref) < 1e-12


def test_tdvp_refuses_real_time_steps():
    from scikit_tt_gb300.solvers import ode
    from scikit_tt_gb300.tensor_train import TT
    op = TT([np.eye(2).reshape(1, 2, 2, 1)] * 3)
    x = TT([np.ones((1, 2, 1, 1))] * 3)
    with pytest.raises(NotImplementedError):
        ode.tdvp1site(op, x, 0.1, 2)


ARR_CASES = ['arr_kuramoto_rcond12', 'arr_kuramoto_rcond2', 'arr_three_mode']


def arr_inputs(z):
    theta = [z[f'theta_{i}'] for i in range(int(z['theta_n']))]
    x0 = [z[f'x0_{i}'] for i in range(int(z['x0_n']))]
    refs = [[z[f'sol{k}_{i}'] for i in range(int(z[f'sol{k}_n']))] for k in range(int(z['n_out']))]
    return theta, x0, refs


def kuramoto_basis():
    from scikit_tt_gb300.data_driven import transform as tdt
    return [[tdt.ConstantFunction(0)] + [tdt.Sin(i, 1) for i in range(10)],
            [tdt.ConstantFunction(0)] + [tdt.Cos(i, 1) for i in range(10)]]


def three_mode_basis():
    from scikit_tt_gb300.data_driven import transform as tdt
    return [[tdt.ConstantFunction(0), tdt.Identity(0), tdt.Monomial(0, 2), tdt.Sin(0, 2)],
            [tdt.ConstantFunction(1), tdt.Identity(1), tdt.Monomial(1, 2), tdt.Monomial(1, 3),
             tdt.GaussFunction(1, 0.0, 0.5)],
            [tdt.ConstantFunction(2), tdt.Identity(2), tdt.Legendre(2, 2)]]


@pytest.mark.parametrize('name', ARR_CASES)
def test_oracle_arr_matches_reference(golden, name):
    z, _ = golden(name)
    theta, x0, refs = arr_inputs(z)
    sols = O.arr(theta, z['y'], [x0] * len(refs), repeats=int(z['repeats']), rcond=float(z['rcond']))
    for s, r in zip(sols, refs):
        v = O.full_vector(r)
        assert np.linalg.norm(O.full_vector(s) - v) / np.linalg.norm(v) < 1e-12


@pytest.mark.parametrize('name', ['arr_kuramoto_rcond2', 'arr_three_mode'])
def test_basis_functions_match_reference(golden, name):
    """The package's basis functions evaluate to the reference's values."""
    from scikit_tt_gb300.data_driven import regression
    z, _ = golden(name)
    basis = kuramoto_basis() if name.startswith('arr_kuramoto') else three_mode_basis()
    theta = regression.evaluate_basis(z['x'], basis)
    for i, t in enumerate(theta):
        assert np.allclose(t, z[f'theta_{i}'], rtol=1e-14, atol=1e-15)


@pytest.mark.parametrize('name', ['sle_mals_laplace_d6', 'sle_mals_laplace_d6_r4', 'sle_mals_coupled_d5_lu'])
def test_oracle_mals_matches_reference(golden, name):
    """Two-site MALS (sle.py:98-191): same ranks, same tensor."""
    z, cores = golden(name)
    mr = int(z['max_rank'])
    sol = O.sle_mals(cores('op'), cores('x0'), cores('rhs'), repeats=int(z['repeats']), solver=str(z['solver']),
                     threshold=float(z['threshold']), max_rank=np.inf if mr < 0 else mr)
    assert [c.shape[0] for c in sol] + [1] == [int(r) for r in z['ranks']]
    v = O.full_vector(sol)
    assert np.linalg.norm(v - z['full']) / np.linalg.norm(z['full']) < 1e-12


def test_oracle_ode_integrators_match_reference(golden):
    """Implicit / explicit Euler, trapezoidal rule, adaptive step size and their
    error helpers (ode.py:16-636) on a Markov generator."""
    z, cores = golden('ode_markov')
    op, x0, guess = cores('op'), cores('x0'), cores('guess')
    steps = [float(h) for h in z['steps']]

    def same(prefix, sol):
        assert len(sol) == int(z[prefix + '_n'])
        for k, s in enumerate(sol):
            r = z[f'{prefix}_{k}']
            assert np.linalg.norm(O.full_vector(s) - r) / np.linalg.norm(r) < 1e-12

    sol = O.implicit_euler(op, x0, guess, steps)
    same('impl', sol)
    np.testing.assert_allclose(O.errors_impl_euler(op, sol, steps), z['impl_err'], rtol=1e-8, atol=1e-14)
    sol = O.trapezoidal_rule(op, x0, guess, steps)
    same('trap', sol)
    np.testing.assert_allclose(O.errors_trapezoidal(op, sol, steps), z['trap_err'], rtol=1e-8, atol=1e-14)
    sol = O.explicit_euler(op, x0, [0.05] * 3)
    same('expl', sol)
    np.testing.assert_allclose(O.errors_expl_euler(op, sol, [0.05] * 3), z['expl_err'], atol=1e-14)
    sol, times = O.adaptive_step_size(op, x0, guess, 2.0, step_size_first=0.05)
    same('adapt', sol)
    np.testing.assert_allclose(times, z['adapt_times'], rtol=1e-12, atol=1e-15)


@pytest.mark.parametrize('name', ['evp_power_markov', 'evp_power_markov_gevp'])
def test_oracle_power_method_matches_reference(golden, name):
    """Inverse power iteration through sle.als (evp.py:182-250)."""
    z, cores = golden(name)
    op = cores('op')
    gevp = O.tt_eye([c.shape[1] for c in op]) if bool(z['gevp']) else None
    val, vec = O.power_method(op, cores('x0'), gevp, repeats=int(z['repeats']), sigma=float(z['sigma']))
    assert abs(val - float(z['val'])) < 1e-12
    v, r = O.full_vector(vec), z['vec0']
    assert min(np.linalg.norm(v - r), np.linalg.norm(v + r)) / np.linalg.norm(r) < 1e-12


@pytest.mark.parametrize('solver', ['solve', 'lu'])
def test_oracle_mals_toeplitz_known_answer(golden, solver):
    """The reference's own MALS known answer (tests/test_sle.py:61-85): the
    Toeplitz(1..1024) system as an order-10 TT, one MALS sweep with
    threshold 1e-14 and max_rank 10, against the dense solve (tolerance 1e-7
    as there)."""
    z, cores = golden('sle_toeplitz')
    mat = sla.toeplitz(np.arange(1, 2 ** 10 + 1), np.arange(1, 2 ** 10 + 1)).astype(float)
    from scikit_tt_gb300.tensor_train import _hosvd
    op = _hosvd(mat.reshape([2] * 20), 0, np.inf)
    sol = O.sle_mals(op, cores('x0'), cores('rhs'), repeats=1, solver=solver, threshold=1e-14, max_rank=10)
    exact = np.linalg.solve(mat, np.ones(1024))
    got = O.full_vector(sol)
    assert np.linalg.norm(got - exact) / np.linalg.norm(exact) < 1e-7
    assert max(c.shape[3] for c in sol) <= 10


def test_oracle_evp_deflation_matches_reference(golden):
    """evp.als with a previous eigentensor and a shift (evp.py:376-381): the
    second-lowest eigenpair of the Ising d=8 chain, as the reference finds it."""
    z, cores = golden('evp_ising_d8_deflation')
    val, vec, its = O.evp_als(cores('op'), cores('x0'), previous=[cores('prev')], shift=100.0, repeats=8,
                              sigma=float(z['sigma']))
    assert abs(val - float(z['val'])) < 1e-10
    assert its == int(z['its'])
    v, r = O.full_vector(vec), z['vec']
    assert min(np.linalg.norm(v - r), np.linalg.norm(v + r)) / np.linalg.norm(r) < 1e-7
    assert abs(float(z['val']) - np.linalg.eigvalsh(O.full_matrix(cores('op')))[1]) < 1e-8


@pytest.mark.parametrize('prefix,step,steps,order,prev,normalize',
                         [('o2', 0.1, 4, 2, False, 1), ('o4', 0.1, 4, 3, False, 1), ('o2p', 0.05, 3, 2, True, 2)])
def test_oracle_hod_matches_reference(golden, prefix, step, steps, order, prev, normalize):
    """Higher-order differencing (ode.py:117-247), orders 2 and 4 (an odd order is
    raised by one), with and without a given previous value."""
    z, cores = golden('ode_hod')
    sol = O.hod(cores('op'), cores('x0'), step, steps, order=order,
                previous_value=cores('prev') if prev else None, normalize=normalize)
    assert len(sol) == int(z[prefix + '_n'])
    for k, s in enumerate(sol):
        r = z[f'{prefix}_{k}']
        assert np.linalg.norm(O.full_vector(s) - r) / np.linalg.norm(r) < 1e-12
