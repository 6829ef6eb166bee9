"""Device EVP ALS against the reference's outputs and the free-fermion energy."""

import numpy as np
import pytest

from oracle import tt_oracle as O

pytestmark = pytest.mark.gpu


def _tt(cores):
    from scikit_tt_gb300.tensor_train import TT
    return TT([np.array(c) for c in cores])


@pytest.mark.parametrize('name', ['evp_ising_d12_eig', 'evp_ising_d12_eigh', 'evp_ising_d16_eig', 'evp_ising_d16_eigh'])
def test_evp_matches_reference(golden, name):
    from scikit_tt_gb300.solvers import evp
    z, cores = golden(name)
    val, vec, its = evp.als(_tt(cores('op')), _tt(cores('x0')), repeats=int(z['repeats']), solver=str(z['solver']),
                            sigma=float(z['sigma']), conv_eps=float(z['conv_eps']))
    assert abs(val - float(z['val'])) < 1e-10
    d = len(cores('op'))
    e0 = O.ising_exact_e0(d, 1.0, 1.0)
    assert abs(abs(val) - abs(e0)) < 1e-10
    v, r = O.full_vector(vec.cores), O.full_vector(cores('vec'))
    assert min(np.linalg.norm(v - r), np.linalg.norm(v + r)) / np.linalg.norm(r) < 1e-7


def test_evp_raw_guess_converges_to_ground_state():
    # unnormalised U[0,1) guess, as in the 48-site workload (reduced size)
    from scikit_tt_gb300 import workloads as wl
    from scikit_tt_gb300.solvers import evp
    w = wl.ising_evp(d=20, x_rank=24, repeats=6)
    val, vec, its = evp.als(_tt(w.op), _tt(w.x0), repeats=w.repeats, sigma=w.sigma)
    assert abs(val - O.ising_exact_e0(20, 1.0, 1.0)) < 1e-10


def test_evp_deflation_second_eigenvalue():
    from scikit_tt_gb300 import workloads as wl
    from scikit_tt_gb300.solvers import evp
    d = 8
    w = wl.ising_evp(d=d, x_rank=16, repeats=8)
    x0 = O.ortho_right(w.x0)
    v0, t0, _ = evp.als(_tt(w.op), _tt(x0), repeats=8, sigma=w.sigma)
    ref_vals = np.linalg.eigvalsh(O.full_matrix(w.op))
    assert abs(v0 - ref_vals[0]) < 1e-10
    nrm = O.stable_norm(t0.cores)
    t0n = [t0.cores[0] / nrm] + t0.cores[1:]
    v1, _, _ = evp.als(_tt(w.op), _tt(x0), previous=[_tt(t0n)], shift=100.0, repeats=8, sigma=w.sigma)
    oracle = O.evp_als(w.op, x0, previous=[t0n], shift=100.0, repeats=8, sigma=w.sigma)
    assert abs(v1 - oracle[0]) < 1e-9
    assert abs(v1 - ref_vals[1]) < 1e-8


def _same_up_to_sign(v, r):
    return min(np.linalg.norm(v - r), np.linalg.norm(v + r)) / np.linalg.norm(r)


@pytest.mark.parametrize('solver,k', [('eig', 1), ('eigs', 1), ('eig', 3), ('eigs', 3)])
def test_evp_nonsymmetric_matches_oracle(solver, k):
    # column-stochastic transfer operator with nonsymmetric cores: Arnoldi path
    from scikit_tt_gb300 import workloads as wl
    from scikit_tt_gb300.solvers import evp
    w = wl.markov_evp()
    x0 = O.ortho_right(w.x0)
    ref_vals, ref_vecs, ref_its = O.evp_als(w.op, x0, number_ev=k, repeats=4, solver=solver, sigma=1.0,
                                            conv_eps=0.0)
    vals, vecs, its = evp.als(_tt(w.op), _tt(x0), number_ev=k, repeats=4, solver=solver, sigma=1.0, conv_eps=0.0)
    assert its == ref_its
    if k == 1:
        assert abs(vals - np.real(ref_vals)) < 1e-9
        assert _same_up_to_sign(O.full_vector(vecs.cores), np.real(O.full_vector(ref_vecs))) < 1e-6
    else:
        assert np.max(np.abs(np.asarray(vals) - np.real(ref_vals))) < 1e-9
        for e in range(k):
            assert _same_up_to_sign(O.full_vector(vecs[e].cores), np.real(O.full_vector(ref_vecs[e]))) < 1e-6


@pytest.mark.parametrize('solver', ['eigh', 'eig'])
def test_evp_symmetric_block_of_three(solver):
    # number_ev = 3 on the Ising chain: Lanczos with three Ritz pairs and the
    # rank-r re-gauging of the eigenvector block
    from scikit_tt_gb300 import workloads as wl
    from scikit_tt_gb300.solvers import evp
    w = wl.ising_evp(d=8, x_rank=8, repeats=4)
    x0 = O.ortho_right(w.x0)
    sigma = w.sigma if solver == 'eig' else 1.0
    ref_vals, ref_vecs, ref_its = O.evp_als(w.op, x0, number_ev=3, repeats=4, solver=solver, sigma=sigma,
                                            conv_eps=0.0)
    vals, vecs, its = evp.als(_tt(w.op), _tt(x0), number_ev=3, repeats=4, solver=solver, sigma=sigma, conv_eps=0.0)
    assert np.max(np.abs(np.asarray(vals) - np.real(ref_vals))) < 1e-9
    for e in range(3):
        assert _same_up_to_sign(O.full_vector(vecs[e].cores), np.real(O.full_vector(ref_vecs[e]))) < 1e-6


def test_evp_complex_wanted_eigenvalue_is_refused():
    # a plane rotation has eigenvalues exp(+-i t): the pair closest to sigma = 1
    # is complex, which real cores cannot hold
    from scikit_tt_gb300.solvers import evp
    t = 0.3
    rot = np.array([[np.cos(t), -np.sin(t)], [np.sin(t), np.cos(t)]])
    op = [rot.reshape(1, 2, 2, 1), np.eye(2).reshape(1, 2, 2, 1)]
    x0 = [np.ones((1, 2, 1, 2)), np.ones((2, 2, 1, 1))]
    with pytest.raises(NotImplementedError):
        evp.als(_tt(op), _tt(x0), repeats=1, solver='eig', sigma=1.0)


@pytest.mark.parametrize('name', ['evp_markov_eig_k1', 'evp_markov_eig_k3', 'evp_markov_eigs_k3',
                                  'evp_ising_d8_eigh_k3', 'evp_ising_d8_eig_k3'])
def test_evp_blocks_match_reference(golden, name):
    # device Arnoldi / block path against the reference's own outputs
    from scikit_tt_gb300.solvers import evp
    z, cores = golden(name)
    k = int(z['number_ev'])
    vals, vecs, its = evp.als(_tt(cores('op')), _tt(cores('x0')), number_ev=k, repeats=int(z['repeats']),
                              solver=str(z['solver']), sigma=float(z['sigma']), conv_eps=float(z['conv_eps']))
    assert its == int(z['its'])
    assert np.max(np.abs(np.atleast_1d(vals) - z['vals'])) < 1e-9
    vecs = [vecs] if k == 1 else vecs
    for e in range(k):
        assert _same_up_to_sign(O.full_vector(vecs[e].cores), z[f'vec{e}']) < 1e-6


@pytest.mark.parametrize('name', ['evp_power_markov', 'evp_power_markov_gevp'])
def test_power_method_matches_reference(golden, name):
    # inverse power iteration through the device sle.als, TT.norm and TT.dot
    from scikit_tt_gb300 import tensor_train as tt
    from scikit_tt_gb300.solvers import evp
    z, cores = golden(name)
    op = _tt(cores('op'))
    gevp = tt.eye(op.row_dims) if bool(z['gevp']) else None
    val, vec = evp.power_method(op, _tt(cores('x0')), operator_gevp=gevp, repeats=int(z['repeats']),
                                sigma=float(z['sigma']))
    assert abs(val - float(z['val'])) < 1e-10
    assert _same_up_to_sign(O.full_vector(vec.cores), z['vec0']) < 1e-7


def _vec_err(u, v):
    """Distance of two eigenvectors up to sign; the reference's vectors of
    nonsymmetric problems carry an arbitrary global complex phase, removed here."""
    u, v = np.asarray(u).ravel(), np.asarray(v).ravel()
    if np.iscomplexobj(v):
        k = np.argmax(np.abs(v))
        v = (v * np.conj(v[k]) / np.abs(v[k])).real
    return min(np.linalg.norm(u - v), np.linalg.norm(u + v)) / np.linalg.norm(v)


@pytest.mark.parametrize('solver', ['eig', 'eigs', 'eigh'])
def test_triple_well_known_answer(golden, solver):
    """The reference's own eigenproblem test (tests/test_evp.py:16-150) on the
    device: the Ulam transfer operator of the triple-well data, rank-15 ones
    guess, number_ev=3, 10 sweeps.  Its assertions (eigenvalues within 5e-3 and
    eigenvectors within 5e-2 of the dense eigs answer), and agreement with the
    reference's own evp.als result to 1e-8 (eigenvalues) / 1e-6 (vectors)."""
    from scikit_tt_gb300.solvers import evp
    z, cores = golden('evp_triple_well')
    op = _tt(cores('sym') if solver == 'eigh' else cores('op'))
    vals, vecs, _ = evp.als(op, _tt(cores('x0')), number_ev=3, repeats=10, solver=solver)
    mv = z['sym_vals'] if solver == 'eigh' else z['mat_vals']
    mx = z['sym_vecs'] if solver == 'eigh' else z['mat_vecs']
    idx = np.argsort(mv) if solver == 'eigs' else np.argsort(mv)[::-1]
    mv, mx = mv[idx], mx[:, idx]
    for i in range(3):
        assert abs(mv[i] - vals[i]) / mv[i] < 5e-3
        assert _vec_err(vecs[i].matricize(), mx[:, i]) < 5e-2
        assert abs(vals[i] - z[f'{solver}_vals'][i]) <= 1e-8 * abs(z[f'{solver}_vals'][i])
        assert _vec_err(vecs[i].matricize(), z[f'{solver}_vecs'][i]) < 1e-6


def test_triple_well_identity_gevp_and_power_method(golden):
    """The same test's number_ev=1 solve with the identity operator_gevp and the
    inverse power method, against the reference's results and the dense answer."""
    from scikit_tt_gb300.solvers import evp
    from scikit_tt_gb300 import tensor_train as tt
    z, cores = golden('evp_triple_well')
    op = _tt(cores('op'))
    val, vec, _ = evp.als(op, _tt(cores('x0')), operator_gevp=tt.eye(op.row_dims), repeats=10)
    assert abs(val - float(z['gevp_val'])) <= 1e-8 * abs(float(z['gevp_val']))
    assert _vec_err(vec.matricize(), z['gevp_vec']) < 1e-6
    pv, pvec = evp.power_method(_tt(cores('op')), _tt(cores('x0')))
    top = z['mat_vals'][np.argmax(z['mat_vals'])]
    assert abs(pv - top) / abs(top) < 5e-3
    assert abs(pv - float(z['power_val'])) <= 1e-8 * abs(float(z['power_val']))
    assert _vec_err(pvec.matricize(), z['power_vec']) < 1e-6


@pytest.mark.parametrize('name', ['evp_gevp_ising_d6_eig', 'evp_gevp_ising_d6_eigh'])
def test_gevp_matches_reference(golden, name):
    """Generalised problem A x = lambda B x with an SPD mass operator (evp.py:272-287,
    314-329, 367-368 and the b= local solves of evp.py:423-439): the reference's
    eigenvalue to 1e-9 and eigentensor to 1e-6 up to sign (unit 2-norm for 'eig',
    unit B-norm for 'eigh', as the reference's local solvers return them)."""
    from scikit_tt_gb300.solvers import evp
    z, cores = golden(name)
    val, vec, its = evp.als(_tt(cores('op')), _tt(cores('x0')), operator_gevp=_tt(cores('gevp')),
                            repeats=int(z['repeats']), solver=str(z['solver']), sigma=float(z['sigma']),
                            conv_eps=float(z['conv_eps']))
    ref = float(z['val'])
    assert abs(val - ref) <= 1e-9 * max(1.0, abs(ref))
    assert its == int(z['its'])
    assert _vec_err(vec.matricize(), _tt(cores('vec')).matricize()) < 1e-6
    assert evp.last_stats['local_solves'] > 0


@pytest.mark.parametrize('precision', ['fp64', 'mixed'])
def test_gevp_in_a_mixed_batch(golden, precision):
    """A generalised request beside a linear system and a standard eigenproblem in one
    launch: each matches its own reference result."""
    from scikit_tt_gb300 import workloads as wl
    from scikit_tt_gb300.serving import Request, solve_batch
    zg, cg = golden('evp_gevp_ising_d6_eig')
    w = wl.laplace_sle(d=6, n=2, rhs_rank=2, x_rank=3, repeats=2, seed=4)
    we = wl.ising_evp(d=6, g=0.8, x_rank=3, repeats=3, seed=2)
    reqs = [Request('gevp', cg('op'), cg('x0'), cg('gevp'), repeats=int(zg['repeats']), solver='eig',
                    sigma=float(zg['sigma']), conv_eps=float(zg['conv_eps'])),
            Request('sle', w.op, w.x0, w.rhs, repeats=w.repeats),
            Request('evp', we.op, we.x0, repeats=we.repeats, sigma=we.sigma)]
    solve_batch(reqs, precision=precision)
    assert abs(reqs[0].value - float(zg['val'])) <= 1e-9 * max(1.0, abs(float(zg['val'])))
    assert _vec_err(reqs[0].solution.matricize(), _tt(cg('vec')).matricize()) < 1e-6
    tol = 1e-10 if precision == 'fp64' else 1e-8
    assert O.stable_rel_diff(reqs[1].solution.cores, O.sle_als(w.op, w.x0, w.rhs, repeats=w.repeats)) < tol
    ref_val, _, _ = O.evp_als(we.op, O.ortho_right(we.x0), repeats=we.repeats, sigma=we.sigma)
    assert abs(reqs[2].value - ref_val) < 1e-9
