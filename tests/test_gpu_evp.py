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
