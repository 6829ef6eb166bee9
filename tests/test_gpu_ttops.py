"""Device TT operations and the ode.py helpers against reference outputs."""

import numpy as np
import pytest

from oracle import tt_oracle as O

pytestmark = pytest.mark.gpu


def test_tt_ops(golden):
    from scikit_tt_gb300.tensor_train import TT
    z, cores = golden('ttops')
    t, A = TT(cores('t')), TT(cores('A'))
    assert abs(t.norm() - float(z['norm'])) < 1e-12 * float(z['norm'])
    assert abs(A.norm() - float(z['opnorm'])) < 1e-12 * float(z['opnorm'])
    np.testing.assert_allclose(A.dot(t).full().reshape(-1), z['prod_full'], rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose((A @ t).matricize(), z['prod_full'], rtol=1e-12, atol=1e-12)
    tl = TT(cores('t')).ortho_left()
    np.testing.assert_allclose(tl.full().reshape(-1), z['left_full'], rtol=1e-12, atol=1e-12)
    for i in range(tl.order - 1):
        c = tl.cores[i].reshape(-1, tl.ranks[i + 1])
        np.testing.assert_allclose(c.T @ c, np.eye(tl.ranks[i + 1]), atol=1e-13)
    tr = TT(cores('t')).ortho_right()
    np.testing.assert_allclose(tr.full().reshape(-1), z['right_full'], rtol=1e-12, atol=1e-12)
    for i in range(1, tr.order):
        c = tr.cores[i].reshape(tr.ranks[i], -1)
        np.testing.assert_allclose(c @ c.T, np.eye(tr.ranks[i]), atol=1e-13)


def test_norm_of_huge_train_is_finite():
    # a d=48 U[0,1) rank-16 train has norm ~1e60: the log-carried device norm stays accurate
    from scikit_tt_gb300 import workloads as wl
    from scikit_tt_gb300.tensor_train import TT
    w = wl.ising_evp(d=48, x_rank=16)
    n_dev = TT([c.copy() for c in w.x0]).norm()
    n_ref = O.stable_norm(w.x0)
    assert np.isfinite(n_dev) and abs(n_dev / n_ref - 1) < 1e-10


def test_ode_helpers(golden):
    from scikit_tt_gb300.solvers import sle
    from scikit_tt_gb300.tensor_train import TT
    z, _ = golden('helpers')
    op, sol = TT([z['A0'], z['A1']]), TT([z['x0c'], z['x1c']])
    sl, sr = [z['Lp'], None], [None, z['Rn']]
    getattr(sle, '__construct_stack_left_op')(1, sl, op, sol)
    getattr(sle, '__construct_stack_right_op')(0, sr, op, sol)
    M = getattr(sle, '__construct_micro_matrix_als')(0, [z['Ls']], [z['Rs']], op, sol)
    np.testing.assert_allclose(sl[1], z['left'], rtol=1e-12, atol=1e-12 * np.abs(z['left']).max())
    np.testing.assert_allclose(sr[0], z['right'], rtol=1e-12, atol=1e-12 * np.abs(z['right']).max())
    np.testing.assert_allclose(M, z['micro'], rtol=1e-12, atol=1e-12 * np.abs(z['micro']).max())


@pytest.mark.parametrize('key', ['left_thr', 'right_max', 'ortho_both'])
def test_truncated_ortho_matches_reference(golden, key):
    # device one-sided Jacobi SVD per core with the reference's rank rule
    from scikit_tt_gb300.tensor_train import TT
    z, cores = golden('ttops_trunc')
    t = TT([np.array(c) for c in cores('t')])
    fn = {'left_thr': lambda x: x.ortho_left(threshold=1e-6),
          'right_max': lambda x: x.ortho_right(max_rank=3),
          'ortho_both': lambda x: x.ortho(threshold=1e-12, max_rank=4)}[key]
    r = fn(t)
    assert list(r.ranks) == list(z[key + '_ranks'])
    v, ref = O.full_vector(r.cores), z[key + '_full']
    assert np.linalg.norm(v - ref) / np.linalg.norm(ref) < 1e-12
    # the swept cores are orthonormal
    if key == 'left_thr':
        for c in r.cores[:-1]:
            m = c.reshape(-1, c.shape[3])
            assert np.allclose(m.T @ m, np.eye(m.shape[1]), atol=1e-12)
