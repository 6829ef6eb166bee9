"""Seeded workload builders: operators equal their dense definitions."""

import numpy as np

from oracle import tt_oracle as O
from scikit_tt_gb300 import workloads as wl


def _kron_sum(d, n, mats_at):
    out = np.zeros((n ** d, n ** d))
    for i, m in mats_at:
        ops = [np.eye(n)] * d
        ops = list(ops)
        for site, mat in m:
            ops[site] = mat
        term = ops[0]
        for o in ops[1:]:
            term = np.kron(term, o)
        out += i * term
    return out


def test_laplace_op_dense():
    d, n = 4, 3
    L = wl.laplacian(n)
    terms = [(1.0, [(i, L)]) for i in range(d)] + [(1.0, [])]
    np.testing.assert_allclose(O.full_matrix(wl.laplace_op(d, n)), _kron_sum(d, n, terms), atol=1e-10)


def test_coupled_op_dense():
    d, n = 5, 3
    c = np.random.default_rng(3).uniform(0, 0.5, d)
    L, D = wl.laplacian(n), np.diag(np.linspace(-1, 1, n))
    terms = [(1.0, [(i, L)]) for i in range(d)] + [(1.0, [])] + [(c[i], [(i, D), (i + 1, D)]) for i in range(d - 1)]
    A = O.full_matrix(wl.coupled_op(d, n, c))
    np.testing.assert_allclose(A, _kron_sum(d, n, terms), atol=1e-10)
    np.testing.assert_allclose(A, A.T, atol=1e-12)


def test_ising_matches_reference_builder():
    # models.ising cores (scikit_tt/models.py:10-44) against a dense Hamiltonian
    d = 5
    H = O.full_matrix(wl.ising_op(d, 1.0, 0.7))
    X = np.array([[0.0, 1.0], [1.0, 0.0]])
    Z = np.diag([1.0, -1.0])
    terms = [(-1.0, [(i, Z), (i + 1, Z)]) for i in range(d - 1)] + [(-0.7, [(i, X)]) for i in range(d)]
    np.testing.assert_allclose(H, _kron_sum(d, 2, terms), atol=1e-12)


def test_workload_shapes():
    w = wl.coupled_sle()
    assert len(w.op) == 32 and w.op[1].shape == (4, 8, 8, 4)
    assert w.rhs[1].shape == (8, 8, 1, 8) and w.x0[1].shape == (32, 8, 1, 32)
    b = wl.batch_instance(3)
    assert 8 <= b.meta['d'] <= 32 and b.meta['n'] in (2, 4, 8) and 4 <= b.meta['r'] <= 48
    e = wl.ising_evp(d=12, x_rank=8)
    assert e.x0[3].shape == (8, 2, 1, 8) and np.all(e.x0[3] >= 0)
