"""Device SLE ALS against the reference's own outputs and the oracle.

Tolerances (relative, gauge-invariant full-tensor differences computed stably):
plain FP64 <= 1e-10, mixed (FP32 Krylov + FP64 refinement) <= 1e-8.
"""

import numpy as np
import pytest
import scipy.linalg as sla

from oracle import tt_oracle as O

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-10
TOL_MIXED = 1e-8


def _tt(cores):
    from scikit_tt_gb300.tensor_train import TT
    return TT([np.array(c) for c in cores])


def _solve(z, cores, precision='fp64', solver=None):
    from scikit_tt_gb300.solvers import sle
    sol, st = sle.als_ex(_tt(cores('op')), _tt(cores('x0')), _tt(cores('rhs')), repeats=int(z['repeats']),
                         solver=solver or str(z['solver']), precision=precision)
    return sol, st


@pytest.mark.parametrize('name', ['sle_laplace_d10', 'sle_laplace_d10_lu', 'sle_laplace_d10_r8', 'sle_coupled_d8'])
def test_sle_fp64_matches_reference(golden, name):
    z, cores = golden(name)
    sol, st = _solve(z, cores)
    ref = cores('sol')
    assert sol.ranks == [c.shape[0] for c in ref] + [1]
    assert O.stable_rel_diff(sol.cores, ref) < TOL_FP64
    assert st['max_local_residual'] <= 1e-13


@pytest.mark.parametrize('name', ['sle_laplace_d10', 'sle_laplace_d10_r8', 'sle_coupled_d8'])
def test_sle_mixed_matches_reference(golden, name):
    z, cores = golden(name)
    sol, st = _solve(z, cores, precision='mixed')
    assert O.stable_rel_diff(sol.cores, cores('sol')) < TOL_MIXED
    assert st['max_local_residual'] <= 1e-10


def test_sle_toeplitz_known_answer(golden):
    # scikit_tt tests/test_sle.py:37-59 on the device
    from scikit_tt_gb300.tensor_train import TT
    z, cores = golden('sle_toeplitz')
    mat = sla.toeplitz(np.arange(1, 2 ** 10 + 1), np.arange(1, 2 ** 10 + 1)).astype(float)
    op = TT(mat.reshape([2] * 20))
    from scikit_tt_gb300.solvers import sle
    for solver in ('solve', 'lu'):
        sol = sle.als(op, _tt(cores('x0')), _tt(cores('rhs')), repeats=1, solver=solver)
        exact = np.linalg.solve(mat, np.ones(1024))
        got = sol.matricize()
        assert np.linalg.norm(got - exact) / np.linalg.norm(exact) < 1e-7
        ref = O.full_vector(cores('sol'))
        assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-6


def test_sle_workload1_full_size_vs_oracle():
    from scikit_tt_gb300 import workloads as wl
    from scikit_tt_gb300.solvers import sle
    w = wl.laplace_sle()
    sol = sle.als(_tt(w.op), _tt(w.x0), _tt(w.rhs), repeats=w.repeats)
    ref = O.sle_als(w.op, w.x0, w.rhs, repeats=w.repeats)
    assert O.stable_rel_diff(sol.cores, ref) < TOL_FP64
    # the rank-limited global residual the reference reaches (1.061e-2)
    res = O.stable_residual(w.op, sol.cores, w.rhs)
    assert abs(res - O.stable_residual(w.op, ref, w.rhs)) < 1e-9


def test_sle_single_core_and_rank_one():
    from scikit_tt_gb300.solvers import sle
    rng = np.random.default_rng(5)
    # order 1: the whole system is one local solve
    A = rng.standard_normal((1, 6, 6, 1)) + 6 * np.eye(6)[None, :, :, None]
    b = rng.standard_normal((1, 6, 1, 1))
    x0 = rng.standard_normal((1, 6, 1, 1))
    sol = sle.als(_tt([A]), _tt([x0]), _tt([b]), repeats=1)
    ref = O.sle_als([A], [x0], [b], repeats=1)
    np.testing.assert_allclose(sol.cores[0], ref[0], rtol=1e-12, atol=1e-13)
    # rank-one guess, uneven mode sizes
    d, dims = 4, [3, 2, 4, 2]
    op = [rng.standard_normal((1, n, n, 1)) + 4 * np.eye(n)[None, :, :, None] for n in dims]
    rhs = [rng.standard_normal((1, n, 1, 1)) for n in dims]
    x1 = [rng.standard_normal((1, n, 1, 1)) for n in dims]
    sol = sle.als(_tt(op), _tt(x1), _tt(rhs), repeats=2)
    ref = O.sle_als(op, x1, rhs, repeats=2)
    assert O.stable_rel_diff(sol.cores, ref) < TOL_FP64


def test_sle_zero_rhs_and_errors():
    from scikit_tt_gb300 import workloads as wl
    from scikit_tt_gb300.solvers import sle
    w = wl.laplace_sle(d=5, n=3)
    zero = [np.zeros_like(c) for c in w.rhs]
    sol = sle.als(_tt(w.op), _tt(w.x0), _tt(zero), repeats=1)
    assert all(np.all(c == 0) for c in sol.cores[:1])
    with pytest.raises(ValueError):
        sle.als(_tt(w.op), _tt(w.x0), _tt(w.rhs), repeats=1, solver='bogus')
    bad = [c.copy() for c in w.rhs]
    bad[2] = np.ones((bad[2].shape[0], 3, 1, bad[2].shape[3] + 1))
    with pytest.raises(ValueError):
        sle.als(_tt(w.op), _tt(w.x0), _tt(w.rhs[:3] + [np.ones((3, 3, 1, 1))]), repeats=1)
    nan = [c.copy() for c in w.rhs]
    nan[1][0, 0, 0, 0] = np.nan
    from scikit_tt_gb300._lib import EngineError
    with pytest.raises(EngineError):
        sle.als(_tt(w.op), _tt(w.x0), _tt(nan), repeats=1)
    # the context stays usable after an error
    sol = sle.als(_tt(w.op), _tt(w.x0), _tt(w.rhs), repeats=1)
    assert O.stable_rel_diff(sol.cores, O.sle_als(w.op, w.x0, w.rhs, repeats=1)) < TOL_FP64


def test_sle_singular_operator_raises():
    from scikit_tt_gb300.solvers import sle
    rng = np.random.default_rng(9)
    op = [np.zeros((1, 3, 3, 1)) for _ in range(3)]
    rhs = [rng.standard_normal((1, 3, 1, 1)) for _ in range(3)]
    x0 = [rng.standard_normal((1, 3, 1, 1)) for _ in range(3)]
    with pytest.raises(np.linalg.LinAlgError):
        sle.als(_tt(op), _tt(x0), _tt(rhs), repeats=1)


@pytest.mark.parametrize('name', ['sle_mals_laplace_d6', 'sle_mals_laplace_d6_r4', 'sle_mals_coupled_d5_lu'])
def test_mals_matches_reference(golden, name):
    # two-site MALS: merged-site matrix-free solve + one-sided Jacobi SVD split
    from scikit_tt_gb300.solvers import sle
    z, cores = golden(name)
    mr = int(z['max_rank'])
    sol = sle.mals(_tt(cores('op')), _tt(cores('x0')), _tt(cores('rhs')), repeats=int(z['repeats']),
                   solver=str(z['solver']), threshold=float(z['threshold']), max_rank=np.inf if mr < 0 else mr)
    ref = z['full']
    v = O.full_vector(sol.cores)
    assert np.linalg.norm(v - ref) / np.linalg.norm(ref) < 1e-9
    if mr > 0:
        assert list(sol.ranks) == list(z['ranks'])
    else:
        assert max(abs(a - b) for a, b in zip(sol.ranks, z['ranks'])) <= 2


@pytest.mark.parametrize('precision,tol', [('fp64', TOL_FP64), ('mixed', TOL_MIXED)])
def test_sle_graph_replay_uses_new_inputs(precision, tol):
    """The single-solve sweep is captured in a CUDA graph on its first call and
    replayed by later calls with the same shapes: every call must solve its own
    inputs (three different seeds, identical shapes)."""
    from scikit_tt_gb300 import workloads as wl
    from scikit_tt_gb300.solvers import sle
    for seed in (11, 12, 13):
        w = wl.coupled_sle(d=7, n=4, rhs_rank=3, x_rank=6, repeats=2, seed=seed)
        sol, _ = sle.als_ex(_tt(w.op), _tt(w.x0), _tt(w.rhs), repeats=w.repeats, precision=precision)
        ref = O.sle_als(w.op, w.x0, w.rhs, repeats=w.repeats)
        assert O.stable_rel_diff(sol.cores, ref) < tol
