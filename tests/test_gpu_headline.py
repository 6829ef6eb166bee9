"""Parity on the full-size workloads the throughput numbers are quoted on.

* The coupled-Laplacian SLE (d=32, n=8, operator rank 4, RHS rank 8, guess
  rank 32, 4 sweeps, seed 0): the reference's own sle.als solution
  (``sle_coupled_d32_headline.npz``, made by tests/golden/make_golden.py) against
  the single-solve drop-in (plain FP64 and mixed) and the batched engine that
  the benchmark times (plain FP64 and mixed, this instance in a batch with
  others).
* The 16 smallest-seed instances of the uneven batch (d 8..32, n in {2,4,8},
  ranks 4..48): the reference's solutions (``sle_batch_subset.npz``) against
  the batched engine in both precisions.

Gates (relative, gauge-invariant full-tensor differences computed stably):
plain FP64 <= 1e-10, mixed <= 1e-8; the stable global residual
||A x - b|| / ||b|| of the device solution equals the reference's to
1e-3 of its value plus the parity tolerance (the reference reaches 7.0e-6
on the headline: ALS at fixed rank 32 is rank-limited; instances that
converge reach the rounding floor, where only the tolerance is meaningful).
"""

import numpy as np
import pytest

from oracle import tt_oracle as O

TOL_FP64 = 1e-10
TOL_MIXED = 1e-8
RES_RTOL = 1e-3


def _tt(cores):
    from scikit_tt_gb300.tensor_train import TT
    return TT([np.array(c) for c in cores])


def _fingerprint(cores):
    return np.array([sum(float(c.sum()) for c in cores), sum(float((c * c).sum()) for c in cores)])


def _headline():
    from scikit_tt_gb300 import workloads as wl
    return wl.coupled_sle(seed=0, d=32, n=8, rhs_rank=8, x_rank=32, repeats=4)


def test_headline_fixture_matches_seeded_inputs(golden):
    """The seeded generator still yields the inputs the reference solved (CPU)."""
    z, _ = golden('sle_coupled_d32_headline')
    w = _headline()
    for key, cores in (('fp_op', w.op), ('fp_rhs', w.rhs), ('fp_x0', w.x0)):
        np.testing.assert_allclose(_fingerprint(cores), z[key], rtol=1e-13)


def test_batch_subset_fixture_matches_seeded_inputs(golden):
    from scikit_tt_gb300 import workloads as wl
    z, _ = golden('sle_batch_subset')
    for j in z['seeds']:
        w = wl.batch_instance(int(j))
        np.testing.assert_allclose(_fingerprint(w.rhs), z[f'j{j}_fp_rhs'], rtol=1e-13)
        np.testing.assert_allclose(_fingerprint(w.x0), z[f'j{j}_fp_x0'], rtol=1e-13)


def test_headline_reference_residual_by_oracle(golden):
    """The stored global residual is the oracle's stable residual of the stored
    solution (CPU; the GPU tests compare against this number)."""
    z, cores = golden('sle_coupled_d32_headline')
    w = _headline()
    res = O.stable_residual(w.op, cores('sol'), w.rhs)
    assert abs(res - float(z['global_rel_residual'])) <= 1e-12 * max(res, 1e-300) + 1e-15


def _check(sol_cores, ref_cores, w, z_res, tol):
    diff = O.stable_rel_diff(sol_cores, ref_cores)
    res = O.stable_residual(w.op, sol_cores, w.rhs)
    assert diff < tol, f'parity {diff:.3e} above {tol:.0e}'
    # a residual at the rounding floor (converged instances) agrees only to the parity tolerance
    assert abs(res - z_res) <= RES_RTOL * z_res + tol, f'global residual {res:.6e} vs reference {z_res:.6e}'
    return diff, res


@pytest.mark.gpu
@pytest.mark.parametrize('precision,tol', [('fp64', TOL_FP64), ('mixed', TOL_MIXED)])
def test_headline_dropin_matches_reference(golden, precision, tol):
    from scikit_tt_gb300.solvers import sle
    z, cores = golden('sle_coupled_d32_headline')
    w = _headline()
    sol, st = sle.als_ex(_tt(w.op), _tt(w.x0), _tt(w.rhs), repeats=w.repeats, precision=precision)
    ref = cores('sol')
    assert sol.ranks == [c.shape[0] for c in ref] + [1]
    _check(sol.cores, ref, w, float(z['global_rel_residual']), tol)


@pytest.mark.gpu
@pytest.mark.parametrize('precision,tol,local', [('fp64', TOL_FP64, 0.0), ('mixed', TOL_MIXED, 1e-10)])
def test_headline_batch_matches_reference(golden, precision, tol, local):
    """The batched engine the benchmark times: the headline instance together
    with three other seeds of the same workload in one launch."""
    from scikit_tt_gb300 import workloads as wl
    from scikit_tt_gb300.solvers import sle
    z, cores = golden('sle_coupled_d32_headline')
    ws = [_headline()] + [wl.coupled_sle(seed=s, d=32, n=8, rhs_rank=8, x_rank=32, repeats=4) for s in (1, 2, 3)]
    probs = [(_tt(w.op), _tt(w.x0), _tt(w.rhs)) for w in ws]
    sols, st = sle.als_batch(probs, repeats=4, precision=precision, tol=local)
    _check(sols[0].cores, cores('sol'), ws[0], float(z['global_rel_residual']), tol)
    if precision == 'mixed':
        assert st['max_local_residual'] <= 1e-8


@pytest.mark.gpu
@pytest.mark.parametrize('precision,tol,local', [('fp64', TOL_FP64, 0.0), ('mixed', TOL_MIXED, 1e-11)])
def test_uneven_batch_subset_matches_reference(golden, precision, tol, local):
    """Mixed precision solves each local system to 1e-11 here: instance 13
    (d=11, n=8, rank 25) lands 2.6e-8 from the reference at 1e-10 and 6.4e-9
    at 1e-11 (its local systems are the worst conditioned of the subset)."""
    from scikit_tt_gb300 import workloads as wl
    from scikit_tt_gb300.solvers import sle
    z, cores = golden('sle_batch_subset')
    seeds = [int(j) for j in z['seeds']]
    ws = [wl.batch_instance(j) for j in seeds]
    probs = [(_tt(w.op), _tt(w.x0), _tt(w.rhs)) for w in ws]
    sols, st = sle.als_batch(probs, repeats=4, precision=precision, tol=local)
    for j, w, sol in zip(seeds, ws, sols):
        ref = cores(f'j{j}_sol')
        diff = O.stable_rel_diff(sol.cores, ref)
        assert diff < tol, f'instance {j} {w.meta}: parity {diff:.3e}'
        res, z_res = O.stable_residual(w.op, sol.cores, w.rhs), float(z[f'j{j}_global_rel_residual'])
        assert abs(res - z_res) <= RES_RTOL * z_res + tol, f'instance {j}: residual {res:.4e} vs {z_res:.4e}'
