"""Alternating linear scheme for ``A x = b`` in the TT format, on the GPU.

Drop-in for ``scikit_tt/solvers/sle.py``: ``als`` keeps its signature
(sle.py:10) and returns a host ``TT``.  The whole sweep -- interface stacks,
local right-hand sides, matrix-free local solves, QR/RQ re-gauging -- runs in
``libttals.so``; see ``ttals_sle_als`` in ``include/ttals.h``.

Precision is chosen outside the reference signature (module attribute
``PRECISION`` or the ``als_ex`` entry point): ``'fp64'`` (default, parity with
the reference to round-off) or ``'mixed'`` (FP32 Krylov inner solves with
FP64 residual refinement).

The private helpers that ``scikit_tt/solvers/ode.py:13`` imports by name are
provided with the same names and in-place semantics (real data).
"""

from __future__ import annotations

from typing import List

import numpy as np

from .. import _lib
from ..tensor_train import TT

PRECISION = 'fp64'
_PREC = {'fp64': _lib.PREC_FP64, 'mixed': _lib.PREC_MIXED}

last_stats = {}


def als_ex(operator: TT, initial_guess: TT, right_hand_side: TT, repeats: int = 1, solver: str = 'solve',
           precision: str = None, tol: float = 0.0):
    """``als`` plus engine options; returns ``(solution, stats)``.

    ``tol`` is the relative residual every local system is solved to (0 picks
    1e-13 for fp64 and 1e-10 for mixed)."""
    if solver not in _lib.SLE_SOLVERS:
        # the reference silently skips the local solve for unknown strings
        # (sle.py:505-509); the device path refuses instead
        raise ValueError("solver must be 'solve' or 'lu'")
    precision = precision or PRECISION
    if precision not in _PREC:
        raise ValueError("precision must be 'fp64' or 'mixed'")
    op, x0, b = _lib.Packed(operator.cores), _lib.Packed(initial_guess.cores), _lib.Packed(right_hand_side.cores)
    lib = _lib.load()
    dims = np.array(operator.row_dims, dtype=np.int64)
    ranks = np.zeros(operator.order + 1, dtype=np.int64)
    if repeats > 0:
        _lib.check(lib.ttals_als_ranks(operator.order, _lib.i64ptr(dims), _lib.i64ptr(x0.ranks),
                                       _lib.i64ptr(ranks)))
    else:
        ranks[:] = x0.ranks
    total = int(sum(ranks[i] * dims[i] * ranks[i + 1] for i in range(operator.order)))
    out = np.empty(max(total, 1), dtype=np.float64)
    out_ranks = np.zeros(operator.order + 1, dtype=np.int64)
    st = _lib.Stats()
    _lib.check(lib.ttals_sle_als(_lib.context(), op.desc, x0.desc, b.desc, int(repeats), _lib.SLE_SOLVERS[solver],
                                 _PREC[precision], float(tol), _lib.dptr(out), 0, _lib.i64ptr(out_ranks), st))
    if repeats == 0:
        # the reference returns the untouched copy of the initial guess
        return initial_guess.copy(), st.as_dict()
    cores = _lib.unpack(out, operator.row_dims, [1] * operator.order, out_ranks)
    return TT(cores), st.as_dict()


def als(operator: 'TT', initial_guess: 'TT', right_hand_side: 'TT', repeats: int = 1, solver: str = 'solve') -> 'TT':
    """Alternating linear scheme (Holtz, Rohwedder, Schneider 2012), signature of
    sle.py:10.  Returns the approximate solution of ``operator @ x =
    right_hand_side`` after ``repeats`` forward+backward sweeps."""
    global last_stats
    sol, last_stats = als_ex(operator, initial_guess, right_hand_side, repeats, solver)
    return sol


def mals(operator: 'TT', initial_guess: 'TT', right_hand_side: 'TT', repeats: int = 1, solver: str = 'solve',
         threshold: float = 1e-12, max_rank: int = np.inf) -> 'TT':
    """Modified ALS (two-site, rank-adaptive), signature of sle.py:98.

    Each pair of neighbouring cores is solved as one merged site by the device
    matrix-free GMRES, then split by a truncated SVD (singular values with
    sigma_k / sigma_0 <= ``threshold`` dropped, at most ``max_rank`` kept), in
    the reference's sweep order (sle.py:128-189).  Ranks above 1024 on a bond
    need a ``max_rank``."""
    global last_stats
    if solver not in _lib.SLE_SOLVERS:
        raise ValueError("solver must be 'solve' or 'lu'")
    if operator.order < 2:
        raise NotImplementedError('mals needs at least two cores')
    op, x0, b = _lib.Packed(operator.cores), _lib.Packed(initial_guess.cores), _lib.Packed(right_hand_side.cores)
    lib = _lib.load()
    mr = 0 if max_rank == np.inf else int(max_rank)
    cap = np.zeros(1, dtype=np.int64)
    _lib.check(lib.ttals_sle_mals(_lib.context(), op.desc, x0.desc, b.desc, int(repeats), _lib.SLE_SOLVERS[solver],
                                  float(threshold), mr, 0.0, None, 0, None, _lib.i64ptr(cap), None))
    out = np.empty(max(int(cap[0]), 1), dtype=np.float64)
    out_ranks = np.zeros(operator.order + 1, dtype=np.int64)
    st = _lib.Stats()
    _lib.check(lib.ttals_sle_mals(_lib.context(), op.desc, x0.desc, b.desc, int(repeats), _lib.SLE_SOLVERS[solver],
                                  float(threshold), mr, 0.0, _lib.dptr(out), 0, _lib.i64ptr(out_ranks), None, st))
    last_stats = st.as_dict()
    if repeats == 0:
        return initial_guess.copy()
    return TT(_lib.unpack(out, operator.row_dims, [1] * operator.order, out_ranks))


# ---------------------------------------------------------------------------
# private helpers imported by scikit_tt/solvers/ode.py:13 (device-backed)
# ---------------------------------------------------------------------------

def _stack(left, stack, x, op):
    r0, n, _, r1 = x.shape
    R0, R1 = op.shape[0], op.shape[3]
    stack = np.ascontiguousarray(stack, dtype=np.float64)
    xc = np.ascontiguousarray(x[:, :, 0, :], dtype=np.float64)
    oc = np.ascontiguousarray(op, dtype=np.float64)
    out = np.empty((r1, R1, r1) if left else (r0, R0, r0), dtype=np.float64)
    _lib.check(_lib.load().ttals_stack_op(_lib.context(), 1 if left else 0, _lib.dptr(stack), _lib.dptr(xc),
                                          _lib.dptr(oc), r0, n, r1, R0, R1, _lib.dptr(out), 0))
    return out


def __construct_stack_left_op(i: int, stack_left_op: List[np.ndarray], operator: 'TT', solution: 'TT'):
    """In-place left operator stack (sle.py:194-219) on the device."""
    if i == 0:
        stack_left_op[i] = np.array([1], ndmin=3)
    else:
        stack_left_op[i] = _stack(True, stack_left_op[i - 1], solution.cores[i - 1], operator.cores[i - 1])


def __construct_stack_right_op(i: int, stack_right_op: List[np.ndarray], operator: 'TT', solution: 'TT'):
    """In-place right operator stack (sle.py:250-276) on the device."""
    if i == operator.order - 1:
        stack_right_op[i] = np.array([1], ndmin=3)
    else:
        stack_right_op[i] = _stack(False, stack_right_op[i + 1], solution.cores[i + 1], operator.cores[i + 1])


def __construct_micro_matrix_als(i: int, stack_left_op: List[np.ndarray], stack_right_op: List[np.ndarray],
                                 operator: 'TT', solution: 'TT') -> np.ndarray:
    """Dense local operator (sle.py:308-347), assembled on the device."""
    r0, r1, n = solution.ranks[i], solution.ranks[i + 1], operator.row_dims[i]
    R0, R1 = operator.ranks[i], operator.ranks[i + 1]
    L = np.ascontiguousarray(stack_left_op[i], dtype=np.float64)
    A = np.ascontiguousarray(operator.cores[i], dtype=np.float64)
    Rt = np.ascontiguousarray(stack_right_op[i], dtype=np.float64)
    for arr in (L, A, Rt):
        if np.iscomplexobj(arr):
            raise NotImplementedError('complex operators are not supported by the device path')
    N = r0 * n * r1
    out = np.empty((N, N), dtype=np.float64)
    _lib.check(_lib.load().ttals_micro_matrix(_lib.context(), _lib.dptr(L), _lib.dptr(A), _lib.dptr(Rt), r0, n, r1,
                                              R0, R1, _lib.dptr(out), 0))
    return out


def __construct_micro_matrix_mals(i, stack_left_op, stack_right_op, operator, solution):
    """Dense two-site micro matrix (sle.py:350-390): the one-site assembly of the
    merged site (mode n_i n_{i+1}, operator core A_i x A_{i+1}) on the device."""
    A1, A2 = operator.cores[i], operator.cores[i + 1]
    n1, n2 = A1.shape[1], A2.shape[1]
    merged = np.einsum('abcd,defg->abecfg', A1, A2).reshape(A1.shape[0], n1 * n2, n1 * n2, A2.shape[3])
    r0, r1 = solution.ranks[i], solution.ranks[i + 2]
    L = np.ascontiguousarray(stack_left_op[i], dtype=np.float64)
    Rt = np.ascontiguousarray(stack_right_op[i + 1], dtype=np.float64)
    A = np.ascontiguousarray(merged, dtype=np.float64)
    N = r0 * n1 * n2 * r1
    out = np.empty((N, N), dtype=np.float64)
    _lib.check(_lib.load().ttals_micro_matrix(_lib.context(), _lib.dptr(L), _lib.dptr(A), _lib.dptr(Rt), r0, n1 * n2,
                                              r1, A.shape[0], A.shape[3], _lib.dptr(out), 0))
    return out


def als_batch(problems, repeats=1, precision: str = None, tol: float = 0.0):
    """Solve many independent systems in one launch (one CTA per system).

    ``problems``: sequence of ``(operator, initial_guess, right_hand_side)`` TT
    triples (shapes may differ); ``repeats``: int or per-problem list.  Returns
    ``(solutions, stats)``; each solution equals what ``als`` returns for that
    problem (to the local-solve tolerance)."""
    precision = precision or PRECISION
    if precision not in _PREC:
        raise ValueError("precision must be 'fp64' or 'mixed'")
    count = len(problems)
    if count == 0:
        return [], {}
    reps = list(repeats) if isinstance(repeats, (list, tuple)) else [int(repeats)] * count
    packs = [(_lib.Packed(a.cores), _lib.Packed(x.cores), _lib.Packed(b.cores)) for a, x, b in problems]
    lib = _lib.load()
    outs, ranks_all = [], []
    for (a, x, b), (pa, px, pb) in zip(problems, packs):
        dims = np.array(a.row_dims, dtype=np.int64)
        rk = np.zeros(a.order + 1, dtype=np.int64)
        _lib.check(lib.ttals_als_ranks(a.order, _lib.i64ptr(dims), _lib.i64ptr(px.ranks), _lib.i64ptr(rk)))
        total = int(sum(rk[i] * dims[i] * rk[i + 1] for i in range(a.order)))
        outs.append(np.empty(max(total, 1), dtype=np.float64))
        ranks_all.append(rk)
    ops = (_lib.TTDesc * count)(*[p[0].desc for p in packs])
    xs = (_lib.TTDesc * count)(*[p[1].desc for p in packs])
    bs = (_lib.TTDesc * count)(*[p[2].desc for p in packs])
    rep_arr = (_lib.C.c_int32 * count)(*reps)
    out_ptrs = (_lib.C.POINTER(_lib.C.c_double) * count)(*[_lib.dptr(o) for o in outs])
    st = _lib.Stats()
    _lib.check(lib.ttals_sle_als_batch(_lib.context(), count, ops, xs, bs, rep_arr, _PREC[precision], float(tol),
                                       out_ptrs, 0, st))
    sols = [TT(_lib.unpack(o, a.row_dims, [1] * a.order, rk)) for o, (a, _, _), rk in zip(outs, problems, ranks_all)]
    return sols, st.as_dict()
