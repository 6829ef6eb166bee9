"""Linear-ODE integrators in the TT format on the device engine.

Drop-ins for the step methods of ``scikit_tt/solvers/ode.py`` that are built on
the ALS hot path: every implicit step is one device ``sle.als`` call on the
shifted operator ``I - h A`` (or ``I - h/2 A``), warm-started from the previous
step's solution; products and norms run through the device ``TT.dot`` and
``TT.norm``.  Signatures, defaults and return values follow the reference:

* ``explicit_euler``      ode.py:16-83   (x_{k+1} = (I + h A) x_k, re-truncated)
* ``errors_expl_euler``   ode.py:85-115
* ``hod``                 ode.py:117-247 (higher-order differencing,
  x_{k+1} = x_{k-1} + 2 sinh(h A) x_k with a truncated series)
* ``implicit_euler``      ode.py:249-331 ((I - h A) x_{k+1} = x_k)
* ``errors_impl_euler``   ode.py:333-364
* ``trapezoidal_rule``    ode.py:366-451 ((I - h/2 A) x_{k+1} = (I + h/2 A) x_k)
* ``errors_trapezoidal``  ode.py:453-485
* ``adaptive_step_size``  ode.py:487-636 (implicit Euler against two half steps
  or the trapezoidal rule, step control by local error and closeness to the
  stationary state)

* ``tdvp1site``           ode.py:1188-1288 (one-site TDVP)
* ``tdvp2site``           ode.py:1290-1396 (two-site TDVP, truncated splits)
* ``tdvp``                ode.py:1076-1186 (adaptive one-/two-site TDVP)

``tt_solver='mals'`` runs the device two-site solver; ``progress`` is accepted
and ignored.  The TDVP functions run every local exponential on the device
(one persistent Krylov kernel per local step) and need a real exponent
``-1j * step_size``: imaginary-time steps (``step_size = -1j * dt``), the
setting of the reference's own TDVP test.  Real-time steps would need complex
cores, which the device path does not hold; they raise ``NotImplementedError``.
"""

from __future__ import annotations

import math
from typing import List

import numpy as np

from .. import _lib
from .. import tensor_train as tt
from . import sle


def _shifted(operator, alpha):
    """I + alpha * operator as a TT operator (rank sum, tensor_train.py:282-344)."""
    return tt.eye(operator.row_dims) + alpha * operator


def _solve(op, guess, rhs, tt_solver, micro_solver, repeats, threshold, max_rank):
    if tt_solver == 'als':
        return sle.als(op, guess, rhs, solver=micro_solver, repeats=repeats)
    if tt_solver == 'mals':
        return sle.mals(op, guess, rhs, solver=micro_solver, threshold=threshold, repeats=repeats, max_rank=max_rank)
    raise ValueError("tt_solver must be 'als' or 'mals'")


def explicit_euler(operator, initial_value, step_sizes: List[float], threshold: float = 1e-12,
                   max_rank: int = 50, normalize: int = 1, progress: bool = True) -> List:
    """x_{k+1} = (I + h_k A) x_k, re-truncated by ``ortho(threshold, max_rank)``."""
    solution = [initial_value]
    for h in step_sizes:
        nxt = _shifted(operator, h).dot(solution[-1])
        nxt = nxt.ortho(threshold=threshold, max_rank=max_rank)
        if normalize > 0:
            nxt = (1 / nxt.norm(p=normalize)) * nxt
        solution.append(nxt.copy())
    return solution


def errors_expl_euler(operator, solution: List, step_sizes: List[float]) -> List[float]:
    """Relative residuals |x_{k+1} - (I + h A) x_k| / |x_k|."""
    return [(solution[k + 1] - _shifted(operator, step_sizes[k]).dot(solution[k])).norm() / solution[k].norm()
            for k in range(len(solution) - 1)]


def _odd_series(operator, scale, step, order):
    """scale*step*A + sum_{k=2}^{order/2} 2/(2k-1)! * step^(2k-1) * A^(2k-1), the
    odd part of the exponential series the higher-order differencing scheme
    steps with (ode.py:186-191, 203-208)."""
    series = (scale * step) * operator.copy()
    power = operator.copy()
    for k in range(2, order // 2 + 1):
        power = power.dot(operator).dot(operator)
        series = series + (2 / math.factorial(2 * k - 1) * step ** (2 * k - 1)) * power
    return series


def hod(operator, initial_value, step_size: float, number_of_steps: int, order: int = 2, previous_value=None,
        op_hod=None, threshold: float = 1e-12, max_rank: int = 50, normalize: int = 1, progress: bool = True) -> List:
    """Higher-order differencing (ode.py:117-247): x_{k+1} = x_{k-1} + 2 sinh(h A) x_k
    with sinh truncated after the power A^(order-1) (odd ``order`` is raised by
    one), re-truncated by ``ortho(threshold, max_rank)`` after every step.
    Without ``previous_value`` the state half a step back comes from one
    explicit Euler half step and one backward application of the series at
    h/2.  Products, truncations and 2-norms run on the device."""
    if order % 2 != 0:
        order += 1
    if op_hod is None:
        op_hod = _odd_series(operator, 2.0, step_size, order).ortho(threshold=threshold)
    solution = [initial_value]
    for i in range(number_of_steps):
        if i == 0:
            if previous_value is None:
                # h*A + sum 2/(2k-1)! (h/2)^(2k-1) A^(2k-1); 2 * (h/2) == h exactly
                op_first = _odd_series(operator, 2.0, step_size / 2, order).ortho(threshold=threshold)
                back = _shifted(operator, -0.5 * step_size).dot(solution[0])
                prev = solution[0] - op_first.dot(back)
            else:
                prev = previous_value
            if normalize > 0:
                prev = (1 / prev.norm(p=normalize)) * prev
            prev = prev.ortho(threshold=threshold, max_rank=max_rank)
        else:
            prev = solution[i - 1].copy()
        nxt = (prev + op_hod.dot(solution[i])).ortho(threshold=threshold, max_rank=max_rank)
        if normalize > 0:
            nxt = (1 / nxt.norm(p=normalize)) * nxt
        solution.append(nxt.copy())
    return solution


def implicit_euler(operator, initial_value, initial_guess, step_sizes: List[float], repeats: int = 1,
                   tt_solver: str = 'als', threshold: float = 1e-12, max_rank=np.inf, micro_solver='solve',
                   normalize=1, progress=True) -> List:
    """(I - h_k A) x_{k+1} = x_k, each step one device ALS solve warm-started from the last."""
    solution = [initial_value]
    current = initial_guess
    for h in step_sizes:
        current = _solve(_shifted(operator, -h), current, solution[-1], tt_solver, micro_solver, repeats, threshold,
                         max_rank)
        if normalize > 0:
            current = (1 / current.norm(p=normalize)) * current
        solution.append(current.copy())
    return solution


def errors_impl_euler(operator, solution: List, step_sizes: List[float]) -> List[float]:
    """Relative residuals |(I - h A) x_{k+1} - x_k| / |x_k|."""
    return [(_shifted(operator, -step_sizes[k]).dot(solution[k + 1]) - solution[k]).norm() / solution[k].norm()
            for k in range(len(solution) - 1)]


def trapezoidal_rule(operator, initial_value, initial_guess, step_sizes: List[float], repeats: int = 1,
                     tt_solver: str = 'als', threshold=1e-12, max_rank: int = np.inf, micro_solver: str = 'solve',
                     normalize: int = 1, progress: bool = True) -> List:
    """(I - h/2 A) x_{k+1} = (I + h/2 A) x_k."""
    solution = [initial_value]
    current = initial_guess
    for h in step_sizes:
        rhs = _shifted(operator, 0.5 * h).dot(solution[-1])
        current = _solve(_shifted(operator, -0.5 * h), current, rhs, tt_solver, micro_solver, repeats, threshold,
                         max_rank)
        if normalize > 0:
            current = (1 / current.norm(p=normalize)) * current
        solution.append(current.copy())
    return solution


def errors_trapezoidal(operator, solution: List, step_sizes: List[float]) -> List[float]:
    """Relative residuals of the trapezoidal steps."""
    errs = []
    for k in range(len(solution) - 1):
        rhs = _shifted(operator, 0.5 * step_sizes[k]).dot(solution[k])
        errs.append((_shifted(operator, -0.5 * step_sizes[k]).dot(solution[k + 1]) - rhs).norm() / rhs.norm())
    return errs


def adaptive_step_size(operator, initial_value, initial_guess, time_end: float, step_size_first: float = 1e-10,
                       repeats: int = 1, solver: str = 'solve', error_tol: float = 1e-1, closeness_tol: float = 0.5,
                       step_size_min: float = 1e-14, step_size_max: float = 10, closeness_min: float = 1e-3,
                       factor_max: float = 2, factor_safe: float = 0.9, second_method: str = 'two_step_Euler',
                       normalize: int = 1, progress: bool = True):
    """Adaptive implicit Euler (ode.py:487-636); returns ``(solution, time_steps)``.

    A step of size h is implicit Euler (normalised in the 1-norm); its
    companion is two implicit Euler half steps or one trapezoidal step.  The
    step is accepted when both the relative local error and the relative
    change of |A x| (closeness to the stationary state) are within tolerance;
    the next step size is the safety-scaled minimum of the three factors."""
    solution = [initial_value]
    closeness_pre = operator.dot(initial_value).norm()
    guess = initial_guess
    time = 0
    time_steps = [0]
    h = step_size_first
    while time < time_end and closeness_pre > closeness_min and h > step_size_min:
        t_1 = sle.als(_shifted(operator, -h), guess.copy(), solution[-1], solver=solver, repeats=repeats)
        t_1 = (1 / t_1.norm(p=1)) * t_1
        t_2 = []
        if second_method == 'two_step_Euler':
            t_2 = sle.als(_shifted(operator, -0.5 * h), guess.copy(), solution[-1], solver=solver, repeats=repeats)
            t_2 = sle.als(_shifted(operator, -0.5 * h), t_2.copy(), solution[-1], solver=solver, repeats=repeats)
        if second_method == 'trapezoidal_rule':
            t_2 = sle.als(_shifted(operator, -0.5 * h), guess.copy(), _shifted(operator, 0.5 * h).dot(solution[-1]),
                          solver=solver, repeats=repeats)
        if normalize > 0:
            t_2 = (1 / t_2.norm(p=normalize)) * t_2
        closeness = operator.dot(t_1).norm()
        local_error = (t_1 - t_2).norm() / t_1.norm()
        closeness_difference = (closeness - closeness_pre) / closeness_pre
        factor_local = error_tol / local_error
        factor_closeness = closeness_tol / np.abs(closeness_difference)
        h_new = np.amin([factor_max, factor_safe * factor_local, factor_safe * factor_closeness]) * h
        if factor_local > 1 and factor_closeness > 1:
            time = np.min([time + h, time_end])
            h = np.amin([h_new, time_end - time, step_size_max])
            solution.append(t_2.copy())
            time_steps.append(time)
            guess = t_1
            closeness_pre = closeness
        else:
            h = h_new
    return solution, time_steps


# ----------------------------------------------------------------------------
# TDVP
# ----------------------------------------------------------------------------

_TDVP_KIND = {'adaptive': 0, 'one_site': 1, 'two_site': 2}

# statistics of the last TDVP run (device time, launches, local exponentials)
last_stats = {}


def _real_cores(t, what):
    cores = []
    for c in t.cores:
        if np.iscomplexobj(c):
            if np.any(np.imag(c) != 0):
                raise NotImplementedError(f'{what}: complex cores are not supported by the device TDVP path')
            c = np.real(c)
        cores.append(np.asarray(c, dtype=np.float64))
    return cores


def _krylov_dim(local_solver):
    """ode.py:1233-1238: no solver or 'exact' -> exact exponentials, anything
    else -> the local Krylov method, dimension 5 unless given (the dict is
    updated in place, as there)."""
    if not local_solver or local_solver['method'] == 'exact':
        return 0
    if not local_solver.get('dimension'):
        local_solver.setdefault('dimension', 5)
    return int(local_solver['dimension'])


def _run_tdvp(kind, operator, initial_value, step_size, number_of_steps, krylov_dim, threshold, max_rank,
              normalize):
    tau = -1j * complex(step_size)
    if tau.imag != 0.0:
        raise NotImplementedError('the device TDVP path needs a real exponent -1j*step_size (imaginary-time steps); '
                                  'real-time steps need complex cores')
    steps = int(number_of_steps)
    op_c = _real_cores(operator, 'operator')
    x_c = _real_cores(initial_value, 'initial_value')
    d = len(op_c)
    dims = [c.shape[1] for c in op_c]
    r0 = [c.shape[0] for c in x_c] + [x_c[-1].shape[3]]
    mr = 0 if max_rank is None or max_rank == np.inf else int(max_rank)
    cap = list(r0)
    if kind != 1:
        lft = np.cumprod([1] + dims).tolist()
        rgt = (np.cumprod(([1] + dims[::-1]))[::-1]).tolist()
        for i in range(1, d):
            c = min(lft[i], rgt[i])
            if mr > 0:
                c = min(c, mr)
            cap[i] = max(c, r0[i])
    step_total = sum(cap[i] * dims[i] * cap[i + 1] for i in range(d))
    out = np.empty(max(steps * step_total, 1))
    out_ranks = np.zeros(max(steps, 1) * (d + 1), dtype=np.int64)
    op, x0 = _lib.Packed(op_c), _lib.Packed(x_c)
    st = _lib.Stats()
    _lib.check(_lib.load().ttals_tdvp(_lib.context(), op.desc, x0.desc, _TDVP_KIND[kind], float(tau.real), steps,
                                       int(krylov_dim), float(threshold), mr, int(normalize), 0.0, _lib.dptr(out),
                                       out.size, 0, _lib.i64ptr(out_ranks), st))
    global last_stats
    last_stats = st.as_dict()
    solution = [initial_value]
    off = 0
    for k in range(steps):
        rk = out_ranks[k * (d + 1):(k + 1) * (d + 1)]
        cores = _lib.unpack(out[off:], dims, [1] * d, rk)
        off += sum(int(rk[i] * dims[i] * rk[i + 1]) for i in range(d))
        solution.append(tt.TT(cores))
    return solution


def tdvp1site(operator, initial_value, step_size, number_of_steps: int, local_solver=None, normalize: int = 0):
    """One-site TDVP (ode.py:1188-1288): each step a forward half sweep (local
    exponential of every core by step/2, QR, backward step of the bond matrix)
    and a backward half sweep (the reference always uses exact exponentials
    there).  Returns the list of states, ``initial_value`` first."""
    return _run_tdvp('one_site', operator, initial_value, step_size, number_of_steps, _krylov_dim(local_solver),
                     0.0, np.inf, normalize)


def tdvp2site(operator, initial_value, step_size, number_of_steps: int, local_solver=None, threshold=1e-12,
              max_rank=50, normalize: int = 0):
    """Two-site TDVP (ode.py:1290-1396): two-site local exponentials, truncated
    SVD splits (``threshold`` relative to the largest singular value,
    ``max_rank``), one-site backward steps."""
    return _run_tdvp('two_site', operator, initial_value, step_size, number_of_steps, _krylov_dim(local_solver),
                     threshold, max_rank, normalize)


def tdvp(operator, initial_value, step_size, number_of_steps: int, threshold=1e-12, max_rank=50,
         normalize: int = 0):
    """Adaptive TDVP (ode.py:1076-1186): a two-site update on every bond whose
    rank is below ``max_rank`` and below the dimensions on both sides, else a
    one-site update.  The reference calls its update helpers without their
    ``local_solver`` argument and stops with a TypeError; this runs the
    evident intent with exact local exponentials."""
    return _run_tdvp('adaptive', operator, initial_value, step_size, number_of_steps, 0, threshold, max_rank,
                     normalize)
