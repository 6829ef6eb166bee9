"""NumPy restatement of scikit_tt's tensor-train ALS hot path (CPU oracle).

TEST INFRASTRUCTURE ONLY: imported by ``tests/``, ``__graft_entry__.smoke()``
and ``bench.py`` (CPU baseline / reference arm).  The product package never
imports it.

A tensor train is a plain ``list`` of 4-D NumPy cores ``(r_i, m_i, n_i,
r_{i+1})`` (row dimension m, column dimension n), exactly the layout of
``scikit_tt/tensor_train.py:184-188``.  The algorithms follow the reference
line by line in meaning (same contractions, same dense local solves, same
QR/RQ/SVD rank rules, same sweep schedule and stopping rule); the code itself
is written with ``einsum`` instead of chains of ``tensordot``.

Pinned against the reference's own outputs: ``tests/golden/*.npz`` were
produced by ``tests/golden/make_golden.py`` from the reference package, and
``tests/test_oracle_golden.py`` checks this module against them.
"""

from __future__ import annotations

import math

import numpy as np
import scipy.linalg as sla
import scipy.sparse.linalg as spla

# ----------------------------------------------------------------------------
# interface stacks (sle.py:194-305, evp.py:253-334)
# ----------------------------------------------------------------------------


def stack_left_op(prev, x, a, conj_first=False):
    """Left operator stack ``L_i[s, R', s']`` from ``L_{i-1}``, core ``x`` (3-D
    ``(a, n, s)``) and operator core ``a`` ``(R, m, n, R')``.

    SLE (sle.py:217-219): ``sum L[a,R,a'] x[a,n,s] A[R,m,n,R'] conj(x)[a',m,s']``.
    EVP (evp.py:281-283) conjugates the first factor instead
    (``conj_first=True``); both agree for real data.
    """
    xl = np.conj(x) if conj_first else x
    xr = x if conj_first else np.conj(x)
    return np.einsum('aRb,ans,RmnQ,bmt->sQt', prev, xl, a, xr, optimize=True)


def stack_right_op(nxt, x, a):
    """Right operator stack ``R_i[a, R, a']`` (sle.py:274-276, evp.py:323-325):
    ``sum x[a,n,s] A[R,m,n,R'] conj(x)[a',m,s'] R_{i+1}[s,R',s']``."""
    return np.einsum('ans,RmnQ,bmt,sQt->aRb', x, a, np.conj(x), nxt, optimize=True)


def stack_left_vec(prev, x, b):
    """Left stack of a TT vector against the solution (sle.py:246-247,
    evp.py:291-292): ``Lb_i[g, s'] = sum Lb[h,a'] b[h,m,g] conj(x)[a',m,s']``."""
    return np.einsum('hb,hmg,bmt->gt', prev, b, np.conj(x), optimize=True)


def stack_right_vec(nxt, x, b):
    """Right stack of a TT vector (sle.py:303-305, evp.py:333-334):
    ``Rb_i[h, a'] = sum b[h,m,g] conj(x)[a',m,s'] Rb_{i+1}[g,s']``."""
    return np.einsum('hmg,bmt,gt->hb', b, np.conj(x), nxt, optimize=True)


def micro_matrix(left, a, right):
    """Dense local operator (sle.py:339-345, evp.py:359-365):
    ``M[(a',m,s'), (a,n,s)] = sum L[a,R,a'] A[R,m,n,R'] Rt[s,R',s']``."""
    r0, _, r0p = left.shape
    rr, _, rrp = right.shape
    m, n = a.shape[1], a.shape[2]
    t = np.einsum('aRb,RmnQ,sQt->bmtans', left, a, right, optimize=True)
    return t.reshape(r0p * m * rrp, r0 * n * rr)


def micro_vec(left, b, right):
    """Local right-hand side (sle.py:424-428, evp.py:377-379):
    ``f[(a',m,s')] = sum Lb[h,a'] b[h,m,g] Rb[g,s']`` as an ``(N, 1)`` column."""
    f = np.einsum('hb,hmg,gt->bmt', left, b, right, optimize=True)
    return f.reshape(-1, 1)


# ----------------------------------------------------------------------------
# sle.als (sle.py:10-95, 475-547)
# ----------------------------------------------------------------------------


def _update_core_sle(i, mop, mrhs, cores, ranks, dims, solver, direction):
    """Local solve plus QR/RQ re-gauging, sle.py:475-547."""
    if solver == 'solve':
        cores[i] = np.linalg.solve(mop, mrhs)
    elif solver == 'lu':
        lu = sla.lu_factor(mop, overwrite_a=True, check_finite=False)
        cores[i] = sla.lu_solve(lu, mrhs, trans=0, overwrite_b=True, check_finite=False)
    # any other solver string: the reference skips the solve and re-gauges the
    # old core (sle.py:505-509 has no else branch)
    a, n, s = ranks[i], dims[i], ranks[i + 1]
    if direction == 'forward':
        q, _ = sla.qr(np.reshape(cores[i], (a * n, s)), mode='economic', check_finite=False)
        ranks[i + 1] = q.shape[1]
        cores[i] = q.reshape(a, n, 1, ranks[i + 1])
    else:
        if i > 0:
            _, q = sla.rq(np.reshape(cores[i], (a, n * s)), mode='economic', check_finite=False)
            ranks[i] = q.shape[0]
            cores[i] = q.reshape(ranks[i], n, 1, s)
        else:
            cores[i] = np.reshape(cores[i], (a, n, 1, s))


def sle_als(op, x0, b, repeats=1, solver='solve'):
    """One-site ALS for ``op @ x = b`` (sle.py:10-95).  Returns the core list."""
    d = len(op)
    cores = [c.copy() for c in x0]
    ranks = [c.shape[0] for c in cores] + [cores[-1].shape[3]]
    dims = [c.shape[1] for c in op]
    sl_op, sl_b, sr_op, sr_b = [None] * d, [None] * d, [None] * d, [None] * d

    def right(i):
        if i == d - 1:
            sr_op[i] = np.ones((1, 1, 1))
            sr_b[i] = np.ones((1, 1))
        else:
            x = cores[i + 1][:, :, 0, :]
            sr_op[i] = stack_right_op(sr_op[i + 1], x, op[i + 1])
            sr_b[i] = stack_right_vec(sr_b[i + 1], x, b[i + 1][:, :, 0, :])

    def left(i):
        if i == 0:
            sl_op[i] = np.ones((1, 1, 1))
            sl_b[i] = np.ones((1, 1))
        else:
            x = cores[i - 1][:, :, 0, :]
            sl_op[i] = stack_left_op(sl_op[i - 1], x, op[i - 1])
            sl_b[i] = stack_left_vec(sl_b[i - 1], x, b[i - 1][:, :, 0, :])

    def micro(i):
        return (micro_matrix(sl_op[i], op[i], sr_op[i]),
                micro_vec(sl_b[i], b[i][:, :, 0, :], sr_b[i]))

    for i in range(d - 1, -1, -1):          # sle.py:54-56
        right(i)
    for _ in range(repeats):                 # sle.py:62-93
        for i in range(d):
            left(i)
            if i < d - 1:
                mop, mrhs = micro(i)
                _update_core_sle(i, mop, mrhs, cores, ranks, dims, solver, 'forward')
        for i in range(d - 1, -1, -1):
            right(i)
            mop, mrhs = micro(i)
            _update_core_sle(i, mop, mrhs, cores, ranks, dims, solver, 'backward')
    return cores


# ----------------------------------------------------------------------------
# sle.mals (sle.py:98-191, 350-472, 550-650)
# ----------------------------------------------------------------------------


def _merged_vec(b1, b2):
    """Two-site right-hand side core (h, m1 m2, g) of sle.py:466-470."""
    h, m1, _ = b1.shape
    _, m2, g = b2.shape
    return np.einsum('aib,bjc->aijc', b1, b2).reshape(h, m1 * m2, g)


def _split_mals(i, sol, cores, ranks, dims, threshold, max_rank, direction):
    """SVD split of the two-site solution, sle.py:604-650: reshape to
    (r_i n_i) x (n_{i+1} r_{i+2}), gesvd, keep sigma_k / sigma_0 > threshold,
    then at most max_rank.  Forward keeps U as core i; backward keeps V as
    core i+1 and, at the first pair, U diag(s) as core 0."""
    a, n1, n2, s = ranks[i], dims[i], dims[i + 1], ranks[i + 2]
    u, sv, v = sla.svd(sol.reshape(a * n1, n2 * s), full_matrices=False, check_finite=False,
                       lapack_driver='gesvd')
    if threshold != 0:
        keep = np.where(sv / sv[0] > threshold)[0]
        u, sv, v = u[:, keep], sv[keep], v[keep, :]
    if max_rank != np.inf:
        k = int(min(u.shape[1], max_rank))
        u, sv, v = u[:, :k], sv[:k], v[:k, :]
    k = sv.shape[0]
    ranks[i + 1] = k
    if direction == 'forward':
        cores[i] = u.reshape(a, n1, 1, k)
    else:
        cores[i + 1] = v.reshape(k, n2, 1, s)
        if i == 0:
            cores[0] = (u * sv).reshape(a, n1, 1, k)


def sle_mals(op, x0, b, repeats=1, solver='solve', threshold=1e-12, max_rank=np.inf):
    """Two-site MALS for ``op @ x = b`` (sle.py:98-191).  The micro system of
    sites (i, i+1) is the one-site system of the merged site (sle.py:350-390,
    433-472); the split follows ``_split_mals``.  Returns the core list."""
    d = len(op)
    cores = [c.copy() for c in x0]
    ranks = [c.shape[0] for c in cores] + [cores[-1].shape[3]]
    dims = [c.shape[1] for c in op]
    sl_op, sl_b, sr_op, sr_b = [None] * d, [None] * d, [None] * d, [None] * d

    def right(i):
        if i == d - 1:
            sr_op[i], sr_b[i] = np.ones((1, 1, 1)), np.ones((1, 1))
        else:
            x = cores[i + 1][:, :, 0, :]
            sr_op[i] = stack_right_op(sr_op[i + 1], x, op[i + 1])
            sr_b[i] = stack_right_vec(sr_b[i + 1], x, b[i + 1][:, :, 0, :])

    def left(i):
        if i == 0:
            sl_op[i], sl_b[i] = np.ones((1, 1, 1)), np.ones((1, 1))
        else:
            x = cores[i - 1][:, :, 0, :]
            sl_op[i] = stack_left_op(sl_op[i - 1], x, op[i - 1])
            sl_b[i] = stack_left_vec(sl_b[i - 1], x, b[i - 1][:, :, 0, :])

    def update(i, direction):                      # sle.py:550-603
        mop = micro_matrix(sl_op[i], _merged_op(op[i], op[i + 1]), sr_op[i + 1])
        mrhs = micro_vec(sl_b[i], _merged_vec(b[i][:, :, 0, :], b[i + 1][:, :, 0, :]), sr_b[i + 1])
        if solver == 'solve':
            sol = np.linalg.solve(mop, mrhs)
        elif solver == 'lu':
            sol = sla.lu_solve(sla.lu_factor(mop, check_finite=False), mrhs, check_finite=False)
        else:
            raise ValueError(f'unknown solver {solver!r}')
        _split_mals(i, sol, cores, ranks, dims, threshold, max_rank, direction)

    for i in range(d - 1, 0, -1):                  # sle.py:148-150
        right(i)
    for _ in range(repeats):                       # sle.py:156-189
        for i in range(d - 1):
            left(i)
            if i < d - 2:
                update(i, 'forward')
        for i in range(d - 2, -1, -1):
            right(i + 1)
            update(i, 'backward')
    return cores


# ----------------------------------------------------------------------------
# linear ODE integrators (ode.py:16-115, 249-636) and evp.power_method
# (evp.py:182-250): compositions of sle.als / sle.mals with TT algebra.
# Operators here are small (full vectors are used for the norms).
# ----------------------------------------------------------------------------


def tt_eye(dims):
    """Identity operator, ranks 1 (tensor_train.py:1870-1893)."""
    return [np.eye(n).reshape(1, n, n, 1) for n in dims]


def _shifted(op, alpha):
    """``tt.eye + alpha * op`` as a rank sum (tensor_train.py:282-344, 368-399)."""
    return tt_add(tt_eye([c.shape[1] for c in op]), tt_scale(op, alpha))


def _vnorm(t):
    return float(np.linalg.norm(full_vector(t)))


def _normalise(t, p):
    return tt_scale(t, 1.0 / _norm_p(t, p)) if p > 0 else t


def explicit_euler(op, x0, step_sizes, threshold=1e-12, max_rank=50, normalize=1):
    """ode.py:16-82: x_{k+1} = (I + h A) x_k, then ``TT.ortho(threshold,
    max_rank)`` (left sweep untruncated in rank, right sweep capped,
    tensor_train.py:1312-1332), then division by the p-norm."""
    sol = [x0]
    for h in step_sizes:
        t = tt_matmul(_shifted(op, h), sol[-1])
        t = ortho_right(ortho_left(t, threshold), threshold, max_rank)
        sol.append(_normalise(t, normalize))
    return sol


def errors_expl_euler(op, sol, step_sizes):
    """ode.py:85-114: ||x_{k+1} - (I + h A) x_k|| / ||x_k||."""
    return [_vnorm(tt_add(sol[k + 1], tt_scale(tt_matmul(_shifted(op, h), sol[k]), -1.0))) / _vnorm(sol[k])
            for k, h in enumerate(step_sizes)]


def _tt_ortho(t, threshold=0.0, max_rank=np.inf):
    """TT.ortho (tensor_train.py:1312-1332): left sweep uncapped, right sweep capped."""
    return ortho_right(ortho_left(t, threshold), threshold, max_rank)


def _odd_series(op, scale, step, order):
    """scale*step*A + sum_{k=2}^{order/2} 2/(2k-1)! step^(2k-1) A^(2k-1) (ode.py:186-191, 203-208)."""
    series = tt_scale(op, scale * step)
    power = [c.copy() for c in op]
    for k in range(2, order // 2 + 1):
        power = tt_matmul(tt_matmul(power, op), op)
        series = tt_add(series, tt_scale(power, 2 / math.factorial(2 * k - 1) * step ** (2 * k - 1)))
    return series


def hod(op, x0, step_size, number_of_steps, order=2, previous_value=None, op_hod=None, threshold=1e-12,
        max_rank=50, normalize=1):
    """Higher-order differencing, ode.py:117-247: x_{k+1} = x_{k-1} + S x_k with
    S = 2hA + sum_k 2/(2k-1)! h^(2k-1) A^(2k-1) (order raised to even), every
    new state re-truncated by TT.ortho(threshold, max_rank) and normalised; the
    state before x_0 is x_0 - S_{h/2} (I - h/2 A) x_0 unless given."""
    if order % 2:
        order += 1
    if op_hod is None:
        op_hod = _tt_ortho(_odd_series(op, 2.0, step_size, order), threshold)
    sol = [x0]
    for i in range(number_of_steps):
        if i == 0:
            if previous_value is None:
                op_first = _tt_ortho(_odd_series(op, 2.0, step_size / 2, order), threshold)
                back = tt_matmul(_shifted(op, -0.5 * step_size), sol[0])
                prev = tt_add(sol[0], tt_scale(tt_matmul(op_first, back), -1.0))
            else:
                prev = previous_value
            prev = _tt_ortho(_normalise(prev, normalize), threshold, max_rank)
        else:
            prev = sol[i - 1]
        nxt = _tt_ortho(tt_add(prev, tt_matmul(op_hod, sol[i])), threshold, max_rank)
        sol.append(_normalise(nxt, normalize))
    return sol


def _tt_solve(tt_solver, mop, guess, rhs, micro_solver, repeats, threshold, max_rank):
    if tt_solver == 'als':
        return sle_als(mop, guess, rhs, repeats=repeats, solver=micro_solver)
    return sle_mals(mop, guess, rhs, repeats=repeats, solver=micro_solver, threshold=threshold, max_rank=max_rank)


def implicit_euler(op, x0, guess, step_sizes, repeats=1, tt_solver='als', threshold=1e-12, max_rank=np.inf,
                   micro_solver='solve', normalize=1):
    """ode.py:249-330: (I - h A) x_{k+1} = x_k by ALS/MALS, warm-started from
    the previous solution, then division by the p-norm."""
    sol, t = [x0], guess
    for h in step_sizes:
        t = _tt_solve(tt_solver, _shifted(op, -h), t, sol[-1], micro_solver, repeats, threshold, max_rank)
        t = _normalise(t, normalize)
        sol.append(t)
    return sol


def errors_impl_euler(op, sol, step_sizes):
    """ode.py:333-363: ||(I - h A) x_{k+1} - x_k|| / ||x_k||."""
    return [_vnorm(tt_add(tt_matmul(_shifted(op, -h), sol[k + 1]), tt_scale(sol[k], -1.0))) / _vnorm(sol[k])
            for k, h in enumerate(step_sizes)]


def trapezoidal_rule(op, x0, guess, step_sizes, repeats=1, tt_solver='als', threshold=1e-12, max_rank=np.inf,
                     micro_solver='solve', normalize=1):
    """ode.py:366-451: (I - h/2 A) x_{k+1} = (I + h/2 A) x_k."""
    sol, t = [x0], guess
    for h in step_sizes:
        rhs = tt_matmul(_shifted(op, 0.5 * h), sol[-1])
        t = _tt_solve(tt_solver, _shifted(op, -0.5 * h), t, rhs, micro_solver, repeats, threshold, max_rank)
        t = _normalise(t, normalize)
        sol.append(t)
    return sol


def errors_trapezoidal(op, sol, step_sizes):
    """ode.py:453-485: ||(I - h/2 A) x_{k+1} - (I + h/2 A) x_k|| / ||(I + h/2 A) x_k||."""
    out = []
    for k, h in enumerate(step_sizes):
        fwd = tt_matmul(_shifted(op, 0.5 * h), sol[k])
        out.append(_vnorm(tt_add(tt_matmul(_shifted(op, -0.5 * h), sol[k + 1]), tt_scale(fwd, -1.0))) / _vnorm(fwd))
    return out


def adaptive_step_size(op, x0, guess, time_end, step_size_first=1e-10, repeats=1, solver='solve', error_tol=1e-1,
                       closeness_tol=0.5, step_size_min=1e-14, step_size_max=10, closeness_min=1e-3, factor_max=2,
                       factor_safe=0.9, second_method='two_step_Euler', normalize=1):
    """ode.py:487-636: an implicit Euler step t1 (1-norm normalised) against a
    second method t2 (two half implicit Euler solves, both with the previous
    state as right-hand side as the reference has it, or the trapezoidal
    rule); a step is accepted when the local error and the relative change
    of ||A x|| both stay inside their tolerances.  Returns (states, times)."""
    sol, times = [x0], [0]
    closeness_pre = _vnorm(tt_matmul(op, x0))
    t_tmp, time, h = guess, 0, step_size_first
    while time < time_end and closeness_pre > closeness_min and h > step_size_min:
        t1 = _normalise(sle_als(_shifted(op, -h), t_tmp, sol[-1], repeats=repeats, solver=solver), 1)
        if second_method == 'two_step_Euler':
            t2 = sle_als(_shifted(op, -0.5 * h), t_tmp, sol[-1], repeats=repeats, solver=solver)
            t2 = sle_als(_shifted(op, -0.5 * h), t2, sol[-1], repeats=repeats, solver=solver)
        else:
            t2 = sle_als(_shifted(op, -0.5 * h), t_tmp, tt_matmul(_shifted(op, 0.5 * h), sol[-1]), repeats=repeats,
                         solver=solver)
        t2 = _normalise(t2, normalize)
        closeness = _vnorm(tt_matmul(op, t1))
        local_error = _vnorm(tt_add(t1, tt_scale(t2, -1.0))) / _vnorm(t1)
        closeness_difference = (closeness - closeness_pre) / closeness_pre
        factor_local = error_tol / local_error
        factor_closeness = closeness_tol / np.abs(closeness_difference)
        h_new = np.amin([factor_max, factor_safe * factor_local, factor_safe * factor_closeness]) * h
        if factor_local > 1 and factor_closeness > 1:
            time = np.min([time + h, time_end])
            h = np.amin([h_new, time_end - time, step_size_max])
            sol.append(t2)
            times.append(time)
            t_tmp, closeness_pre = t1, closeness
        else:
            h = h_new
    return sol, times


def power_method(op, x0, op_gevp=None, repeats=10, sigma=0.999):
    """evp.py:182-250: inverse power iteration x <- (A - sigma M)^{-1} M x by
    one ALS sweep per step (M = I without ``op_gevp``), x <- x / ||x||, and the
    Rayleigh quotient x^T A x (/ x^T M x).  Returns (eigenvalue, cores)."""
    dims = [c.shape[1] for c in op]
    mass = op_gevp if op_gevp is not None else tt_eye(dims)
    shifted = tt_add(op, tt_scale(mass, -sigma))
    x, val = x0, 0.0
    for _ in range(repeats):
        rhs = x if op_gevp is None else tt_matmul(op_gevp, x)
        x = sle_als(shifted, x, rhs)
        x = tt_scale(x, 1.0 / _vnorm(x))
        v = full_vector(x)
        val = float(v @ full_matrix(op) @ v)
        if op_gevp is not None:
            val /= float(v @ full_matrix(op_gevp) @ v)
    return val, x


# ----------------------------------------------------------------------------
# evp.als (evp.py:17-179, 386-495)
# ----------------------------------------------------------------------------


def _local_eig(mop, mgevp, number_ev, solver, sigma, real):
    """Local eigensolve and selection rule, evp.py:414-443."""
    vals = vecs = None
    if solver == 'eigs':
        v0 = np.ones(mop.shape[0])
        vals, vecs = spla.eigs(mop, M=mgevp, sigma=sigma, k=number_ev, v0=v0)
        idx = np.abs(vals - sigma).argsort()[::-1]
        vals, vecs = vals[idx], vecs[:, idx]
    if solver == 'eig':
        vals, vecs = sla.eig(mop, b=mgevp, overwrite_a=True, overwrite_b=True, check_finite=False)
        idx = np.abs(vals - sigma).argsort()
        vals, vecs = vals[idx[:number_ev]], vecs[:, idx[:number_ev]]
    if solver == 'eigh':
        n = mop.shape[0]
        vals, vecs = sla.eigh(mop, b=mgevp, overwrite_a=True, overwrite_b=True, check_finite=False,
                              subset_by_index=(n - number_ev, n - 1))
        vals, vecs = vals[::-1], vecs[:, ::-1]
    if real is True:
        vals = np.real(vals)
    return vals, vecs


def evp_als(op, x0, previous=(), shift=0.0, op_gevp=None, number_ev=1, repeats=1,
            conv_eps=1e-10, solver='eig', sigma=1.0, real=True):
    """One-site ALS eigensolver (evp.py:17-179).

    Returns ``(eigenvalue(s), cores or list of core lists, iterations)`` with the
    reference's return conventions: for ``number_ev == 1`` the best pair over the
    sweeps (evp.py:151-155), else the last sweep's values and one TT per
    eigenvector (evp.py:172-175).
    """
    d = len(op)
    cores = [c.copy() for c in x0]
    ranks = [c.shape[0] for c in cores] + [cores[-1].shape[3]]
    dims = [c.shape[1] for c in op]
    prev = list(previous)
    so_l, so_r = [None] * d, [None] * d
    sg_l, sg_r = [None] * d, [None] * d
    sp_l = [[None] * d for _ in prev]
    sp_r = [[None] * d for _ in prev]

    def left(i):                                   # evp.py:253-292
        if i == 0:
            so_l[i] = np.ones((1, 1, 1))
            if op_gevp is not None:
                sg_l[i] = np.ones((1, 1, 1))
            for j in range(len(prev)):
                sp_l[j][i] = np.ones((1, 1))
            return
        x = cores[i - 1][:, :, 0, :]
        so_l[i] = stack_left_op(so_l[i - 1], x, op[i - 1], conj_first=True)
        if op_gevp is not None:
            sg_l[i] = stack_left_op(sg_l[i - 1], x, op_gevp[i - 1], conj_first=True)
        for j in range(len(prev)):
            sp_l[j][i] = stack_left_vec(sp_l[j][i - 1], x, prev[j][i - 1][:, :, 0, :])

    def right(i):                                  # evp.py:295-334
        if i == d - 1:
            so_r[i] = np.ones((1, 1, 1))
            if op_gevp is not None:
                sg_r[i] = np.ones((1, 1, 1))
            for j in range(len(prev)):
                sp_r[j][i] = np.ones((1, 1))
            return
        x = cores[i + 1][:, :, 0, :]
        so_r[i] = stack_right_op(so_r[i + 1], x, op[i + 1])
        if op_gevp is not None:
            sg_r[i] = stack_right_op(sg_r[i + 1], x, op_gevp[i + 1])
        for j in range(len(prev)):
            sp_r[j][i] = stack_right_vec(sp_r[j][i + 1], x, prev[j][i + 1][:, :, 0, :])

    def micro(i):                                  # evp.py:337-383
        mop = micro_matrix(so_l[i], op[i], so_r[i])
        mg = micro_matrix(sg_l[i], op_gevp[i], sg_r[i]) if op_gevp is not None else None
        for j in range(len(prev)):
            t = micro_vec(sp_l[j][i], prev[j][i][:, :, 0, :], sp_r[j][i])
            mop = mop + shift * t.dot(np.conj(t.T))
        return mop, mg

    def update(i, mop, mg, direction):             # evp.py:386-495
        vals, vecs = _local_eig(mop, mg, number_ev, solver, sigma, real)
        a, n, s = ranks[i], dims[i], ranks[i + 1]
        if direction == 'forward':
            u, _, _ = sla.svd(vecs.reshape(a * n, s * number_ev), check_finite=False, lapack_driver='gesvd')
            r = min(s, u.shape[1])
            ranks[i + 1] = r
            cores[i] = u[:, :r].reshape(a, n, 1, r)
        else:
            if i > 0:
                vt = vecs.transpose()
                _, _, v = sla.svd(vt.reshape(number_ev * a, n * s), check_finite=False, lapack_driver='gesvd')
                r = min(a, v.shape[0])
                ranks[i] = r
                cores[i] = v[:r, :].reshape(r, n, 1, s)
            else:
                cores[i] = vecs.reshape(a, n, 1, s, number_ev)
        return vals

    for i in range(d - 1, -1, -1):
        right(i)
    it = 1
    vals_pre = np.array([np.inf] * number_ev)[None, :]
    converged = False
    val_opt, cores_opt = np.inf, None
    vals = None
    while it <= repeats and not converged:         # evp.py:118-165
        for i in range(d):
            left(i)
            if i < d - 1:
                mop, mg = micro(i)
                vals = update(i, mop, mg, 'forward')
        for i in range(d - 1, -1, -1):
            right(i)
            mop, mg = micro(i)
            vals = update(i, mop, mg, 'backward')
        it += 1
        if number_ev == 1 and np.abs(vals[0] - sigma) < np.abs(val_opt - sigma):
            val_opt = vals[0].copy()
            cores_opt = [cores[0][:, :, :, :, 0]] + cores[1:]
        last = vals_pre[-min(3, vals_pre.shape[0]):, :]
        if np.amax(np.abs(last - vals)) < conv_eps:
            converged = True
        vals_pre = np.vstack((vals_pre, vals))
    if number_ev == 1:
        return val_opt, cores_opt, it - 1
    tts = [[cores[0][:, :, :, :, k]] + cores[1:] for k in range(number_ev)]
    return vals, tts, it - 1


# ----------------------------------------------------------------------------
# TT algebra used by the harness (tensor_train.py)
# ----------------------------------------------------------------------------


def tt_matmul(t, u):
    """Core-wise operator product (tensor_train.py:447-501); the combined rank
    index has ``t``'s rank as the major index.  Returns cores (no scalar
    collapse)."""
    out = []
    for c1, c2 in zip(t, u):
        r1, m, _, r2 = c1.shape
        s1, _, p, s2 = c2.shape
        out.append(np.einsum('aijb,cjkd->acikbd', c1, c2).reshape(r1 * s1, m, p, r2 * s2))
    return out


def tt_add(t, u):
    """Block-diagonal rank sum (tensor_train.py:282-344)."""
    d = len(t)
    rt = [c.shape[0] for c in t] + [1]
    ru = [c.shape[0] for c in u] + [1]
    ranks = [1] + [rt[i] + ru[i] for i in range(1, d)] + [1]
    out = []
    for i in range(d):
        m, n = t[i].shape[1], t[i].shape[2]
        dt = np.result_type(t[i], u[i])
        c = np.zeros((ranks[i], m, n, ranks[i + 1]), dtype=dt)
        c[:rt[i], :, :, :rt[i + 1]] = t[i]
        c[ranks[i] - ru[i]:, :, :, ranks[i + 1] - ru[i + 1]:] = u[i]
        out.append(c)
    return out


def tt_scale(t, alpha):
    """Scalar times TT: scales the first core (tensor_train.py:368-399)."""
    return [alpha * t[0]] + [c.copy() for c in t[1:]]


def ortho_left(t, threshold=0.0, max_rank=np.inf):
    """SVD left-orthonormalisation (tensor_train.py:1161-1191); returns new cores."""
    t = [c.copy() for c in t]
    d = len(t)
    for i in range(d - 1):
        r, m, n, s = t[i].shape
        try:
            u, sv, v = sla.svd(t[i].reshape(r * m * n, s), full_matrices=False, check_finite=False)
        except sla.LinAlgError:
            u, sv, v = sla.svd(t[i].reshape(r * m * n, s), full_matrices=False, check_finite=False,
                               lapack_driver='gesvd')
        if threshold != 0:
            keep = np.where(sv / sv[0] > threshold)[0]
            u, sv, v = u[:, keep], sv[keep], v[keep, :]
        if max_rank != np.inf:
            k = int(min(u.shape[1], max_rank))
            u, sv, v = u[:, :k], sv[:k], v[:k, :]
        t[i] = u.reshape(r, m, n, u.shape[1])
        t[i + 1] = np.tensordot(np.diag(sv).dot(v), t[i + 1], axes=(1, 0))
    return t


def ortho_right(t, threshold=0.0, max_rank=np.inf):
    """SVD right-orthonormalisation (tensor_train.py:1267-1299); returns new cores."""
    t = [c.copy() for c in t]
    d = len(t)
    for i in range(d - 1, 0, -1):
        r, m, n, s = t[i].shape
        try:
            u, sv, v = sla.svd(t[i].reshape(r, m * n * s), full_matrices=False, check_finite=False)
        except sla.LinAlgError:
            u, sv, v = sla.svd(t[i].reshape(r, m * n * s), full_matrices=False, check_finite=False,
                               lapack_driver='gesvd')
        if threshold != 0:
            keep = np.where(sv / sv[0] > threshold)[0]
            u, sv, v = u[:, keep], sv[keep], v[keep, :]
        if max_rank != np.inf:
            k = int(min(v.shape[0], max_rank))
            u, sv, v = u[:, :k], sv[:k], v[:k, :]
        k = v.shape[0]
        t[i] = v.reshape(k, m, n, s)
        p = t[i - 1]
        t[i - 1] = (p.reshape(-1, p.shape[3]).dot(u).dot(np.diag(sv))).reshape(p.shape[0], p.shape[1],
                                                                                  p.shape[2], k)
    return t


def norm2(t):
    """2-norm (tensor_train.py:1409-1425): flatten operator cores, right-
    orthonormalise, Frobenius norm of the first core."""
    is_op = not (all(c.shape[1] == 1 for c in t) or all(c.shape[2] == 1 for c in t))
    if is_op:
        t = [c.reshape(c.shape[0], c.shape[1] * c.shape[2], 1, c.shape[3]) for c in t]
    t = ortho_right(t)
    return float(np.linalg.norm(t[0].ravel()))


def full_vector(t):
    """Dense vector of a TT with unit column dims (tensor_train.py:1061-1090)."""
    v = t[0].reshape(t[0].shape[1], t[0].shape[3])
    for c in t[1:]:
        v = np.tensordot(v, c[:, :, 0, :], axes=(1, 0)).reshape(-1, c.shape[3])
    return v.reshape(-1)


def full_matrix(t):
    """Dense matrix of a TT operator (tensor_train.py:1061-1090)."""
    mat = t[0].reshape(t[0].shape[1], t[0].shape[2], t[0].shape[3])
    for c in t[1:]:
        mat = np.tensordot(mat, c, axes=(2, 0))
        mat = mat.transpose(0, 2, 1, 3, 4)
        mat = mat.reshape(mat.shape[0] * mat.shape[1], mat.shape[2] * mat.shape[3], c.shape[3])
    return mat[:, :, 0]


# ----------------------------------------------------------------------------
# numerically stable metrics (needed at large d, where ||b|| reaches 1e40)
# ----------------------------------------------------------------------------


def stable_norm(t):
    """Euclidean norm via a left-to-right QR sweep with the norm carried in the
    last core; avoids the over/underflow the SVD-based ``norm`` meets on
    unnormalised trains."""
    t = [c.reshape(c.shape[0], -1, c.shape[3]) for c in t]
    logscale = 0.0
    carry = np.ones((1, 1))
    for i, c in enumerate(t):
        c = np.tensordot(carry, c, axes=(1, 0))
        r, k, s = c.shape
        if i == len(t) - 1:
            nrm = np.linalg.norm(c.ravel())
            return float(nrm * np.exp(logscale)) if nrm > 0 else 0.0
        q, rr = np.linalg.qr(c.reshape(r * k, s))
        sc = np.linalg.norm(rr)
        if sc == 0:
            return 0.0
        logscale += np.log(sc)
        carry = rr / sc
    return 0.0


def stable_rel_diff(x, y):
    """``||x - y|| / ||y||`` of two TT vectors, computed stably."""
    ny = stable_norm(y)
    return stable_norm(tt_add(x, tt_scale(y, -1.0))) / ny


def stable_residual(op, x, b):
    """``||op @ x - b|| / ||b||`` computed stably (left-orthonormal sweep)."""
    ax = tt_matmul(op, x)
    return stable_rel_diff(ax, b)


def ising_exact_e0(d, coupling, field):
    """Ground energy of the open transverse-field Ising chain
    ``H = -J sum z_i z_{i+1} - g sum x_i`` by free fermions (Pfeuty 1970):
    ``E0 = -sum_k sigma_k(B)`` with ``B = bidiag(g on the diagonal, J above)``."""
    bmat = np.diag(field * np.ones(d)) + np.diag(coupling * np.ones(d - 1), 1)
    return -float(np.sum(np.linalg.svd(bmat, compute_uv=False)))


# ----------------------------------------------------------------------------
# TDVP time stepping (ode.py:1076-1616, 1689-1758)
# ----------------------------------------------------------------------------
#
# Every step is x <- exp(tau H) x with a REAL exponent tau = -1j * step_size
# (imaginary-time steps), computed in real arithmetic: the reference's complex
# arrays keep zero imaginary parts for such steps.


def truncated_svd(mat, threshold=0.0, max_rank=np.inf):
    """utils.py:111-158: thin SVD, keep sigma_i / sigma_0 > threshold, then at
    most max_rank values."""
    try:
        u, s, v = sla.svd(mat, full_matrices=False, check_finite=False)
    except np.linalg.LinAlgError:
        u, s, v = sla.svd(mat, full_matrices=False, check_finite=False, lapack_driver='gesvd')
    if threshold != 0:
        idx = np.where(s / s[0] > threshold)[0]
        u, s, v = u[:, idx], s[idx], v[idx, :]
    if max_rank != np.inf:
        k = int(min(len(s), max_rank))
        u, s, v = u[:, :k], s[:k], v[:k, :]
    return u, s, v


def local_krylov(mop, v0, dim, coef):
    """ode.py:1689-1758 with the exponent coefficient coef (= -1j * step):
    three-term Lanczos recurrence from the UNNORMALISED start vector, no
    reorthogonalisation, then ``sum_j [exp(coef T) e_1]_j v_j``."""
    T = np.zeros((dim, dim))
    vs = [v0]
    w = mop @ v0
    alpha = w @ v0
    T[0, 0] = alpha
    w = w - alpha * v0
    for i in range(1, dim):
        beta = np.linalg.norm(w)
        T[i, i - 1] = T[i - 1, i] = beta
        vs.append(w / beta)
        w = mop @ vs[-1]
        alpha = w @ vs[-1]
        T[i, i] = alpha
        w = w - alpha * vs[-1] - beta * vs[-2]
    e1 = np.zeros(dim)
    e1[0] = 1.0
    c = spla.expm_multiply(coef * T, e1)
    out = c[0] * vs[0]
    for j in range(1, dim):
        out = out + c[j] * vs[j]
    return out


def _expv(mop, v, coef, kdim):
    """exp(coef M) v: scipy's expm_multiply (local solver 'exact') or the local
    Krylov method of dimension kdim."""
    if kdim:
        return local_krylov(mop, v, kdim, coef)
    return spla.expm_multiply(coef * mop, v)


def _merged_op(a1, a2):
    """Two-site operator core (R, m1 m2, n1 n2, Q) of the two-site micro matrix
    (sle.py:350-390)."""
    r, m1, n1, _ = a1.shape
    _, m2, n2, q = a2.shape
    return np.einsum('aijb,bklc->aikjlc', a1, a2).reshape(r, m1 * m2, n1 * n2, q)


def _norm_p(cores, p):
    """TT.norm (tensor_train.py:1334-1420) for p = 1 (sum of entries) or 2."""
    if p == 1:
        v = np.ones((1,))
        for c in cores:
            v = v @ np.sum(c[:, :, 0, :], axis=1)
        return float(v[0])
    return float(np.linalg.norm(full_vector(cores)))


class _TdvpState:
    """Cores, ranks and interface stacks of one TDVP run."""

    def __init__(self, op, x0):
        self.op = op
        self.d = len(op)
        self.cores = [c.copy() for c in x0]
        self.dims = [c.shape[1] for c in op]
        self.sl = [None] * self.d
        self.sr = [None] * self.d

    def r(self, i):
        return self.cores[i].shape[0] if i < self.d else 1

    def left(self, i):                              # sle.py:194-219
        if i == 0:
            self.sl[0] = np.ones((1, 1, 1))
        else:
            self.sl[i] = stack_left_op(self.sl[i - 1], self.cores[i - 1][:, :, 0, :], self.op[i - 1])

    def right(self, i):                             # sle.py:250-276
        if i == self.d - 1:
            self.sr[i] = np.ones((1, 1, 1))
        else:
            self.sr[i] = stack_right_op(self.sr[i + 1], self.cores[i + 1][:, :, 0, :], self.op[i + 1])

    def micro1(self, i):                            # sle.py:308-347
        return micro_matrix(self.sl[i], self.op[i], self.sr[i])

    def micro2(self, i):                            # sle.py:350-390
        return micro_matrix(self.sl[i], _merged_op(self.op[i], self.op[i + 1]), self.sr[i + 1])

    def update1(self, i, mop, tau, direction, kdim):
        """__update_core_tdvp, ode.py:1398-1509 (the backward half sweep is
        always exact there)."""
        c = self.cores
        r1, n, r2 = c[i].shape[0], c[i].shape[1], c[i].shape[3]
        half = 0.5 * tau
        if direction == 'forward':
            if i < self.d - 1:
                x = _expv(mop, c[i].reshape(-1), half, kdim)
                q, r = sla.qr(x.reshape(r1 * n, r2), mode='economic', check_finite=False)
                k = q.shape[1]
                c[i] = q.reshape(r1, n, 1, k)
                qb = np.tensordot(q, np.eye(r2), axes=0).transpose([0, 3, 1, 2]).reshape(r1 * n * r2, k * r2)
                r = _expv(qb.T @ mop @ qb, r.reshape(-1), -half, kdim).reshape(k, r2)
                c[i + 1] = np.tensordot(r, c[i + 1], axes=(1, 0))
            else:
                c[i] = _expv(mop, c[i].reshape(-1), tau, kdim).reshape(r1, n, 1, r2)
        else:
            if i > 0:
                x = c[i].reshape(-1)
                if i < self.d - 1:
                    x = _expv(mop, x, half, 0)
                r, q = sla.rq(x.reshape(r1, n * r2), mode='economic', check_finite=False)
                k = q.shape[0]
                c[i] = q.reshape(k, n, 1, r2)
                qb = np.tensordot(np.eye(r1), q, axes=0).transpose([0, 3, 1, 2]).reshape(r1 * n * r2, r1 * k)
                r = _expv(qb.T @ mop @ qb, r.reshape(-1), -half, 0).reshape(r1, k)
                c[i - 1] = np.tensordot(c[i - 1], r, axes=(3, 0))
            else:
                c[i] = _expv(mop, c[i].reshape(-1), half, 0).reshape(r1, n, 1, r2)

    def update2(self, i, mop, tau, threshold, max_rank, direction, kdim):
        """__update_core_tdvp2site, ode.py:1512-1614."""
        c = self.cores
        half = 0.5 * tau
        ri, ni, nj, rk = c[i].shape[0], self.dims[i], self.dims[i + 1], c[i + 1].shape[3]
        x = np.tensordot(c[i], c[i + 1], axes=1).reshape(-1)
        x = _expv(mop, x, half, kdim)
        u, s, v = truncated_svd(x.reshape(ri * ni, nj * rk), threshold, max_rank)
        k = s.shape[0]
        if direction == 'forward':
            c[i] = u.reshape(ri, ni, 1, k)
            c[i + 1] = (np.diag(s) @ v).reshape(k, nj, 1, rk)
            if i < self.d - 2:
                ub = np.kron(u, np.eye(nj * rk))
                y = _expv(ub.T @ mop @ ub, c[i + 1].reshape(-1), -half, kdim)
                c[i + 1] = y.reshape(k, nj, 1, rk)
        else:
            c[i] = (u @ np.diag(s)).reshape(ri, ni, 1, k)
            c[i + 1] = v.reshape(k, nj, 1, rk)
            if i > 0:
                vb = np.kron(np.eye(ri * ni), v.T)
                y = _expv(vb.T @ mop @ vb, c[i].reshape(-1), -half, kdim)
                c[i] = y.reshape(ri, ni, 1, k)

    def finish_step(self, normalize, states):
        if normalize > 0:
            self.cores = tt_scale(self.cores, 1.0 / _norm_p(self.cores, normalize))
        states.append([x.copy() for x in self.cores])


def tdvp1site(op, x0, tau, steps, kdim=0, normalize=0):
    """ode.py:1188-1288.  tau: real exponent of one full step (-1j * step_size);
    kdim: 0 for local_solver 'exact', else the local Krylov dimension.
    Returns the list of states (initial value first) as core lists."""
    S = _TdvpState(op, x0)
    d = S.d
    for i in range(d - 1, -1, -1):
        S.right(i)
    states = [[x.copy() for x in x0]]
    for _ in range(steps):
        for i in range(d):
            S.left(i)
            S.update1(i, S.micro1(i), tau, 'forward', kdim)
        for i in range(d - 1, -1, -1):
            S.right(i)
            S.update1(i, S.micro1(i), tau, 'backward', kdim)
        S.finish_step(normalize, states)
    return states


def tdvp2site(op, x0, tau, steps, kdim=0, threshold=1e-12, max_rank=50, normalize=0):
    """ode.py:1290-1396 (arguments as tdvp1site)."""
    S = _TdvpState(op, x0)
    d = S.d
    for i in range(d - 1, 0, -1):
        S.right(i)
    states = [[x.copy() for x in x0]]
    for _ in range(steps):
        for i in range(d - 1):
            S.left(i)
            S.update2(i, S.micro2(i), tau, threshold, max_rank, 'forward', kdim)
        for i in range(d - 2, -1, -1):
            S.right(i + 1)
            S.update2(i, S.micro2(i), tau, threshold, max_rank, 'backward', kdim)
        S.finish_step(normalize, states)
    return states


def tdvp_adaptive(op, x0, tau, steps, threshold=1e-12, max_rank=50, normalize=0):
    """ode.py:1076-1186, the adaptive one-/two-site mix.  The reference calls
    its update helpers without their ``local_solver`` argument (a TypeError on
    the first update), so this restates the evident intent: the exact local
    exponential, and every micro matrix built from the current cores (the
    stacks are rebuilt right before each use).  Parity unpinned: there are no
    reference outputs for this function."""
    S = _TdvpState(op, x0)
    d = S.d
    mr = np.inf if max_rank is None else max_rank

    def fresh_left(i):
        for j in range(i + 1):
            S.left(j)

    def fresh_right(i):
        for j in range(d - 1, i - 1, -1):
            S.right(j)

    states = [[x.copy() for x in x0]]
    for _ in range(steps):
        i = 0
        while i < d - 1:
            fresh_left(i)
            if S.r(i + 1) < mr and S.r(i + 1) < min(S.r(i) * S.dims[i], S.dims[i + 1] * S.r(i + 2)):
                fresh_right(i + 1)
                S.update2(i, S.micro2(i), tau, threshold, mr, 'forward', 0)
            else:
                fresh_right(i)
                S.update1(i, S.micro1(i), tau, 'forward', 0)
            i += 1
        while i > 0:
            if S.r(i) < mr and S.r(i) < min(S.r(i - 1) * S.dims[i - 1], S.dims[i] * S.r(i + 1)):
                i -= 1
                fresh_left(i)
                fresh_right(i + 1)
                S.update2(i, S.micro2(i), tau, threshold, mr, 'backward', 0)
            else:
                fresh_left(i)
                fresh_right(i)
                S.update1(i, S.micro1(i), tau, 'backward', 0)
                i -= 1
        S.finish_step(normalize, states)
    return states


# ----------------------------------------------------------------------------
# regression.arr (data_driven/regression.py:15-142, 297-494)
# ----------------------------------------------------------------------------


def arr(theta, y_data, x0s, repeats=1, rcond=1e-2):
    """Alternating ridge regression on pre-evaluated basis values
    ``theta[i]`` (n_i x m, regression.py:323-326); ``x0s``: one core list per
    output row.  Returns the fitted core lists."""
    d = len(theta)
    m = theta[0].shape[1]
    out = []
    for k in range(y_data.shape[0]):
        cores = [c.copy() for c in x0s[k]]
        rhs = y_data[k, :]
        sl, sr = [None] * d, [None] * d

        def left(i):                                     # regression.py:297-327
            if i == 0:
                sl[0] = np.ones((1, m))
            else:
                sl[i] = np.einsum('ij,kj,ikl->lj', sl[i - 1], theta[i - 1], cores[i - 1][:, :, 0, :])

        def right(i):                                    # regression.py:330-361
            if i == d - 1:
                sr[i] = np.ones((1, m))
            else:
                sr[i] = np.einsum('ikl,kj,lj->ij', cores[i + 1][:, :, 0, :], theta[i + 1], sr[i + 1])

        def update(i, direction):                        # regression.py:364-494
            a, n, s = cores[i].shape[0], theta[i].shape[0], cores[i].shape[3]
            phi = np.einsum('ij,kj,lj->iklj', sl[i], theta[i], sr[i]).reshape(a * n * s, m)
            x, _, _, _ = sla.lstsq(phi.T, rhs, cond=rcond, lapack_driver='gelss')
            if direction == 'forward':
                q, _ = sla.qr(x.reshape(a * n, s), mode='economic', check_finite=False)
                cores[i] = q.reshape(a, n, 1, q.shape[1])
            elif i > 0:
                _, q = sla.rq(x.reshape(a, n * s), mode='economic', check_finite=False)
                cores[i] = q.reshape(q.shape[0], n, 1, s)
            else:
                cores[i] = x.reshape(a, n, 1, s)

        for i in range(d - 1, -1, -1):
            right(i)
        for _ in range(repeats):
            for i in range(d):
                left(i)
                if i < d - 1:
                    update(i, 'forward')
            for i in range(d - 1, -1, -1):
                right(i)
                update(i, 'backward')
        out.append(cores)
    return out
