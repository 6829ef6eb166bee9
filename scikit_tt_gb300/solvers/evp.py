"""Alternating linear scheme for eigenproblems in the TT format, on the GPU.

Drop-in for ``scikit_tt/solvers/evp.py``: ``als`` keeps its signature
(evp.py:17-27) and return convention ``(eigenvalue(s), eigentensor(s),
iterations)``.  The sweep runs in ``libttals.so`` (``ttals_evp_als``): the
local eigenproblem is solved matrix-free by Lanczos with full
reorthogonalisation (symmetric operators) or Arnoldi with Francis-QR Ritz
values (operators with nonsymmetric cores, ``'eig'`` / ``'eigs'``), and the
eigenvalues are selected by the reference's rule for ``solver`` -- the
``number_ev`` largest, descending, for ``'eigh'`` (evp.py:434-439); the
``number_ev`` closest to ``sigma`` for ``'eig'`` (ascending distance,
evp.py:423-432) and ``'eigs'`` (descending distance, evp.py:414-421).  With
``number_ev > 1`` the eigenvector block is re-gauged to its ``r`` leading
singular directions as in evp.py:455-486, and the last sweep's eigenvalues and
eigentensors are returned (evp.py:170-177).

Implemented: ``number_ev`` 1..8, ``previous`` / ``shift`` deflation,
``operator_gevp`` equal to the identity train, and generalised problems
``A x = lambda B x`` with a symmetric operator and a symmetric positive
definite ``operator_gevp`` (``number_ev == 1``, no ``previous``): those run as
one request of the batched engine (``ttals_solve_batch``, request kind
``TTALS_REQ_GEVP``), whose local solver is Lanczos on ``B^{-1} A`` in the B
inner product with FP64 GMRES solves for ``B^{-1}`` (evp.py:272-287,
314-329, 367-368 and the ``b=`` / ``M=`` local solves of evp.py:410-439).
Other generalised problems, ``'eigh'`` on a nonsymmetric operator and wanted
eigenvalues with a nonzero imaginary part raise ``NotImplementedError``.
"""

from __future__ import annotations

from typing import List

import numpy as np

from .. import _lib
from ..tensor_train import TT

last_stats = {}


def _is_identity(op: TT) -> bool:
    if op is None:
        return True
    return all(c.shape[0] == 1 and c.shape[3] == 1 and c.shape[1] == c.shape[2]
               and np.array_equal(c[0, :, :, 0], np.eye(c.shape[1])) for c in op.cores)


def _host_norm(cores) -> float:
    """Frobenius norm of a TT operator by a left-to-right QR sweep on the host
    (argument validation: operator cores are small), scale carried in logs."""
    carry, logs = np.ones((1, 1)), 0.0
    for c in cores:
        m = np.tensordot(carry, c.reshape(c.shape[0], -1, c.shape[3]), axes=(1, 0))
        m = m.reshape(-1, c.shape[3])
        r = np.linalg.qr(m, mode='r')
        sc = np.linalg.norm(r)
        if sc == 0:
            return 0.0
        logs += np.log(sc)
        carry = r / sc
    return float(np.exp(logs) * np.linalg.norm(carry))


def _is_symmetric(op: TT) -> bool:
    """Core-wise symmetric cores, or a globally symmetric operator such as the
    rank-sum 0.5 (A + A^T): ||A - A^T|| <= 1e-12 ||A|| (host norms).  The
    local operators of a symmetric operator in orthonormal frames are
    symmetric, which is what the Lanczos eigensolver needs."""
    if all(np.allclose(c, np.transpose(c, (0, 2, 1, 3)), rtol=0, atol=1e-14 * max(1.0, np.abs(c).max()))
           for c in op.cores):
        return True
    if op.row_dims != op.col_dims:
        return False
    nrm = _host_norm(op.cores)
    return nrm > 0 and _host_norm((op - op.transpose()).cores) <= 1e-12 * nrm


def _gevp_als(operator, initial_guess, operator_gevp, repeats, conv_eps, solver, sigma):
    """Generalised symmetric-definite problem through the batched engine (one
    request on one CTA, FP64).  Returns the reference's ``(eigenvalue,
    eigentensor, iterations)`` for ``number_ev == 1``."""
    global last_stats
    lib = _lib.load()
    op, x0, og = _lib.Packed(operator.cores), _lib.Packed(initial_guess.cores), _lib.Packed(operator_gevp.cores)
    dims = np.array(operator.row_dims, dtype=np.int64)
    ranks = np.zeros(operator.order + 1, dtype=np.int64)
    _lib.check(lib.ttals_als_ranks(operator.order, _lib.i64ptr(dims), _lib.i64ptr(x0.ranks), _lib.i64ptr(ranks)))
    out = np.empty(max(1, int(sum(ranks[i] * dims[i] * ranks[i + 1] for i in range(operator.order)))))
    val = np.zeros(1)
    its = np.zeros(1, dtype=np.int32)
    r = _lib.Request()
    r.kind = _lib.REQ_GEVP
    r.op, r.x0, r.rhs = op.desc, x0.desc, og.desc
    r.repeats = int(repeats)
    r.solver = _lib.EVP_SOLVERS[solver]
    r.sigma = float(sigma)
    r.conv_eps = float(conv_eps)
    r.out_data = _lib.dptr(out)
    r.out_value = _lib.dptr(val)
    r.out_iterations = its.ctypes.data_as(_lib.C.POINTER(_lib.C.c_int32))
    arr = (_lib.Request * 1)(r)
    st = _lib.Stats()
    _lib.check(lib.ttals_solve_batch(_lib.context(), 1, arr, _lib.PREC_FP64, 0.0, 0, st))
    last_stats = st.as_dict()
    cores = _lib.unpack(out, operator.row_dims, [1] * operator.order, ranks)
    return np.float64(val[0]), TT(cores), int(its[0])


def als(operator: 'TT', initial_guess: 'TT', previous: List['TT'] = [], shift: float = 0,
        operator_gevp: 'TT' = None, number_ev: int = 1, repeats: int = 1, conv_eps: float = 1e-10,
        solver: str = 'eig', sigma: float = 1, real: bool = True):
    """ALS eigensolver with the signature of evp.py:17-27."""
    global last_stats
    if solver not in _lib.EVP_SOLVERS:
        raise ValueError("solver must be 'eig', 'eigs' or 'eigh'")
    if not _is_identity(operator_gevp):
        if operator_gevp.row_dims != operator.row_dims or operator_gevp.col_dims != operator.col_dims:
            raise ValueError('operator_gevp must have the dimensions of operator')
        if number_ev != 1 or len(previous) > 0:
            raise NotImplementedError('generalised eigenproblems support number_ev == 1 without previous on the '
                                      'device path')
        if not (_is_symmetric(operator) and _is_symmetric(operator_gevp)):
            raise NotImplementedError('generalised eigenproblems need a symmetric operator and a symmetric '
                                      'positive definite operator_gevp on the device path')
        if repeats < 1:
            return np.inf, None, 0
        return _gevp_als(operator, initial_guess, operator_gevp, repeats, conv_eps, solver, sigma)
    if solver == 'eigh' and not _is_symmetric(operator):
        raise NotImplementedError("solver='eigh' needs a symmetric operator")
    if not 1 <= number_ev <= 8:
        raise NotImplementedError('number_ev must be between 1 and 8 on the device path')
    op, x0 = _lib.Packed(operator.cores), _lib.Packed(initial_guess.cores)
    prev = [_lib.Packed(p.cores) for p in previous]
    prev_arr = (_lib.TTDesc * max(1, len(prev)))(*[p.desc for p in prev]) if prev else None
    lib = _lib.load()
    dims = np.array(operator.row_dims, dtype=np.int64)
    ranks = np.zeros(operator.order + 1, dtype=np.int64)
    _lib.check(lib.ttals_als_ranks(operator.order, _lib.i64ptr(dims), _lib.i64ptr(x0.ranks), _lib.i64ptr(ranks)))
    sizes = [int(max(ranks[i], x0.ranks[i]) * dims[i] * max(ranks[i + 1], x0.ranks[i + 1]))
             for i in range(operator.order)]
    total = sum(sizes) + (number_ev - 1) * sizes[0]
    out = np.empty(max(total, 1), dtype=np.float64)
    out_ranks = np.zeros(operator.order + 1, dtype=np.int64)
    vals = np.zeros(max(1, number_ev), dtype=np.float64)
    its = _lib.C.c_int32(0)
    st = _lib.Stats()
    code = lib.ttals_evp_als(_lib.context(), op.desc, x0.desc, len(prev), prev_arr, float(shift),
                             int(number_ev), int(repeats), float(conv_eps), _lib.EVP_SOLVERS[solver],
                             float(sigma), _lib.PREC_FP64, 0.0, _lib.dptr(vals), _lib.dptr(out), 0,
                             _lib.i64ptr(out_ranks), _lib.C.byref(its), st)
    _lib.check(code)
    last_stats = st.as_dict()
    if repeats < 1:
        return np.inf, None, 0
    if number_ev == 1:
        cores = _lib.unpack(out, operator.row_dims, [1] * operator.order, out_ranks)
        return np.float64(vals[0]), TT(cores), int(its.value)
    # first core holds the number_ev variants as (r0, n0, 1, r1, number_ev)
    r0, n0, r1 = int(out_ranks[0]), operator.row_dims[0], int(out_ranks[1])
    c0 = out[:r0 * n0 * r1 * number_ev].reshape(r0, n0, 1, r1, number_ev)
    rest = _lib.unpack(out[r0 * n0 * r1 * number_ev:], operator.row_dims[1:], [1] * (operator.order - 1),
                       out_ranks[1:])
    tts = [TT([c0[:, :, :, :, e].copy()] + [c.copy() for c in rest]) for e in range(number_ev)]
    return vals[:number_ev].copy(), tts, int(its.value)


def power_method(operator: 'TT', initial_guess: 'TT', operator_gevp: 'TT' = None, repeats: int = 10,
                 sigma: float = 0.999):
    """Inverse power iteration (evp.py:182-250) on the device engine.

    Each step solves ``(operator - sigma * operator_gevp) x_new = operator_gevp x``
    with the device ``sle.als`` (one sweep, the current iterate as initial
    guess), normalises with the device ``TT.norm`` and returns the Rayleigh
    quotient ``x^T A x (/ x^T M x)`` of the last iterate, as the reference does."""
    from .. import tensor_train as tt
    from . import sle
    if operator_gevp is None:
        operator_shift = operator - sigma * tt.eye(operator.row_dims)
    else:
        operator_shift = operator - sigma * operator_gevp
    eigenvalue = 0
    eigentensor = initial_guess
    for _ in range(repeats):
        if operator_gevp is None:
            eigentensor = sle.als(operator_shift, eigentensor, eigentensor)
        else:
            eigentensor = sle.als(operator_shift, eigentensor, operator_gevp.dot(eigentensor))
        eigentensor = eigentensor * (1 / eigentensor.norm())
        eigenvalue = eigentensor.transpose().dot(operator).dot(eigentensor)
        if operator_gevp is not None:
            eigenvalue *= 1 / (eigentensor.transpose().dot(operator_gevp).dot(eigentensor))
    return eigenvalue, eigentensor
