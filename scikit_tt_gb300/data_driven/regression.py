"""Alternating ridge regression on the device (scikit_tt/data_driven/regression.py:15-142).

``arr(x_data, y_data, basis_list, initial_guess, repeats, rcond, string,
progress)`` keeps the reference's signature and result: a list with one TT
per row of ``y_data``.  The basis functions are evaluated on the samples on
the host exactly as the reference does (regression.py:323-326, once per mode
here instead of at every stack update); all sweeps -- stacks, micro matrices,
the ``lstsq(..., cond=rcond, lapack_driver='gelss')`` fits and the QR/RQ
re-gauging -- run in one engine call (``ttals_arr``).  When ``initial_guess``
is a list, its trains are updated in place and the same list is returned, as
in the reference.  ``progress`` is accepted and ignored.
"""

from __future__ import annotations

from typing import List

import numpy as np

from .. import _lib
from ..tensor_train import TT

last_stats = {}


def evaluate_basis(x_data: np.ndarray, basis_list) -> List[np.ndarray]:
    """theta_i[k, j] = basis_list[i][k](x_data[:, j]) for every mode i."""
    m = x_data.shape[1]
    return [np.array([[f(x_data[:, j]) for j in range(m)] for f in funcs], dtype=np.float64) for funcs in basis_list]


def arr(x_data: np.ndarray, y_data: np.ndarray, basis_list, initial_guess, repeats: int = 1, rcond: float = 10 ** -2,
        string: str = 'ARR', progress=True):
    """Alternating ridge regression (regression.py:15-142)."""
    global last_stats
    order = len(basis_list)
    y_data = np.asarray(y_data, dtype=np.float64)
    if isinstance(initial_guess, list):
        solution = initial_guess
    else:
        solution = [initial_guess.copy() for _ in range(y_data.shape[0])]
    if len(solution) != y_data.shape[0]:
        raise ValueError('one initial guess per row of y_data is needed')
    theta = evaluate_basis(np.asarray(x_data), basis_list)
    m = theta[0].shape[1] if order else 0
    nb = np.array([t.shape[0] for t in theta], dtype=np.int64)
    flat_theta = np.ascontiguousarray(np.concatenate([t.ravel() for t in theta]))
    ys = np.ascontiguousarray(y_data.reshape(y_data.shape[0], -1))
    packs = [_lib.Packed(t.cores) for t in solution]
    descs = (_lib.TTDesc * len(packs))(*[p.desc for p in packs])
    cap = sum(int(p.data.size) for p in packs)
    out = np.empty(max(cap, 1))
    out_ranks = np.zeros(len(packs) * (order + 1), dtype=np.int64)
    st = _lib.Stats()
    _lib.check(_lib.load().ttals_arr(_lib.context(), order, _lib.i64ptr(nb), m, _lib.dptr(flat_theta), len(packs),
                                     _lib.dptr(ys), descs, int(repeats), float(rcond), _lib.dptr(out), out.size,
                                     _lib.i64ptr(out_ranks), st))
    last_stats = st.as_dict()
    off = 0
    dims = [int(v) for v in nb]
    for k, t in enumerate(solution):
        rk = out_ranks[k * (order + 1):(k + 1) * (order + 1)]
        cores = _lib.unpack(out[off:], dims, [1] * order, rk)
        off += sum(int(rk[i] * dims[i] * rk[i + 1]) for i in range(order))
        t.cores = cores
        t.ranks = [int(v) for v in rk]
        t.row_dims = dims
        t.col_dims = [1] * order
    return solution
