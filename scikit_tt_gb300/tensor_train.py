"""Tensor-train container with the API of ``scikit_tt/tensor_train.py``.

Cores are host NumPy arrays of shape ``(r_i, m_i, n_i, r_{i+1})`` exactly as in
the reference (tensor_train.py:184-188), so a TT built here can be handed to
code written for scikit_tt.  The operations of the ALS hot path run on the
GPU through ``libttals.so``:

* ``__matmul__`` / ``dot``  -- device core products  (tensor_train.py:422-524)
* ``ortho_left`` / ``ortho_right`` / ``ortho`` -- device Householder QR/RQ
  sweeps (tensor_train.py:1092-1332); with ``threshold`` > 0 or a finite
  ``max_rank`` a device one-sided Jacobi SVD per core with the reference's
  rank rule (tensor_train.py:1150-1181, 1262-1296)
* ``norm(p=2)`` -- device QR sweep with a log-carried scale
  (tensor_train.py:1334-1430; immune to the over/underflow the SVD-based
  reference meets on unnormalised trains)

Structural helpers (``+``, ``-``, scalar ``*``, ``transpose``, ``copy``,
``element``, ``full``, ``matricize``, ``tensordot``, ``rank_tensordot``,
``concatenate``, ``rank_transpose``, ``tt2qtt``/``qtt2tt``, ``diag``,
``squeeze``) and ``norm(p=1)`` are block copies, small contractions and sums
and stay in NumPy.  ``svd``/``pinv`` at a bond orthonormalise on the device
and split the bond core (one small matrix) on the host.
"""

from __future__ import annotations

from typing import List, Optional, Union

import numpy as np

from . import _lib


class TT(object):
    """Tensor train (Oseledets 2011) with the attribute set of scikit_tt's TT:
    ``order, row_dims, col_dims, ranks, cores``."""

    def __init__(self, x: Union[List[np.ndarray], np.ndarray], threshold: float = 0, max_rank: int = np.inf,
                 progress: bool = False, string: str = None):
        if isinstance(x, list):
            if all(c.ndim == 4 for c in x):
                if all(x[i].shape[3] == x[i + 1].shape[0] for i in range(len(x) - 1)):
                    self.order = len(x)
                    self.row_dims = [c.shape[1] for c in x]
                    self.col_dims = [c.shape[2] for c in x]
                    self.ranks = [c.shape[0] for c in x] + [x[-1].shape[3]]
                    self.cores = x
                    if threshold != 0 or max_rank != np.inf:
                        self.ortho(threshold=threshold, max_rank=max_rank)
                else:
                    raise ValueError('Shapes of list elements do not match.')
            else:
                raise ValueError('List elements must be 4-dimensional arrays.')
        elif isinstance(x, np.ndarray):
            if x.ndim % 2 != 0:
                raise ValueError('Number of dimensions must be a multiple of 2.')
            self.__init__(_hosvd(x, threshold, max_rank))
        else:
            raise TypeError('Parameter must be either a list of cores or an ndarray.')

    def __repr__(self):
        return ('\n'
                'Tensor train with order    = {d}, \n'
                '                  row_dims = {m}, \n'
                '                  col_dims = {n}, \n'
                '                  ranks    = {r}'.format(d=self.order, m=self.row_dims, n=self.col_dims,
                                                         r=self.ranks))

    # ------------------------------------------------------------------ algebra
    def __add__(self, tt_add: 'TT') -> 'TT':
        if not isinstance(tt_add, TT):
            raise TypeError('Unsupported parameter.')
        if self.row_dims != tt_add.row_dims or self.col_dims != tt_add.col_dims:
            raise ValueError('Tensor trains must have the same dimensions')
        d = self.order
        ranks = [1] + [self.ranks[i] + tt_add.ranks[i] for i in range(1, d)] + [1]
        cores = []
        for i in range(d):
            dt = np.result_type(self.cores[i], tt_add.cores[i])
            c = np.zeros((ranks[i], self.row_dims[i], self.col_dims[i], ranks[i + 1]), dtype=dt)
            c[:self.ranks[i], :, :, :self.ranks[i + 1]] = self.cores[i]
            c[ranks[i] - tt_add.ranks[i]:, :, :, ranks[i + 1] - tt_add.ranks[i + 1]:] = tt_add.cores[i]
            cores.append(c)
        return TT(cores)

    def __sub__(self, tt_sub: 'TT') -> 'TT':
        return self + (-1) * tt_sub.copy()

    def __mul__(self, scalar) -> 'TT':
        out = self.copy()
        if isinstance(scalar, (int, float, complex, np.number)):
            out.cores[0] = scalar * out.cores[0]
        else:
            raise TypeError('Unsupported parameter.')
        return out

    def __rmul__(self, scalar) -> 'TT':
        return self.copy() * scalar

    def __matmul__(self, tt_mul: 'TT'):
        """Core-wise product on the device (tensor_train.py:422-501)."""
        if not isinstance(tt_mul, TT):
            raise TypeError('Unsupported argument.')
        if self.col_dims != tt_mul.row_dims:
            raise ValueError('Dimensions do not match.')
        a, b = _lib.Packed(self.cores), _lib.Packed(tt_mul.cores)
        row, col = list(self.row_dims), list(tt_mul.col_dims)
        ranks = [self.ranks[i] * tt_mul.ranks[i] for i in range(self.order + 1)]
        total = sum(ranks[i] * row[i] * col[i] * ranks[i + 1] for i in range(self.order))
        out = np.empty(total, dtype=np.float64)
        lib = _lib.load()
        _lib.check(lib.ttals_tt_matmul(_lib.context(), a.desc, b.desc, _lib.dptr(out), 0))
        prod = TT(_lib.unpack(out, row, col, ranks))
        if np.prod(prod.row_dims) == 1 and np.prod(prod.col_dims) == 1:
            return prod.element([0] * prod.order * 2)
        return prod

    def dot(self, tt_mul: 'TT'):
        return self.__matmul__(tt_mul)

    def transpose(self, cores: Optional[List[int]] = None, conjugate: bool = False, overwrite: bool = False) -> 'TT':
        if cores is None:
            cores = np.arange(0, self.order)
        t = self.copy() if overwrite is False else self
        for i in range(self.order):
            if np.isin(i, cores):
                t.cores[i] = np.transpose(t.cores[i], [0, 2, 1, 3])
                t.row_dims[i], t.col_dims[i] = t.col_dims[i], t.row_dims[i]
                if conjugate:
                    t.cores[i] = np.conj(t.cores[i])
        return t

    def conj(self, overwrite: bool = False) -> 'TT':
        t = self.copy() if overwrite is False else self
        for i in range(self.order):
            t.cores[i] = np.conj(t.cores[i])
        return t

    def isoperator(self) -> bool:
        return not (all(i == 1 for i in self.row_dims) or all(i == 1 for i in self.col_dims))

    def copy(self) -> 'TT':
        return TT([c.copy() for c in self.cores])

    def element(self, indices: List[int]):
        if not isinstance(indices, list):
            raise TypeError('Unsupported parameter.')
        if not all(isinstance(i, (int, np.integer)) for i in indices):
            raise TypeError('Indices must be integers.')
        if len(indices) != 2 * self.order:
            raise ValueError('Number of indices must be twice the order of the tensor train.')
        d = self.order
        if not (all(i >= 0 for i in indices) and all(indices[i] < self.row_dims[i] for i in range(d))
                and all(indices[d + i] < self.col_dims[i] for i in range(d))):
            raise IndexError('Indices out of range.')
        v = self.cores[0][:, indices[0], indices[d], :].reshape(1, self.ranks[1])
        for i in range(1, d):
            v = v.dot(self.cores[i][:, indices[i], indices[d + i], :].reshape(self.ranks[i], self.ranks[i + 1]))
        return v[0, 0]

    def full(self) -> np.ndarray:
        if self.ranks[0] != 1 or self.ranks[-1] != 1:
            raise ValueError('The first and last rank have to be 1!')
        f = self.cores[0].reshape(self.row_dims[0] * self.col_dims[0], self.ranks[1])
        for i in range(1, self.order):
            f = f.dot(self.cores[i].reshape(self.ranks[i], -1))
            f = f.reshape(-1, self.ranks[i + 1])
        p = [None] * 2 * self.order
        p[::2] = self.row_dims
        p[1::2] = self.col_dims
        q = [2 * i for i in range(self.order)] + [1 + 2 * i for i in range(self.order)]
        return f.reshape(p).transpose(q)

    def matricize(self) -> np.ndarray:
        mat = self.cores[0].reshape(self.row_dims[0], self.col_dims[0], self.ranks[1])
        for i in range(1, self.order):
            mat = np.tensordot(mat, self.cores[i], axes=(2, 0))
            mat = mat.transpose([0, 2, 1, 3, 4]).reshape((int(np.prod(self.row_dims[:i + 1])),
                                                           int(np.prod(self.col_dims[:i + 1])), self.ranks[i + 1]))
        m, n = int(np.prod(self.row_dims)), int(np.prod(self.col_dims))
        return mat.reshape(m) if n == 1 else mat.reshape(m, n)

    # ------------------------------------------------ structural helpers (host)
    def _refresh(self):
        self.order = len(self.cores)
        self.row_dims = [c.shape[1] for c in self.cores]
        self.col_dims = [c.shape[2] for c in self.cores]
        self.ranks = [c.shape[0] for c in self.cores] + [self.cores[-1].shape[3]]
        return self

    def rank_transpose(self, overwrite: bool = False) -> 'TT':
        """The same tensor with the core order reversed and each core's two rank
        axes swapped (tensor_train.py:862-904)."""
        t = self if overwrite else self.copy()
        t.cores = [np.transpose(c, (3, 1, 2, 0)) for c in reversed(t.cores)]
        return t._refresh()

    def rank_tensordot(self, matrix: np.ndarray, mode: str = 'last', overwrite: bool = False) -> 'TT':
        """Contract ``matrix`` into the last rank axis (``t ×_last matrix``) or
        the first (``matrix ×_first t``), tensor_train.py:703-746."""
        if len(matrix.shape) != 2:
            raise ValueError('argument matrix has to be 2D-Array')
        t = self if overwrite else self.copy()
        if mode == 'last':
            if t.ranks[-1] != matrix.shape[0]:
                raise ValueError('dimensions do not match')
            t.cores[-1] = np.einsum('amnb,bc->amnc', t.cores[-1], matrix)
        elif mode == 'first':
            if t.ranks[0] != matrix.shape[1]:
                raise ValueError('dimensions do not match')
            t.cores[0] = np.einsum('ca,amnb->cmnb', matrix, t.cores[0])
        else:
            raise ValueError('unknown mode')
        return t._refresh()

    def concatenate(self, other: Union['TT', List[np.ndarray]], overwrite: bool = False) -> 'TT':
        """Append the cores of ``other`` (a TT or a list of 4-D cores) after the
        last core; the rank between them must agree (tensor_train.py:748-793)."""
        t = self if overwrite else self.copy()
        extra = []
        if isinstance(other, TT):
            extra = other.cores
        elif isinstance(other, list):
            if not all(c.ndim == 4 for c in other):
                raise ValueError('list elements must be 4-dimensional arrays')
            if any(other[i].shape[3] != other[i + 1].shape[0] for i in range(len(other) - 1)):
                raise ValueError('List elements must be 4-dimensional arrays.')
            extra = other
        if extra and t.ranks[-1] != extra[0].shape[0]:
            raise ValueError('ranks do not match!')
        t.cores = list(t.cores) + list(extra)
        return t._refresh()

    def tensordot(self, other: 'TT', num_axes: int, mode: str = 'last-first', overwrite: bool = False) -> 'TT':
        """Contract ``num_axes`` modes at one end of ``self`` with ``num_axes``
        modes at one end of ``other`` (tensor_train.py:526-701).  ``mode`` names
        the ends, ``'<self end>-<other end>'``; the contracted ends must carry
        boundary rank 1.  The result chains what is left of both trains through
        the contracted block: with ``self``'s remainder on the side it came from
        and ``other``'s remainder turned (reversed, ranks swapped) where needed to
        meet it.  The block is absorbed into ``self``'s remainder, or into
        ``other``'s when ``self`` is contracted completely."""
        ends = {'last-first': ('last', 'first'), 'first-last': ('first', 'last'),
                'first-first': ('first', 'first'), 'last-last': ('last', 'last')}
        if mode not in ends:
            raise ValueError('unknown mode')
        k = num_axes
        if k > self.order or k > other.order:
            raise ValueError('num_axes is too big')
        se, oe = ends[mode]
        si = list(range(self.order - k, self.order)) if se == 'last' else list(range(k))
        oi = list(range(other.order - k, other.order)) if oe == 'last' else list(range(k))
        if [self.row_dims[i] for i in si] != [other.row_dims[j] for j in oi] or \
                [self.col_dims[i] for i in si] != [other.col_dims[j] for j in oi]:
            raise ValueError('axes do not match')
        s_bound = self.ranks[-1] if se == 'last' else self.ranks[0]
        o_bound = other.ranks[-1] if oe == 'last' else other.ranks[0]
        if s_bound != 1 or o_bound != 1:
            raise ValueError(f'{se} rank of self and {oe} rank of other have to be 1')
        # block[a, a', b, b']: self's ranks before/after the paired cores, then other's
        block = None
        for i, j in zip(si, oi):
            pair = np.einsum('amnc,bmnd->acbd', self.cores[i], other.cores[j])
            block = pair if block is None else np.einsum('acbd,cedf->aebf', block, pair)
        bridge = block[:, 0] if se == 'last' else block[0]            # (open self rank, b, b')
        bridge = bridge[:, :, 0] if oe == 'last' else bridge[:, 0, :]  # (open self rank, open other rank)

        def turned(cores):
            return [np.transpose(c, (3, 1, 2, 0)) for c in reversed(cores)]

        s_rest = self.cores[:self.order - k] if se == 'last' else self.cores[k:]
        o_rest = other.cores[k:] if oe == 'first' else other.cores[:other.order - k]
        if se == 'last':    # self's remainder on the left, other's open end must face left
            left, right = list(s_rest), list(o_rest) if oe == 'first' else turned(o_rest)
        else:               # self's remainder on the right, other's open end must face right
            left, right = (list(o_rest) if oe == 'last' else turned(o_rest)), list(s_rest)
        if not left and not right:
            cores = [bridge[:, None, None, :]]
        elif s_rest and se == 'last':
            left[-1] = np.einsum('amnb,bc->amnc', left[-1], bridge)
            cores = left + right
        elif s_rest:
            right[0] = np.einsum('bc,bmnd->cmnd', bridge, right[0])
            cores = left + right
        elif se == 'last':  # self used up: absorb into other's first remaining core
            right[0] = np.einsum('ab,bmnd->amnd', bridge, right[0])
            cores = right
        else:
            left[-1] = np.einsum('cmnb,ab->cmna', left[-1], bridge)
            cores = left
        if overwrite:
            self.cores = cores
            return self._refresh()
        return TT(cores)

    def tt2qtt(self, row_dims: List[List[int]], col_dims: List[List[int]], threshold: float = 0) -> 'TT':
        """Split every core's mode into the factors ``row_dims[i]`` x
        ``col_dims[i]`` by successive SVDs (gesvd), singular values with
        sigma_k / sigma_0 <= threshold dropped (tensor_train.py:1432-1516).  A
        format conversion on the host."""
        import scipy.linalg as sla
        out = []
        for i, core in enumerate(self.cores):
            r, right = self.ranks[i], self.ranks[i + 1]
            rest_m, rest_n = self.row_dims[i], self.col_dims[i]
            work = core
            for fm, fn in zip(row_dims[i][:-1], col_dims[i][:-1]):
                rest_m, rest_n = rest_m // fm, rest_n // fn
                mat = work.reshape(r, fm, rest_m, fn, rest_n, right).transpose(0, 1, 3, 2, 4, 5)
                u, s, v = sla.svd(mat.reshape(r * fm * fn, rest_m * rest_n * right), full_matrices=False,
                                  check_finite=False, lapack_driver='gesvd')
                if threshold != 0:
                    keep = np.where(s / s[0] > threshold)[0]
                    u, s, v = u[:, keep], s[keep], v[keep, :]
                out.append(u.reshape(r, fm, fn, s.shape[0]))
                work = s[:, None] * v
                r = s.shape[0]
            out.append(work.reshape(r, rest_m, rest_n, right))
        return TT(out)

    def qtt2tt(self, merge_numbers: List[int]) -> 'TT':
        """Merge groups of ``merge_numbers[k]`` consecutive cores into one core
        each (row and column modes combined, tensor_train.py:1518-1575)."""
        out, k = [], 0
        for cnt in merge_numbers:
            core = self.cores[k].copy()
            for j in range(k + 1, k + cnt):
                nxt = self.cores[j]
                core = np.einsum('amnb,bpqc->ampnqc', core, nxt).reshape(
                    core.shape[0], core.shape[1] * nxt.shape[1], core.shape[2] * nxt.shape[2], nxt.shape[3])
            out.append(core)
            k += cnt
        return TT(out)

    def diag(self, diag_list: List) -> 'TT':
        """Turn the vector cores listed in ``diag_list`` into diagonal operator
        cores, core[k, :, :, l] = diag(core[k, :, 0, l]); those cores are
        complex, as in the reference (tensor_train.py:1719-1747)."""
        cores = list(self.cores)
        for i in diag_list:
            r1, n, _, r2 = cores[i].shape
            dc = np.zeros((r1, n, n, r2), dtype=complex)
            idx = np.arange(n)
            dc[:, idx, idx, :] = cores[i][:, :, 0, :]
            cores[i] = dc
        return TT(cores)

    def squeeze(self) -> 'TT':
        """Drop every mode with row and column dimension 1, multiplying its
        (rank x rank) matrix into the neighbouring kept core: modes before the
        first kept one into it from the left (row 0 of the first boundary rank),
        every other one into the kept core before it (tensor_train.py:1749-1804).
        ``self`` is left unchanged; a train without any kept mode squeezes to a
        single 1 x 1 core."""
        keep = [i for i in range(self.order) if not (self.row_dims[i] == 1 and self.col_dims[i] == 1)]
        mats = [c[:, 0, 0, :] for c in self.cores]
        if not keep:
            v = mats[0][:1, :]
            for mtx in mats[1:]:
                v = v @ mtx
            return TT([v.reshape(1, 1, 1, v.shape[1])])
        cores = []
        for pos, i in enumerate(keep):
            core = self.cores[i]
            if pos == 0 and i > 0:
                lead = mats[0][:1, :]
                for mtx in mats[1:i]:
                    lead = lead @ mtx
                core = np.einsum('ab,bmnc->amnc', lead, core)
            stop = keep[pos + 1] if pos + 1 < len(keep) else self.order
            for j in range(i + 1, stop):
                core = core @ mats[j]
            cores.append(core)
        return TT(cores)

    def svd(self, index: int, threshold: float = 0.0, max_rank: int = np.inf, ortho_l: bool = True,
            ortho_r: bool = True, overwrite: bool = False):
        """SVD of a vector train at bond ``index`` (tensor_train.py:1577-1662):
        cores ``0..index-2`` left- and ``index..d-1`` right-orthonormalised on the
        device (truncated by ``threshold`` / ``max_rank``), then the bond core
        ``index-1`` split by gesvd with the same cut.  Returns ``(u, s, v)``: the
        left train (its last rank is the bond), the singular values, the right
        train."""
        import scipy.linalg as sla
        t = self if overwrite else self.copy()
        if ortho_l:
            t = t.ortho_left(end_index=index - 2, threshold=threshold, max_rank=max_rank)
        if ortho_r:
            t = t.ortho_right(end_index=index, threshold=threshold, max_rank=max_rank)
        a, m, b = t.ranks[index - 1], t.row_dims[index - 1], t.ranks[index]
        u, s, v = sla.svd(t.cores[index - 1].reshape(a * m, b), full_matrices=False, check_finite=False,
                          lapack_driver='gesvd')
        if threshold != 0:
            keep = np.where(s / s[0] > threshold)[0]
            u, s, v = u[:, keep], s[keep], v[keep, :]
        if max_rank != np.inf:
            k = int(min(s.shape[0], max_rank))
            u, s, v = u[:, :k], s[:k], v[:k, :]
        t.cores[index - 1] = u.reshape(a, m, 1, s.shape[0])
        t.cores[index] = np.einsum('kb,bmnc->kmnc', v, t.cores[index])
        t._refresh()
        return TT(t.cores[:index]), s, TT(t.cores[index:])

    def pinv(self, index: int, threshold: float = 0.0, ortho_l: bool = True, ortho_r: bool = True,
             overwrite: bool = False) -> 'TT':
        """Pseudo-inverse at bond ``index`` (tensor_train.py:1664-1717): the
        trains of ``svd`` joined with 1/s in place of s."""
        u, s, v = TT.svd(self, index, threshold=threshold, ortho_l=ortho_l, ortho_r=ortho_r, overwrite=overwrite)
        cores = u.cores + v.cores
        cores[index] = np.einsum('k,kmnc->kmnc', np.reciprocal(s), cores[index])
        return TT(cores)

    # ------------------------------------------------------- orthonormalisation
    def _ortho(self, direction, first, last):
        p = _lib.Packed(self.cores)
        out = np.empty(p.data.size, dtype=np.float64)
        ranks = np.zeros(self.order + 1, dtype=np.int64)
        lib = _lib.load()
        _lib.check(lib.ttals_tt_ortho(_lib.context(), p.desc, direction, first, last, _lib.dptr(out), 0,
                                      _lib.i64ptr(ranks)))
        self.cores = _lib.unpack(out, self.row_dims, self.col_dims, ranks)
        self.ranks = [int(r) for r in ranks]
        return self

    def _ortho_trunc(self, direction, first, last, threshold, max_ranks):
        p = _lib.Packed(self.cores)
        out = np.empty(p.data.size, dtype=np.float64)
        ranks = np.zeros(self.order + 1, dtype=np.int64)
        caps = np.array([0 if m == np.inf else int(m) for m in max_ranks], dtype=np.int64)
        _lib.check(_lib.load().ttals_tt_ortho_trunc(_lib.context(), p.desc, direction, first, last, float(threshold),
                                                    _lib.i64ptr(caps), _lib.dptr(out), 0, _lib.i64ptr(ranks)))
        self.cores = _lib.unpack(out, self.row_dims, self.col_dims, ranks)
        self.ranks = [int(r) for r in ranks]
        return self

    def _check_trunc(self, threshold, max_rank):
        """Validates the truncation arguments as tensor_train.py:1124-1145 does and
        returns the per-bond rank caps, or None when nothing is truncated."""
        if not (isinstance(threshold, (int, float, np.floating, np.integer)) and threshold >= 0):
            raise ValueError('Threshold must be greater or equal 0.')
        if (isinstance(max_rank, (int, np.integer)) and max_rank > 0) or max_rank == np.inf:
            caps = [1] + [max_rank] * (self.order - 1) + [1]
        elif isinstance(max_rank, list) and len(max_rank) == self.order + 1 and \
                all((isinstance(m, (int, np.integer)) and m > 0) or m == np.inf for m in max_rank):
            caps = list(max_rank)
        else:
            raise ValueError('Maximum rank(s) must be positive integers.')
        if threshold == 0 and all(m == np.inf for m in caps[1:-1]):
            return None
        return caps

    def ortho_left(self, start_index: int = 0, end_index: Optional[int] = None, threshold: float = 0.0,
                   max_rank=np.inf, progress: bool = False, string: str = 'Left-orthonormalization') -> 'TT':
        """Left-orthonormalise cores ``start_index..end_index`` (default
        ``0..d-2``, tensor_train.py:1092-1205): device Householder QR, or a
        device SVD per core when ``threshold`` / ``max_rank`` truncate."""
        if end_index is None:
            end_index = self.order - 2
        if not (isinstance(start_index, (int, np.integer)) and isinstance(end_index, (int, np.integer))):
            raise TypeError('Start and end indices must be integers.')
        caps = self._check_trunc(threshold, max_rank)
        if caps is not None:
            return self._ortho_trunc(0, int(start_index), int(end_index), threshold, caps)
        return self._ortho(0, int(start_index), int(end_index))

    def ortho_right(self, start_index: Optional[int] = None, end_index: int = 1, threshold: float = 0,
                    max_rank=np.inf) -> 'TT':
        """Right-orthonormalise cores ``start_index..end_index`` (default
        ``d-1..1``, tensor_train.py:1207-1310): device Householder RQ, or a
        device SVD per core when ``threshold`` / ``max_rank`` truncate."""
        if start_index is None:
            start_index = self.order - 1
        if not (isinstance(start_index, (int, np.integer)) and isinstance(end_index, (int, np.integer))):
            raise TypeError('Start and end indices must be integers.')
        caps = self._check_trunc(threshold, max_rank)
        if caps is not None:
            return self._ortho_trunc(1, int(start_index), int(end_index), threshold, caps)
        return self._ortho(1, int(start_index), int(end_index))

    def ortho(self, threshold: float = 0, max_rank=np.inf) -> 'TT':
        self.ortho_left(threshold=threshold).ortho_right(threshold=threshold, max_rank=max_rank)
        return self

    def norm(self, p: int = 2) -> float:
        """p=2: Euclidean / Frobenius norm on the device (tensor_train.py:1404-1425).
        p=1: Manhattan norm / maximum column sum for non-negative entries."""
        if p == 1:
            t = self.copy()
            if all(i == 1 for i in self.row_dims):
                t = t.transpose()
            t.cores = [np.sum(t.cores[i], axis=1).reshape(t.ranks[i], 1, t.col_dims[i], t.ranks[i + 1])
                       for i in range(t.order)]
            t.row_dims = [1] * t.order
            return np.max(t.matricize())
        if p == 2:
            cores = self.cores
            if self.isoperator():
                cores = [c.reshape(c.shape[0], c.shape[1] * c.shape[2], 1, c.shape[3]) for c in cores]
            pk = _lib.Packed(cores)
            out = np.zeros(1, dtype=np.float64)
            _lib.check(_lib.load().ttals_tt_norm(_lib.context(), pk.desc, _lib.dptr(out)))
            return float(out[0])
        raise ValueError('p must be 1 or 2.')


def _hosvd(x, threshold, max_rank):
    """Sequential SVD of a full array into TT cores (tensor_train.py:201-264);
    input conversion only, not part of the ALS path."""
    order = x.ndim // 2
    row_dims, col_dims = x.shape[:order], x.shape[order:]
    ranks = [1] * (order + 1)
    cores = []
    p = [order * j + i for i in range(order) for j in range(2)]
    y = np.transpose(x, p).copy()
    for i in range(order - 1):
        m = ranks[i] * row_dims[i] * col_dims[i]
        y = y.reshape(m, -1)
        u, s, v = np.linalg.svd(y, full_matrices=False)
        if threshold != 0:
            keep = np.where(s / s[0] > threshold)[0]
            u, s, v = u[:, keep], s[keep], v[keep, :]
        if max_rank != np.inf:
            k = int(min(u.shape[1], max_rank))
            u, s, v = u[:, :k], s[:k], v[:k, :]
        ranks[i + 1] = u.shape[1]
        cores.append(u.reshape(ranks[i], row_dims[i], col_dims[i], ranks[i + 1]))
        y = np.diag(s).dot(v)
    cores.append(y.reshape(ranks[-2], row_dims[-1], col_dims[-1], 1))
    return cores


# ---------------------------------------------------------------------------
# constructors (tensor_train.py:1806-2032)
# ---------------------------------------------------------------------------

def _rank_list(ranks, d):
    return ranks if isinstance(ranks, list) else [1] + [ranks] * (d - 1) + [1]


def zeros(row_dims, col_dims, ranks=1) -> TT:
    r = _rank_list(ranks, len(row_dims))
    return TT([np.zeros([r[i], row_dims[i], col_dims[i], r[i + 1]]) for i in range(len(row_dims))])


def ones(row_dims, col_dims, ranks=1) -> TT:
    r = _rank_list(ranks, len(row_dims))
    return TT([np.ones([r[i], row_dims[i], col_dims[i], r[i + 1]]) for i in range(len(row_dims))])


def eye(dims) -> TT:
    cores = [np.zeros([1, d, d, 1]) for d in dims]
    for i, d in enumerate(dims):
        cores[i][0, :, :, 0] = np.eye(d)
    return TT(cores)


def unit(dims, inds) -> TT:
    t = zeros(dims, [1] * len(dims))
    for i in range(t.order):
        t.cores[i][0, inds[i], 0, 0] = 1
    return t


def rand(row_dims, col_dims, ranks=1) -> TT:
    """Random TT with U[0,1) cores drawn from NumPy's global generator, in core
    order (tensor_train.py:1921-1950)."""
    r = _rank_list(ranks, len(row_dims))
    return TT([np.random.rand(r[i], row_dims[i], col_dims[i], r[i + 1]) for i in range(len(row_dims))])


def canonical(row_dims, max_rank) -> TT:
    order = len(row_dims)
    cores = [None] * order
    rl = 1
    for i in range(order // 2):
        k = min(rl * row_dims[i], max_rank)
        cores[i] = np.eye(rl * row_dims[i], k).reshape(rl, row_dims[i], 1, k)
        rl = k
    rr = 1
    for i in range(order // 2):
        k = min(rr * row_dims[-i - 1], max_rank)
        cores[-i - 1] = np.eye(k, row_dims[-i - 1] * rr).reshape(k, row_dims[-i - 1], 1, rr)
        rr = k
    if order % 2 == 1:
        cores[order // 2] = np.eye(rl * row_dims[order // 2], rr).reshape(rl, row_dims[order // 2], 1, rr)
    return TT(cores)


def uniform(row_dims, ranks=1, norm: float = 1) -> TT:
    r = _rank_list(ranks, len(row_dims))
    factor = (norm / (np.sqrt(np.prod(row_dims)) * np.prod(r))) ** np.true_divide(1, len(row_dims))
    return TT([factor * np.ones([r[i], row_dims[i], 1, r[i + 1]]) for i in range(len(row_dims))])


def residual_error(operator: TT, lhs: TT, rhs: TT) -> float:
    """``||operator @ lhs - rhs||`` (tensor_train.py:2035-2074), computed on the
    device as the norm of the rank-summed train ``A@x - b``."""
    ax = operator.dot(lhs)
    return (ax - rhs).norm()


def build_core(matrix_list, iscomplex: bool = False) -> np.ndarray:
    """Operator/vector core from a (nested) list of matrices or zeros
    (tensor_train.py:2144-2262)."""
    if isinstance(matrix_list[0], (np.ndarray, int)):
        mats = [[e] for e in matrix_list]
    else:
        mats = matrix_list
    r1, r2 = len(mats), len(mats[0])
    shape = None
    for row in mats:
        if len(row) != r2:
            raise ValueError('All lists must contain the same number of matrices.\n')
        for e in row:
            if isinstance(e, np.ndarray):
                shape = (e.shape[0], 1) if e.ndim == 1 else e.shape
    cplx = iscomplex or any(isinstance(e, np.ndarray) and np.iscomplexobj(e) for row in mats for e in row)
    core = np.zeros((r1, shape[0], shape[1], r2), dtype=complex if cplx else float)
    for i in range(r1):
        for j in range(r2):
            e = mats[i][j]
            if isinstance(e, np.ndarray):
                core[i, :, :, j] = e.reshape(shape)
            elif e != 0:
                raise TypeError('Parameters in list must be either an 0 or a matrix.\n')
    return core


def build_core_vector(matrix_list, field_type: str = 'float') -> np.ndarray:
    """Column core (r, m, n, 1) from a flat list of matrices, vectors (n = 1) or
    zeros (tensor_train.py:2076-2142).  With ``field_type='complex'`` the
    reference leaves every entry zero (it skips the copy); here the matrices
    are copied in both cases."""
    shape = None
    for e in matrix_list:
        if isinstance(e, np.ndarray):
            shape = (e.shape[0], 1) if e.ndim == 1 else e.shape
            break
    core = np.zeros((len(matrix_list), shape[0], shape[1], 1), dtype=field_type)
    for i, e in enumerate(matrix_list):
        if isinstance(e, np.ndarray):
            core[i, :, :, 0] = e.reshape(shape)
    return core
