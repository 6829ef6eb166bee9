"""The rest of the TT container against the reference's own results
(``tests/golden/ttops_container.npz``, made by ``make_golden.py container``):
``tensordot`` in its four modes (partial and complete contractions and a
mismatch), ``rank_tensordot``, ``concatenate``, ``rank_transpose``,
``tt2qtt`` / ``qtt2tt``, ``diag``, ``squeeze``, ``build_core_vector``
(tensor_train.py:526-904, 1432-1804, 2076-2142), all host operations; and
``svd`` / ``pinv`` (1577-1717), whose orthonormalisation sweeps run on the
device and are replaced here by host SVD sweeps over the same core ranges."""

import numpy as np
import pytest

from scikit_tt_gb300 import tensor_train as tt
from scikit_tt_gb300.tensor_train import TT

RT = dict(rtol=1e-12, atol=1e-12)


def _t(cores):
    return TT([c.copy() for c in cores])


TD_CASES = {'lf2': ('a', 'b', 2, 'last-first'), 'fl1': ('b', 'a', 1, 'first-last'),
            'ff2': ('a', 'c', 2, 'first-first'), 'll1': ('a', 'c', 1, 'last-last'),
            'ff_full_self': ('c', 'a', 3, 'first-first'), 'lf_full_self': ('e', 'a', 1, 'last-first'),
            'fl_full_self': ('e', 'a', 1, 'first-last'), 'll_full_self': ('e', 'a', 1, 'last-last'),
            'full_both': ('a', 'a', 4, 'last-first')}


@pytest.mark.parametrize('key', sorted(TD_CASES))
def test_tensordot(golden, key):
    z, cores = golden('ttops_container')
    s, o, k, mode = TD_CASES[key]
    res = _t(cores(s)).tensordot(_t(cores(o)), k, mode=mode)
    ref = [z[f'td_{key}_cores_{i}'] for i in range(int(z[f'td_{key}_cores_n']))]
    assert res.order == len(ref)
    for c, r in zip(res.cores, ref):
        assert c.shape == r.shape
        np.testing.assert_allclose(c, r, **RT)


def test_tensordot_errors(golden):
    z, cores = golden('ttops_container')
    with pytest.raises(ValueError, match='axes do not match'):
        _t(cores('a')).tensordot(_t(cores('b')), 1, mode='last-last')
    assert 'axes do not match' in str(z['td_bad_error'])
    with pytest.raises(ValueError):
        _t(cores('a')).tensordot(_t(cores('b')), 1, mode='middle')
    with pytest.raises(ValueError):
        _t(cores('e')).tensordot(_t(cores('a')), 2, mode='last-first')


def test_rank_ops_and_concatenate(golden):
    z, cores = golden('ttops_container')
    a = _t(cores('a'))
    last = a.rank_tensordot(z['m_last'], mode='last')
    np.testing.assert_allclose(last.cores[-1], z['rtd_last'], **RT)
    assert last.ranks[-1] == 3 and a.ranks[-1] == 1          # a copy unless overwrite=True
    np.testing.assert_allclose(a.rank_tensordot(z['m_first'], mode='first').cores[0], z['rtd_first'], **RT)
    with pytest.raises(ValueError):
        a.rank_tensordot(np.ones((2, 2)), mode='last')
    with pytest.raises(ValueError):
        a.rank_tensordot(np.ones((2, 2)), mode='side')
    cat = _t(cores('a')).concatenate(_t(cores('b')))
    assert cat.order == 7
    np.testing.assert_allclose(cat.full().reshape(-1), z['cat_full'], **RT)
    with pytest.raises(ValueError):
        _t(cores('a')).concatenate([np.ones((2, 2, 1, 1))])
    np.testing.assert_allclose(_t(cores('a')).rank_transpose().full().reshape(-1), z['rtr_full'], **RT)


def test_qtt_round_trip(golden):
    z, cores = golden('ttops_container')
    q = _t(cores('q'))
    rows, cols = [[2, 2], [2, 3], [2]], [[1, 2], [1, 1], [2, 2]]
    qt = q.tt2qtt(rows, cols)
    assert qt.ranks == [int(r) for r in z['qtt_ranks']]
    np.testing.assert_allclose(qt.full().reshape(-1), z['qtt_full'], **RT)
    qt2 = _t(cores('q')).tt2qtt(rows, cols, threshold=0.6)
    assert qt2.ranks == [int(r) for r in z['qtt_thr_ranks']]
    np.testing.assert_allclose(qt2.full().reshape(-1), z['qtt_thr_full'], **RT)
    back = qt.qtt2tt([2, 2, 1])
    assert back.row_dims == [int(r) for r in z['back_rows']]
    np.testing.assert_allclose(back.full().reshape(-1), z['back_full'], **RT)


def test_diag_squeeze_build_core_vector(golden):
    z, cores = golden('ttops_container')
    dg = _t(cores('a')).diag([0, 2])
    assert np.iscomplexobj(dg.cores[0]) and not np.iscomplexobj(dg.cores[1])
    np.testing.assert_allclose(dg.full().reshape(-1), z['diag_full'], **RT)
    src = _t(cores('sq'))
    sq = src.squeeze()
    assert sq.row_dims == [int(r) for r in z['sq_rows']]
    np.testing.assert_allclose(sq.full().reshape(-1), z['sq_full'], **RT)
    assert src.order == 5                       # the input is left as it was
    np.testing.assert_array_equal(tt.build_core_vector([np.arange(4.0).reshape(2, 2), 0, np.eye(2)]), z['bcv'])
    np.testing.assert_array_equal(tt.build_core_vector([np.arange(3.0), 0]), z['bcv_vec'])


@pytest.fixture
def host_sweeps(monkeypatch):
    """Host SVD sweeps over the core ranges the device orthonormalisation gets."""

    def sweep(self, direction, first, last, threshold=0.0, caps=None):
        cores = [c.copy() for c in self.cores]
        d = len(cores)

        def keep(sv, cap):
            k = int(np.sum(sv / sv[0] > threshold)) if threshold else len(sv)
            return min(k, int(cap)) if cap not in (None, np.inf) else k

        if direction == 0:
            for i in range(max(0, first), min(last, d - 2) + 1):
                r, m, n, s = cores[i].shape
                u, sv, v = np.linalg.svd(cores[i].reshape(r * m * n, s), full_matrices=False)
                k = keep(sv, caps[i + 1] if caps else None)
                cores[i] = u[:, :k].reshape(r, m, n, k)
                cores[i + 1] = np.einsum('kb,bmnc->kmnc', sv[:k, None] * v[:k], cores[i + 1])
        else:
            for i in range(min(first, d - 1), max(last, 1) - 1, -1):
                r, m, n, s = cores[i].shape
                u, sv, v = np.linalg.svd(cores[i].reshape(r, m * n * s), full_matrices=False)
                k = keep(sv, caps[i] if caps else None)
                cores[i] = v[:k].reshape(k, m, n, s)
                cores[i - 1] = np.einsum('amnb,bk->amnk', cores[i - 1], u[:, :k] * sv[:k])
        self.cores = cores
        return self._refresh()

    monkeypatch.setattr(TT, '_ortho', lambda self, dr, f, l_: sweep(self, dr, f, l_))
    monkeypatch.setattr(TT, '_ortho_trunc', lambda self, dr, f, l_, thr, caps: sweep(self, dr, f, l_, thr, caps))


def test_svd_and_pinv(golden, host_sweeps):
    z, cores = golden('ttops_container')
    u, s, v = _t(cores('v')).svd(2)
    np.testing.assert_allclose(s, z['svd_s'], **RT)
    um = np.tensordot(u.cores[0], u.cores[1], axes=(3, 0)).reshape(-1, u.ranks[-1])
    ref = z['svd_u_full']
    signs = np.sign(np.sum(um * ref, axis=0))
    np.testing.assert_allclose(um * signs, ref, rtol=1e-10, atol=1e-10)
    full = _t(cores('v')).full().reshape(-1)
    rec = (um * s) @ np.tensordot(v.cores[0], v.cores[1], axes=(3, 0)).reshape(len(s), -1)
    np.testing.assert_allclose(rec.reshape(-1), full, rtol=1e-10, atol=1e-10)
    _, s2, _ = _t(cores('v')).svd(2, max_rank=2)
    np.testing.assert_allclose(s2, z['svd_s_r2'], **RT)
    np.testing.assert_allclose(_t(cores('v')).pinv(2).full().reshape(-1), z['pinv_full'], rtol=1e-10, atol=1e-10)
