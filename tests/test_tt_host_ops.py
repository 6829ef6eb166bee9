"""The TT container's host-side helpers against the reference's own results
(``tests/golden/ttops_struct.npz``, made by ``make_golden.py struct``): rank-sum
``+``/``-`` and scalar products (tensor_train.py:282-420), transposes
(795-870), ``element`` (966-1027), ``full``/``matricize`` (1029-1090),
``norm(p=1)`` (1334-1403), the HOSVD constructor (201-264) and the
constructors eye/ones/unit/canonical/uniform/build_core (1806-2032,
2144-2262).  None of these touch the device."""

import numpy as np

from scikit_tt_gb300 import tensor_train as tt
from scikit_tt_gb300.tensor_train import TT

RT = dict(rtol=1e-12, atol=1e-12)


def test_algebra_and_access(golden):
    z, cores = golden('ttops_struct')
    T, U, A = TT(cores('t')), TT(cores('u')), TT(cores('A'))
    s = T + U
    assert s.ranks == [int(r) for r in z['add_ranks']]
    np.testing.assert_allclose(s.full().reshape(-1), z['add_full'], **RT)
    np.testing.assert_allclose((T - U).full().reshape(-1), z['sub_full'], **RT)
    np.testing.assert_allclose((2.5 * T).full().reshape(-1), z['rmul_full'], **RT)
    np.testing.assert_allclose((T * -0.75).full().reshape(-1), z['mul_full'], **RT)
    np.testing.assert_allclose(A.copy().transpose().full().reshape(-1), z['tr_full'], **RT)
    np.testing.assert_allclose(A.copy().transpose(cores=[0, 2]).full().reshape(-1), z['tr_part_full'], **RT)
    np.testing.assert_allclose(A.matricize(), z['mat_A'], **RT)
    np.testing.assert_allclose(T.matricize(), z['mat_t'], **RT)
    assert abs(A.element([1, 2, 0, 1, 2, 1, 1, 0]) - float(z['elem_A'])) < 1e-12
    assert abs(T.element([1, 0, 1, 2, 0, 0, 0, 0]) - float(z['elem_t'])) < 1e-12
    assert abs(TT(cores('P')).norm(p=1) - float(z['norm1_P'])) < 1e-12 * float(z['norm1_P'])
    assert abs(TT(cores('Q')).norm(p=1) - float(z['norm1_Q'])) < 1e-12 * float(z['norm1_Q'])


def test_hosvd_constructor(golden):
    z, cores = golden('ttops_struct')
    full8 = (TT(cores('t')) + TT(cores('u'))).full()
    h_thr, h_max = TT(full8.copy(), threshold=1e-10), TT(full8.copy(), max_rank=2)
    assert h_thr.ranks == [int(r) for r in z['hosvd_thr_ranks']]
    assert h_max.ranks == [int(r) for r in z['hosvd_max_ranks']]
    np.testing.assert_allclose(h_thr.full().reshape(-1), z['hosvd_thr_full'], **RT)
    np.testing.assert_allclose(h_max.full().reshape(-1), z['hosvd_max_full'], **RT)


def test_constructors(golden):
    z, cores = golden('ttops_struct')
    L = z['L']
    np.testing.assert_allclose(tt.eye([2, 3]).full().reshape(-1), z['eye_full'], **RT)
    np.testing.assert_allclose(tt.ones([2, 3], [1, 2], ranks=2).full().reshape(-1), z['ones_full'], **RT)
    np.testing.assert_allclose(tt.unit([2, 3, 2], [1, 2, 0]).full().reshape(-1), z['unit_full'], **RT)
    np.testing.assert_allclose(tt.canonical([2, 3, 2, 2], 3).full().reshape(-1), z['canonical_full'], **RT)
    np.testing.assert_allclose(tt.uniform([2, 3, 2], ranks=2, norm=3.0).full().reshape(-1), z['uniform_full'], **RT)
    np.testing.assert_array_equal(tt.build_core([[np.eye(3), 0], [L, np.eye(3)]]), z['core_nested'])
    np.testing.assert_array_equal(tt.build_core([L, np.eye(3), 2 * L]), z['core_flat'])
    np.random.seed(5)
    for c, r in zip(tt.rand([2, 3, 4], [1, 2, 1], [1, 3, 2, 1]).cores, cores('rand')):
        np.testing.assert_array_equal(c, r)


def test_container_errors():
    """The argument checks of tensor_train.py:194-198, 263-267."""
    import pytest
    with pytest.raises(ValueError):
        TT([np.ones((1, 2, 1, 2)), np.ones((3, 2, 1, 1))])
    with pytest.raises(ValueError):
        TT([np.ones((1, 2, 1))])
    with pytest.raises(ValueError):
        TT(np.ones((2, 2, 2)))
    with pytest.raises(TypeError):
        TT('cores')


def test_element_errors(golden):
    """The element-access errors of tensor_train.py:990-1027."""
    import pytest
    _, cores = golden('ttops_struct')
    A = TT(cores('A'))
    with pytest.raises(TypeError):
        A.element((1, 2, 0, 1, 2, 1, 1, 0))
    with pytest.raises(TypeError):
        A.element([1.0, 2, 0, 1, 2, 1, 1, 0])
    with pytest.raises(ValueError):
        A.element([1, 2, 0, 1])
    with pytest.raises(IndexError):
        A.element([2, 2, 0, 1, 2, 1, 1, 0])      # row index 2 of a mode of size 2
    with pytest.raises(IndexError):
        A.element([1, 2, 0, 1, 3, 1, 1, 0])      # column index 3 of a mode of size 3
    with pytest.raises(IndexError):
        A.element([1, 2, 0, -1, 2, 1, 1, 0])
