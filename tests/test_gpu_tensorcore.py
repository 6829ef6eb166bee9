"""The FP32 tensor-core apply (3xTF32 mma.sync) of the mixed-precision inner
solver against an FP64 NumPy reference of the same local operator."""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize('a,n,s,R0,R1', [(32, 8, 32, 4, 4), (5, 3, 7, 2, 3), (17, 2, 9, 3, 1), (48, 4, 40, 4, 4),
                                         (1, 8, 32, 1, 4)])
def test_apply_f32_tensor_cores(a, n, s, R0, R1):
    from scikit_tt_gb300 import _lib
    lib, ctx = _lib.load(), _lib.context()
    rng = np.random.default_rng(a * 1000 + s)
    L = rng.standard_normal((a, R0, a)).astype(np.float32)
    A = rng.standard_normal((R0, n, n, R1)).astype(np.float32)
    Rt = rng.standard_normal((s, R1, s)).astype(np.float32)
    y = rng.standard_normal((a, n, s)).astype(np.float32)
    out = np.empty(a * n * s, dtype=np.float32)
    f = lambda x: x.ctypes.data_as(ctypes.POINTER(ctypes.c_float))  # noqa: E731
    _lib.check(lib.ttals_apply_f32(ctx, f(L), f(A), f(Rt), f(y), a, n, s, R0, R1, f(out)))
    ref = np.einsum('aRb,RmnQ,sQt,ans->bmt', L.astype(np.float64), A.astype(np.float64), Rt.astype(np.float64),
                    y.astype(np.float64)).ravel()
    # FP32-level accuracy (3xTF32), relative to the size of the result
    assert np.abs(out - ref).max() <= 2e-5 * np.abs(ref).max()


@pytest.mark.parametrize('a,n,s,R0,R1', [(32, 8, 32, 4, 4), (5, 3, 7, 2, 3), (17, 2, 9, 3, 1), (48, 4, 40, 4, 4),
                                         (1, 8, 32, 1, 4), (24, 8, 24, 3, 4)])
def test_apply_emulated_fp64(a, n, s, R0, R1):
    # Ozaki slicing on BF16 tensor cores: FP64-level accuracy relative to |L||A||Rt||y|
    from scikit_tt_gb300 import _lib
    lib, ctx = _lib.load(), _lib.context()
    rng = np.random.default_rng(a * 77 + s)
    L = rng.standard_normal((a, R0, a)) * np.exp(rng.uniform(-3, 3, (a, R0, a)))
    A = rng.standard_normal((R0, n, n, R1))
    Rt = rng.standard_normal((s, R1, s)) * 1e5
    y = rng.standard_normal((a, n, s)) * 1e-7
    out = np.empty(a * n * s)
    _lib.check(lib.ttals_apply_f64emu(ctx, _lib.dptr(L), _lib.dptr(A), _lib.dptr(Rt), _lib.dptr(y), a, n, s, R0, R1,
                                      _lib.dptr(out)))
    ref = np.einsum('aRb,RmnQ,sQt,ans->bmt', L, A, Rt, y).ravel()
    bound = np.einsum('aRb,RmnQ,sQt,ans->bmt', np.abs(L), np.abs(A), np.abs(Rt), np.abs(y)).ravel()
    # 48-bit slicing relative to row/column maxima: error ~2^-47 K max|A| max|B| per product
    assert np.abs(out - ref).max() <= 1e-13 * bound.max()
    assert np.abs(out - ref).max() <= 1e-11 * np.abs(ref).max()
