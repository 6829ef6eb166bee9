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


def _round_bf16(x):
    u = x.astype(np.float32).view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return u.astype(np.uint32).view(np.float32)


def _round_tf32(x):
    u = x.astype(np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x1000) & ~np.uint64(0x1FFF)
    return u.astype(np.uint32).view(np.float32)


@pytest.mark.parametrize('kind,N,K', [(0, 32, 32), (0, 256, 32), (0, 48, 64), (0, 16, 128),
                                      (1, 32, 32), (1, 128, 16), (1, 64, 8), (1, 256, 64)])
def test_umma_selftest(kind, N, K):
    """One tcgen05.mma tile (M = 128) with shared-memory operands in the
    canonical K-major layout and the accumulator in tensor memory, against
    the product of the same BF16 / TF32-rounded operands in FP64."""
    from scikit_tt_gb300 import _lib
    lib, ctx = _lib.load(), _lib.context()
    rng = np.random.default_rng(17 * N + K + kind)
    A = rng.standard_normal((128, K)).astype(np.float32)
    Bt = rng.standard_normal((N, K)).astype(np.float32)
    out = np.full((128, N), np.nan, dtype=np.float32)
    f = lambda x: x.ctypes.data_as(ctypes.POINTER(ctypes.c_float))  # noqa: E731
    _lib.check(lib.ttals_umma_selftest(ctx, kind, N, K, f(A), f(Bt), f(out)))
    rnd = _round_bf16 if kind == 0 else _round_tf32
    ref = rnd(A).astype(np.float64) @ rnd(Bt).astype(np.float64).T
    # FP32 accumulation of exactly rounded operands
    assert np.abs(out - ref).max() <= 1e-5 * np.abs(ref).max()


def test_mixed_batch_contractions_run_on_tcgen05():
    """The mixed-precision batch kernel's GEMM-shaped contractions (emulated
    FP64 stacks and residuals, 3xTF32 inner applies) complete on tcgen05: the
    statistics count them and report no SIMT fallback."""
    from scikit_tt_gb300 import workloads as wl
    from scikit_tt_gb300.solvers import sle
    from scikit_tt_gb300.tensor_train import TT
    ws = [wl.coupled_sle(seed=s, d=8, n=8, rhs_rank=4, x_rank=16, repeats=1) for s in range(3)]
    probs = [tuple(TT([c.copy() for c in cs]) for cs in (w.op, w.x0, w.rhs)) for w in ws]
    _, st = sle.als_batch(probs, repeats=1, precision='mixed', tol=1e-10)
    assert st['tc_gemms'] > 0
    assert st['tc_fallbacks'] == 0, f"{st['tc_fallbacks']} of {st['tc_gemms'] + st['tc_fallbacks']} fell back"
