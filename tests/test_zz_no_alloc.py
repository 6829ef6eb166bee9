"""ttals_stack_op_noalloc: the interface-stack update for callers that cannot
allocate device memory (their device memory is pre-reserved by their own
pool, or they must avoid the device-wide synchronisation of cudaMalloc and
cudaFree).  Its two contraction intermediates live in a static 16 MiB device
array instead of the context's arena.

Checked through the C ABI against the allocating ttals_stack_op, within the
1e-12 relative tolerance the other stack tests use, on consecutive calls (so
leftover contents of the shared array from the previous call cannot leak
into the next one).  This file is collected last on purpose.
"""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dptr(t):
    return ctypes.cast(t.data_ptr(), ctypes.POINTER(ctypes.c_double))


def test_stack_op_noalloc_matches_allocating_entry_point():
    torch = pytest.importorskip('torch')
    from scikit_tt_gb300 import _lib
    lib = _lib.load()
    ctx = _lib.context()
    rng = np.random.default_rng(2024)
    cases = [(1, 6, 3, 5, 2, 3), (0, 7, 4, 6, 3, 2), (1, 9, 2, 9, 4, 4)]
    for left, r0, n, r1, R0, R1 in cases:
        stack = rng.standard_normal((r0, R0, r0) if left else (r1, R1, r1))
        x = rng.standard_normal((r0, n, r1))
        op = rng.standard_normal((R0, n, n, R1))
        out_shape = (r1, R1, r1) if left else (r0, R0, r0)
        ref = np.empty(out_shape)
        _lib.check(lib.ttals_stack_op(ctx, left, _lib.dptr(stack), _lib.dptr(x), _lib.dptr(op), r0, n, r1, R0, R1,
                                      _lib.dptr(ref), 0))
        dev = torch.device('cuda', 0)
        ds, dx, dop = (torch.from_numpy(a.copy()).to(dev) for a in (stack, x, op))
        dout = torch.full(out_shape, float('nan'), dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        _lib.check(lib.ttals_stack_op_noalloc(ctx, left, _dptr(ds), _dptr(dx), _dptr(dop), r0, n, r1, R0, R1,
                                              _dptr(dout)))
        torch.cuda.synchronize()
        got = dout.cpu().numpy()
        np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())


def test_stack_op_noalloc_rejects_oversized_problem():
    pytest.importorskip('torch')
    from scikit_tt_gb300 import _lib
    lib = _lib.load()
    ctx = _lib.context()
    dummy = np.zeros(1)
    # 2 * 8 * 400^2 * 8 doubles > 16 MiB of scratch
    st = lib.ttals_stack_op_noalloc(ctx, 1, _lib.dptr(dummy), _lib.dptr(dummy), _lib.dptr(dummy), 400, 8, 400, 8, 8,
                                    _lib.dptr(dummy))
    assert st == _lib.ERR_ARG
    assert b'static scratch' in lib.ttals_last_error(ctx)
