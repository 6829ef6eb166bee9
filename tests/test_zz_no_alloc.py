"""ttals_stack_op_noalloc: the interface-stack update for callers that cannot
allocate device memory (their device memory is pre-reserved by their own
pool, or they must avoid the device-wide synchronisation of cudaMalloc and
cudaFree).  Its two contraction intermediates live in a static 16 MiB device
array instead of the context's arena.

Checked through the C ABI against the allocating ttals_stack_op, within the
1e-12 relative tolerance the other stack tests use, on consecutive calls (so
leftover contents of the shared array from the previous call cannot leak
into the next one), including a problem exactly at the array's limit; that a
warmed-up call changes neither the device's free memory nor torch's
allocator; and that oversized problems, problems whose size would overflow
64 bits, and host pointers are refused before anything runs.  This file is
collected last on purpose.
"""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SCRATCH_DOUBLES = 1 << 21   # the static array: 16 MiB of doubles


def _dptr(t):
    return ctypes.cast(t.data_ptr(), ctypes.POINTER(ctypes.c_double))


def _shapes(left, r0, n, r1, R0, R1):
    stack = (r0, R0, r0) if left else (r1, R1, r1)
    out = (r1, R1, r1) if left else (r0, R0, r0)
    return stack, (r0, n, r1), (R0, n, n, R1), out


def _compare(lib, ctx, _lib, torch, rng, left, r0, n, r1, R0, R1):
    s_shape, x_shape, op_shape, out_shape = _shapes(left, r0, n, r1, R0, R1)
    stack, x, op = rng.standard_normal(s_shape), rng.standard_normal(x_shape), rng.standard_normal(op_shape)
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


def test_stack_op_noalloc_matches_allocating_entry_point():
    torch = pytest.importorskip('torch')
    from scikit_tt_gb300 import _lib
    lib = _lib.load()
    ctx = _lib.context()
    rng = np.random.default_rng(2024)
    cases = [(1, 6, 3, 5, 2, 3), (0, 7, 4, 6, 3, 2), (1, 9, 2, 9, 4, 4),
             # exactly at the limit: 2 * max(R) * max(r)^2 * n == the array's size
             (1, 128, 16, 128, 4, 4), (0, 128, 16, 96, 4, 3)]
    for case in cases:
        left, r0, n, r1, R0, R1 = case
        assert 2 * max(R0, R1) * max(r0, r1) ** 2 * n <= SCRATCH_DOUBLES
        _compare(lib, ctx, _lib, torch, rng, *case)


def test_stack_op_noalloc_allocates_nothing():
    torch = pytest.importorskip('torch')
    from scikit_tt_gb300 import _lib
    lib = _lib.load()
    ctx = _lib.context()
    rng = np.random.default_rng(7)
    left, r0, n, r1, R0, R1 = 1, 32, 8, 32, 4, 4
    s_shape, x_shape, op_shape, out_shape = _shapes(left, r0, n, r1, R0, R1)
    dev = torch.device('cuda', 0)
    ds, dx, dop = (torch.from_numpy(rng.standard_normal(s)).to(dev) for s in (s_shape, x_shape, op_shape))
    dout = torch.empty(out_shape, dtype=torch.float64, device=dev)

    def call():
        _lib.check(lib.ttals_stack_op_noalloc(ctx, left, _dptr(ds), _dptr(dx), _dptr(dop), r0, n, r1, R0, R1,
                                              _dptr(dout)))
        torch.cuda.synchronize()

    call()   # warm-up: loads the kernels' module and looks up the array's address once
    free0, _ = torch.cuda.mem_get_info()
    alloc0, reserved0 = torch.cuda.memory_allocated(), torch.cuda.memory_reserved()
    for _ in range(3):
        call()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, f'device free memory changed by {free0 - free1} bytes'
    assert (torch.cuda.memory_allocated(), torch.cuda.memory_reserved()) == (alloc0, reserved0)


def test_stack_op_noalloc_rejects_oversized_problem():
    torch = pytest.importorskip('torch')
    from scikit_tt_gb300 import _lib
    lib = _lib.load()
    ctx = _lib.context()
    # one-element device buffers: a size guard that let a call through would
    # still hand the kernels device memory, never host memory
    one = torch.zeros(1, dtype=torch.float64, device='cuda')
    p = _dptr(one)
    # 2 * 8 * 400^2 * 8 doubles > 16 MiB of scratch
    assert lib.ttals_stack_op_noalloc(ctx, 1, p, p, p, 400, 8, 400, 8, 8, p) == _lib.ERR_ARG
    assert b'static scratch' in lib.ttals_last_error(ctx)
    # one past the limit: 2 * 4 * 128^2 * 17 doubles
    assert lib.ttals_stack_op_noalloc(ctx, 1, p, p, p, 128, 17, 128, 4, 4, p) == _lib.ERR_ARG
    # max(R) * max(r)^2 * n = 2^20 * 2^42 * 4 wraps a 64-bit product to 0
    assert lib.ttals_stack_op_noalloc(ctx, 0, p, p, p, 1 << 21, 4, 1 << 21, 1 << 20, 1, p) == _lib.ERR_ARG
    assert b'static scratch' in lib.ttals_last_error(ctx)
    torch.cuda.synchronize()


def test_stack_op_noalloc_rejects_host_pointers():
    torch = pytest.importorskip('torch')
    from scikit_tt_gb300 import _lib
    lib = _lib.load()
    ctx = _lib.context()
    one = torch.zeros(1, dtype=torch.float64, device='cuda')
    host = np.zeros(1)
    d, h = _dptr(one), _lib.dptr(host)
    # unit dimensions: every buffer involved holds the one element a call would touch
    for args in [(h, d, d, d), (d, h, d, d), (d, d, h, d), (d, d, d, h)]:
        st = lib.ttals_stack_op_noalloc(ctx, 1, args[0], args[1], args[2], 1, 1, 1, 1, 1, args[3])
        assert st == _lib.ERR_ARG
        assert b'device' in lib.ttals_last_error(ctx)
    torch.cuda.synchronize()
