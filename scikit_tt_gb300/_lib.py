"""ctypes binding of ``libttals.so`` (C ABI in ``include/ttals.h``).

The library is the only compute path of this package: when it is missing, or
no CUDA device is present, every call raises ``RuntimeError`` -- there is no
CPU fallback.
"""

from __future__ import annotations

import ctypes as C
import os
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, 'libttals.so')

OK = 0
ERR_ARG = 1
ERR_CUDA = 2
ERR_NOMEM = 3
ERR_SINGULAR = 4
ERR_NONFINITE = 5
ERR_TIMEOUT = 6
ERR_NOCONV = 7
ERR_UNSUPPORTED = 8

PREC_FP64 = 0
PREC_MIXED = 1

SLE_SOLVERS = {'solve': 0, 'lu': 1}
EVP_SOLVERS = {'eig': 0, 'eigs': 1, 'eigh': 2}

# every symbol include/ttals.h declares
EXPORTS = (
    'ttals_create', 'ttals_destroy', 'ttals_last_error', 'ttals_set_stream', 'ttals_als_ranks',
    'ttals_batch_slots', 'ttals_set_batch_variant', 'ttals_wait_probe', 'ttals_sle_als', 'ttals_sle_mals', 'ttals_evp_als', 'ttals_tt_matmul', 'ttals_tt_ortho', 'ttals_tt_ortho_trunc', 'ttals_tt_norm',
    'ttals_stack_op', 'ttals_micro_matrix', 'ttals_set_profiling', 'ttals_measure_peaks',
    'ttals_stack_op_noalloc', 'ttals_sle_als_batch', 'ttals_solve_batch', 'ttals_submit', 'ttals_job_poll',
    'ttals_job_finish', 'ttals_batch_bytes', 'ttals_job_poll_each', 'ttals_job_fetch', 'ttals_job_report',
    'ttals_apply_f32',
    'ttals_apply_f64emu', 'ttals_umma_selftest', 'ttals_tdvp', 'ttals_arr',
)

REQ_SLE = 0
REQ_EVP = 1
REQ_GEVP = 2


class TTDesc(C.Structure):
    _fields_ = [('order', C.c_int32), ('row_dims', C.POINTER(C.c_int64)), ('col_dims', C.POINTER(C.c_int64)),
                ('ranks', C.POINTER(C.c_int64)), ('data', C.POINTER(C.c_double)), ('on_device', C.c_int32)]


class Request(C.Structure):
    _fields_ = [('kind', C.c_int32), ('op', TTDesc), ('x0', TTDesc), ('rhs', TTDesc), ('repeats', C.c_int32),
                ('solver', C.c_int32), ('sigma', C.c_double), ('conv_eps', C.c_double),
                ('out_data', C.POINTER(C.c_double)), ('out_value', C.POINTER(C.c_double)),
                ('out_iterations', C.POINTER(C.c_int32))]


class Stats(C.Structure):
    _fields_ = [('local_solves', C.c_int64), ('krylov_iterations', C.c_int64), ('refinement_steps', C.c_int64),
                ('max_local_residual', C.c_double), ('device_ms', C.c_double), ('kernel_launches', C.c_int64),
                ('solver_launches', C.c_int64), ('solver_ms', C.c_double), ('solver_flops64', C.c_double),
                ('solver_flops32', C.c_double), ('phase_cycles', C.c_double * 8), ('tc_gemms', C.c_int64),
                ('tc_fallbacks', C.c_int64), ('inner_apply_cycles', C.c_double),
                ('batch_tensor_cores', C.c_int32), ('batch_ctas_per_sm', C.c_int32),
                ('batch_solves_per_cta', C.c_int32)]

    def as_dict(self):
        d = {f: getattr(self, f) for f, _ in self._fields_}
        d['phase_cycles'] = list(self.phase_cycles)
        return d


_lib = None
_lock = threading.Lock()
_ctx = None


def load():
    """Load ``libttals.so`` and declare its signatures (raises if absent)."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f'{LIB_PATH} is missing: build it with python -m scikit_tt_gb300.build_ext '
                               '(the package has no CPU fallback)')
        lib = C.CDLL(LIB_PATH)
        P = C.POINTER
        i32, i64, dbl, vp = C.c_int32, C.c_int64, C.c_double, C.c_void_p
        pd, pi64 = P(C.c_double), P(C.c_int64)
        lib.ttals_create.argtypes = [P(vp), C.c_int, C.c_size_t]
        lib.ttals_destroy.argtypes = [vp]
        lib.ttals_last_error.argtypes = [vp]
        lib.ttals_last_error.restype = C.c_char_p
        lib.ttals_set_stream.argtypes = [vp, vp]
        lib.ttals_als_ranks.argtypes = [i32, pi64, pi64, pi64]
        lib.ttals_sle_als.argtypes = [vp, P(TTDesc), P(TTDesc), P(TTDesc), i32, i32, i32, dbl, pd, i32, pi64,
                                      P(Stats)]
        lib.ttals_sle_mals.argtypes = [vp, P(TTDesc), P(TTDesc), P(TTDesc), i32, i32, dbl, C.c_int64, dbl, pd, i32,
                                       pi64, pi64, P(Stats)]
        lib.ttals_evp_als.argtypes = [vp, P(TTDesc), P(TTDesc), i32, P(TTDesc), dbl, i32, i32, dbl, i32, dbl, i32,
                                      dbl, pd, pd, i32, pi64, P(i32), P(Stats)]
        lib.ttals_tt_matmul.argtypes = [vp, P(TTDesc), P(TTDesc), pd, i32]
        lib.ttals_arr.argtypes = [vp, i32, pi64, C.c_int64, pd, i32, pd, P(TTDesc), i32, dbl, pd, C.c_int64, pi64,
                                  P(Stats)]
        lib.ttals_tdvp.argtypes = [vp, P(TTDesc), P(TTDesc), i32, dbl, i32, i32, dbl, C.c_int64, i32, dbl, pd,
                                   C.c_int64, i32, pi64, P(Stats)]
        lib.ttals_batch_slots.argtypes = [vp, C.POINTER(i32)]
        lib.ttals_set_batch_variant.argtypes = [vp, i32]
        lib.ttals_wait_probe.argtypes = [vp, i32, C.c_uint32, C.POINTER(i32)]
        lib.ttals_tt_ortho.argtypes = [vp, P(TTDesc), i32, i32, i32, pd, i32, pi64]
        lib.ttals_tt_ortho_trunc.argtypes = [vp, P(TTDesc), i32, i32, i32, C.c_double, pi64, pd, i32, pi64]
        lib.ttals_tt_norm.argtypes = [vp, P(TTDesc), pd]
        lib.ttals_stack_op.argtypes = [vp, i32, pd, pd, pd, i64, i64, i64, i64, i64, pd, i32]
        lib.ttals_micro_matrix.argtypes = [vp, pd, pd, pd, i64, i64, i64, i64, i64, pd, i32]
        lib.ttals_set_profiling.argtypes = [vp, i32]
        lib.ttals_measure_peaks.argtypes = [vp, pd, pd]
        lib.ttals_sle_als_batch.argtypes = [vp, i32, P(TTDesc), P(TTDesc), P(TTDesc), P(i32), i32, dbl,
                                            P(pd), i32, P(Stats)]
        lib.ttals_solve_batch.argtypes = [vp, i32, P(Request), i32, dbl, i32, P(Stats)]
        lib.ttals_submit.argtypes = [vp, i32, P(Request), i32, dbl, P(vp)]
        lib.ttals_job_poll.argtypes = [vp, P(i32)]
        lib.ttals_job_finish.argtypes = [vp, P(Stats)]
        lib.ttals_job_poll_each.argtypes = [vp, P(i32)]
        pf = P(C.c_float)
        lib.ttals_apply_f32.argtypes = [vp, pf, pf, pf, pf, i64, i64, i64, i64, i64, pf]
        lib.ttals_apply_f64emu.argtypes = [vp, pd, pd, pd, pd, i64, i64, i64, i64, i64, pd]
        lib.ttals_umma_selftest.argtypes = [vp, i32, i32, i32, pf, pf, pf]
        lib.ttals_job_fetch.argtypes = [vp, i32]
        lib.ttals_job_report.argtypes = [vp, i32, pd, i32]
        lib.ttals_batch_bytes.argtypes = [vp, i32, P(Request), P(C.c_int64)]
        lib.ttals_stack_op_noalloc.argtypes = [vp, i32, pd, pd, pd, i64, i64, i64, i64, i64, pd]
        for name in EXPORTS:
            if name not in ('ttals_last_error',):
                getattr(lib, name).restype = C.c_int
        _lib = lib
        return lib


def context():
    """The process-wide engine context on the current CUDA device (created on
    first use).  ``TTALS_DEVICE`` picks the device; ``TTALS_BUDGET_BYTES`` caps
    the device memory the context may hold at once (arena and running jobs;
    unset or 0: 90 % of the memory free at creation)."""
    global _ctx
    if _ctx is not None:
        return _ctx
    lib = load()
    with _lock:
        if _ctx is None:
            dev = int(os.environ.get('TTALS_DEVICE', '0'))
            h = C.c_void_p()
            budget = int(os.environ.get('TTALS_BUDGET_BYTES', '0') or 0)
            st = lib.ttals_create(C.byref(h), dev, budget)
            if st != OK:
                raise RuntimeError(f'ttals_create failed with status {st}: a CUDA device with cooperative launch '
                                   'support is required (the package has no CPU fallback)')
            _ctx = h
    return _ctx


class EngineError(RuntimeError):
    pass


def check(status):
    """Map a C status to the exception types the reference raises."""
    if status == OK:
        return
    msg = load().ttals_last_error(context()).decode(errors='replace')
    if status == ERR_ARG:
        raise ValueError(msg)
    if status == ERR_SINGULAR:
        raise np.linalg.LinAlgError(msg)
    if status == ERR_UNSUPPORTED:
        raise NotImplementedError(msg)
    if status == ERR_NOMEM:
        raise MemoryError(msg)
    raise EngineError(f'status {status}: {msg}')


def dptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def i64ptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_int64))


class Packed:
    """A tensor train flattened for the C ABI (keeps the arrays alive)."""

    def __init__(self, cores):
        for c in cores:
            if np.iscomplexobj(c):
                raise NotImplementedError('complex tensor trains are not supported by the device path')
        self.order = len(cores)
        self.row = np.array([c.shape[1] for c in cores], dtype=np.int64)
        self.col = np.array([c.shape[2] for c in cores], dtype=np.int64)
        self.ranks = np.array([c.shape[0] for c in cores] + [cores[-1].shape[3]], dtype=np.int64)
        self.data = np.ascontiguousarray(np.concatenate([np.asarray(c, dtype=np.float64).ravel() for c in cores]))
        self.desc = TTDesc(self.order, i64ptr(self.row), i64ptr(self.col), i64ptr(self.ranks), dptr(self.data), 0)


def unpack(flat, row, col, ranks, core0_extra=1):
    """Split a flat core buffer into 4-D cores (core 0 may carry an extra axis)."""
    cores = []
    off = 0
    for i in range(len(row)):
        shape = (int(ranks[i]), int(row[i]), int(col[i]), int(ranks[i + 1]))
        cnt = int(np.prod(shape))
        if i == 0 and core0_extra > 1:
            cores.append(flat[off:off + cnt * core0_extra].reshape(shape + (core0_extra,)).copy())
            off += cnt * core0_extra
        else:
            cores.append(flat[off:off + cnt].reshape(shape).copy())
            off += cnt
    return cores
