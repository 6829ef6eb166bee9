"""Failure detection without a GPU fault: a device-side wait that runs out.

The probe waits through the engine's bounded spin (the one every grid barrier
uses) on a flag that nothing sets; the kernel records a timeout status, returns,
and the host reads it.  The context must stay usable afterwards."""

import ctypes as C

import numpy as np
import pytest

from oracle import tt_oracle as O

pytestmark = pytest.mark.gpu


def test_bounded_wait_times_out_and_context_survives():
    from scikit_tt_gb300 import _lib
    from scikit_tt_gb300 import workloads as wl
    from scikit_tt_gb300.solvers import sle
    from scikit_tt_gb300.tensor_train import TT
    lib, ctx = _lib.load(), _lib.context()
    st = C.c_int32(-1)
    _lib.check(lib.ttals_wait_probe(ctx, 1, 1000, C.byref(st)))
    assert st.value == _lib.OK                       # flag already set: no wait
    _lib.check(lib.ttals_wait_probe(ctx, 0, 20000, C.byref(st)))
    assert st.value == _lib.ERR_TIMEOUT              # flag never set: the wait gives up
    # the same context still solves
    w = wl.laplace_sle(d=6, n=4, rhs_rank=3, x_rank=4, repeats=1)
    sol = sle.als(TT([c.copy() for c in w.op]), TT([c.copy() for c in w.x0]), TT([c.copy() for c in w.rhs]),
                  repeats=1)
    ref = O.sle_als(w.op, w.x0, w.rhs, repeats=1)
    assert O.stable_rel_diff(sol.cores, ref) < 1e-10


def test_wait_probe_rejects_unbounded_limits():
    from scikit_tt_gb300 import _lib
    st = C.c_int32(0)
    with pytest.raises(ValueError):
        _lib.check(_lib.load().ttals_wait_probe(_lib.context(), 0, 1 << 30, C.byref(st)))
