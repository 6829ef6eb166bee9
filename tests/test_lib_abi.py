"""The C ABI library builds and exports every symbol include/ttals.h declares
(no device calls: runs without a GPU)."""

import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    src = open(os.path.join(ROOT, 'include', 'ttals.h')).read()
    return sorted(set(re.findall(r'\b(ttals_[a-z_0-9]+)\s*\(', src)))


def test_header_and_library_exports():
    from scikit_tt_gb300 import build_ext, _lib
    path = build_ext.build()
    lib = ctypes.CDLL(path)
    names = declared()
    assert len(names) >= 10
    for n in names:
        assert hasattr(lib, n), n
    assert sorted(_lib.EXPORTS) == names


def test_rank_schedule_host_only():
    from scikit_tt_gb300 import _lib
    import numpy as np
    lib = _lib.load()
    dims = np.array([4] * 10, dtype=np.int64)
    xr = np.array([1] + [5] * 9 + [1], dtype=np.int64)
    out = np.zeros(11, dtype=np.int64)
    assert lib.ttals_als_ranks(10, _lib.i64ptr(dims), _lib.i64ptr(xr), _lib.i64ptr(out)) == 0
    assert list(out) == [1, 4, 5, 5, 5, 5, 5, 5, 5, 4, 1]   # reference ranks after one sweep
