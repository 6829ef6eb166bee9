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


C_CALLER = r'''
#include <stdio.h>
#include "ttals.h"
int main(void) {
  const int64_t dims[10] = {4, 4, 4, 4, 4, 4, 4, 4, 4, 4};
  const int64_t xr[11] = {1, 5, 5, 5, 5, 5, 5, 5, 5, 5, 1};
  int64_t out[11];
  if (ttals_als_ranks(10, dims, xr, out) != TTALS_OK) return 2;
  if (ttals_als_ranks(-1, dims, xr, out) == TTALS_OK) return 3;
  for (int i = 0; i < 11; ++i) printf("%lld ", (long long)out[i]);
  printf("\n");
  return 0;
}
'''


def test_header_is_plain_c_and_links(tmp_path):
    """A C99 caller (what a non-Python binding compiles against) includes
    ttals.h with -pedantic, links libttals.so and calls a host-only entry."""
    import shutil
    import subprocess
    import pytest
    from scikit_tt_gb300 import build_ext
    if shutil.which('gcc') is None:
        pytest.skip('no C compiler')
    lib = build_ext.build()
    src = tmp_path / 'caller.c'
    src.write_text(C_CALLER)
    exe = tmp_path / 'caller'
    libdir = os.path.dirname(lib)
    subprocess.run(['gcc', '-std=c99', '-Wall', '-Wextra', '-pedantic', '-Werror', '-I', os.path.join(ROOT, 'include'),
                    str(src), '-L', libdir, '-l:libttals.so', f'-Wl,-rpath,{libdir}', '-o', str(exe)], check=True)
    res = subprocess.run([str(exe)], capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    assert res.stdout.split() == ['1', '4', '5', '5', '5', '5', '5', '5', '5', '4', '1']


def _header_arity():
    """Parameter count of every ttals_* declaration in the header."""
    src = re.sub(r'/\*.*?\*/', '', open(os.path.join(ROOT, 'include', 'ttals.h')).read(), flags=re.S)
    out = {}
    for m in re.finditer(r'\b(ttals_[a-z_0-9]+)\s*\(([^;{]*?)\)\s*;', src, flags=re.S):
        params = m.group(2).strip()
        out[m.group(1)] = 0 if params in ('', 'void') else params.count(',') + 1
    return out


def test_binding_matches_header_arity():
    """The ctypes binding declares as many arguments as the header for every entry point."""
    from scikit_tt_gb300 import build_ext, _lib
    build_ext.build()
    lib = _lib.load()
    arity = _header_arity()
    assert sorted(arity) == declared()
    for name, n in arity.items():
        assert len(getattr(lib, name).argtypes) == n, name


def test_context_budget_from_environment(monkeypatch):
    """TTALS_BUDGET_BYTES reaches ttals_create (0 when unset: 90 % of free memory)."""
    from scikit_tt_gb300 import _lib
    seen = []

    class Fake:
        def ttals_create(self, h, dev, budget):
            seen.append((dev, budget))
            return _lib.OK

    monkeypatch.setattr(_lib, 'load', lambda: Fake())
    for env, want in ((None, 0), ('150000000000', 150 * 10 ** 9)):
        monkeypatch.setattr(_lib, '_ctx', None)
        if env is None:
            monkeypatch.delenv('TTALS_BUDGET_BYTES', raising=False)
        else:
            monkeypatch.setenv('TTALS_BUDGET_BYTES', env)
        _lib.context()
        assert seen[-1][1] == want
    monkeypatch.setattr(_lib, '_ctx', None)
