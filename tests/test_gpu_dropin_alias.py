"""The drop-in switch as the repository's integration guide documents it: its
module-alias block, taken verbatim from the guide, runs in a fresh interpreter, after which the
code below reaches this package only through ``scikit_tt.*`` import paths, in
the way the reference's tests call the ALS path (tests/test_sle.py:13-59 and
tests/test_evp.py:16-150): the Toeplitz system through the full-array TT
constructor, ``tt.ones(...).ortho_right()`` guesses, the triple-well
eigenproblem (operator from the reference-generated fixture) with eig and the
symmetrised eigh, and the private helpers ``scikit_tt/solvers/ode.py:13``
imports.
"""

import os
import re
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

USER_CODE = r'''
import numpy as np
import scipy.linalg as sla
import scipy.sparse.linalg as splin
from scikit_tt.tensor_train import TT
import scikit_tt.tensor_train as tt
import scikit_tt.solvers.sle as sle
import scikit_tt.solvers.evp as evp
from scikit_tt.solvers.sle import __construct_stack_left_op, __construct_stack_right_op  # noqa: F401
from scikit_tt.solvers.sle import __construct_micro_matrix_als, __construct_micro_matrix_mals  # noqa: F401
import scikit_tt.solvers.ode  # noqa: F401
assert TT.__module__.startswith('scikit_tt_gb300')

# linear system: Toeplitz(1..1024) as an order-10 TT, ones right-hand side, rank-5 ones guess
mat = sla.toeplitz(np.arange(1, 2 ** 10 + 1), np.arange(1, 2 ** 10 + 1)).astype(float)
op = TT(mat.reshape([2] * 20))
rhs = tt.ones(op.row_dims, [1] * op.order)
x0 = tt.ones(op.row_dims, [1] * op.order, ranks=5).ortho_right()
sol = sle.als(op, x0, rhs)
exact = np.linalg.solve(mat, np.ones(1024))
err = np.linalg.norm(sol.matricize() - exact) / np.linalg.norm(exact)
assert err < 1e-7, err
print('sle ok', err)

# eigenproblem: the triple-well Ulam operator, rank-15 ones guess, three eigenpairs
z = np.load(GOLDEN)
cores = [z[f'op_{i}'] for i in range(int(z['op_n']))]
op = TT(cores)
x0 = tt.ones(op.row_dims, [1] * op.order, ranks=15).ortho_right()
vals, vecs, _ = evp.als(op, x0, number_ev=3, repeats=10)
mv = z['mat_vals'][np.argsort(z['mat_vals'])[::-1]]
for i in range(3):
    assert abs(mv[i] - vals[i]) / mv[i] < 5e-3, (i, vals[i], mv[i])
sym = 0.5 * (op + op.transpose())
vals_h, _, _ = evp.als(sym, x0, number_ev=3, repeats=10, solver='eigh')
sv = np.sort(z['sym_vals'])[::-1]
for i in range(3):
    assert abs(sv[i] - vals_h[i]) / sv[i] < 5e-3, (i, vals_h[i], sv[i])
print('evp ok', vals, vals_h)
'''


def _alias_block():
    text = open(os.path.join(ROOT, 'INTEGRATION.md')).read()
    m = re.search(r'aliasing the modules.*?```python\n(.*?)```', text, re.S)
    assert m, 'the integration guide lost its module-alias block'
    return m.group(1)


def test_reference_style_code_through_the_alias_recipe():
    code = 'import sys\nsys.path.insert(0, %r)\n' % ROOT + _alias_block() + \
        'GOLDEN = %r\n' % os.path.join(ROOT, 'tests', 'golden', 'evp_triple_well.npz') + USER_CODE
    res = subprocess.run([sys.executable, '-c', code], capture_output=True, text=True, timeout=900)
    assert res.returncode == 0, res.stdout[-2000:] + res.stderr[-4000:]
    assert 'sle ok' in res.stdout and 'evp ok' in res.stdout
