"""Generate the golden fixtures of ``tests/golden/`` from the reference itself.

Runs the unmodified scikit_tt package, imported read-only from the directory
given by ``--reference PATH`` or the ``SCIKIT_TT_REF`` environment variable
(one of the two is required: the directory that holds the ``scikit_tt``
package), on seeded inputs and stores inputs and outputs as ``.npz``.  The
oracle and the device engine are both checked against these files, so the GPU
tests never need the reference.

    python tests/golden/make_golden.py --reference /path/to/scikit_tt_checkout [case]
"""

from __future__ import annotations

import os
import sys
import time

import numpy as np


def _reference_root():
    """The reference checkout from ``--reference PATH`` or ``SCIKIT_TT_REF``;
    exits with a message when neither names a directory with a scikit_tt package."""
    root = None
    if '--reference' in sys.argv:
        k = sys.argv.index('--reference')
        if k + 1 >= len(sys.argv):
            sys.exit('make_golden.py: --reference needs a path')
        root = sys.argv[k + 1]
        del sys.argv[k:k + 2]
    root = root or os.environ.get('SCIKIT_TT_REF')
    if not root:
        sys.exit('make_golden.py: pass --reference PATH or set SCIKIT_TT_REF to the scikit_tt checkout')
    if not os.path.isfile(os.path.join(root, 'scikit_tt', 'solvers', 'sle.py')):
        sys.exit(f'make_golden.py: {root} does not hold the scikit_tt package (scikit_tt/solvers/sle.py)')
    return root


REF = _reference_root()
HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REF)
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import scipy.linalg as sla  # noqa: E402
import scikit_tt.tensor_train as rtt  # noqa: E402
import scikit_tt.models as rmodels  # noqa: E402
import scikit_tt.solvers.sle as rsle  # noqa: E402
import scikit_tt.solvers.evp as revp  # noqa: E402
import scikit_tt.solvers.ode as rode  # noqa: E402
from scikit_tt.tensor_train import TT as RTT  # noqa: E402

from scikit_tt_gb300 import workloads as wl  # noqa: E402


def pack(prefix, cores, out):
    out[prefix + '_n'] = np.array(len(cores))
    for i, c in enumerate(cores):
        out[f'{prefix}_{i}'] = np.asarray(c)


def sle_case(name, op, rhs, x0, repeats, solver='solve', store_op=True):
    sol = rsle.als(RTT([c.copy() for c in op]), RTT([c.copy() for c in x0]), RTT([c.copy() for c in rhs]),
                   repeats=repeats, solver=solver)
    out = {'repeats': np.array(repeats), 'solver': np.array(solver)}
    if store_op:
        pack('op', op, out)
    pack('rhs', rhs, out)
    pack('x0', x0, out)
    pack('sol', sol.cores, out)
    np.savez_compressed(os.path.join(HERE, name + '.npz'), **out)
    print(name, 'ranks', sol.ranks)


def evp_case(name, op, x0, repeats, solver, sigma, negate=False, conv_eps=1e-10):
    A = RTT([c.copy() for c in op])
    if negate:
        A = -1 * A
    val, vec, its = revp.als(A, RTT([c.copy() for c in x0]), repeats=repeats, solver=solver, sigma=sigma,
                             conv_eps=conv_eps)
    out = {'repeats': np.array(repeats), 'solver': np.array(solver), 'sigma': np.array(sigma),
           'negate': np.array(negate), 'conv_eps': np.array(conv_eps), 'val': np.array(val), 'its': np.array(its)}
    pack('op', [c.copy() for c in A.cores], out)
    pack('x0', x0, out)
    pack('vec', vec.cores, out)
    np.savez_compressed(os.path.join(HERE, name + '.npz'), **out)
    print(name, 'val', val, 'its', its)


def helpers_case():
    """Module-level helpers that scikit_tt/solvers/ode.py:13 imports."""
    rng = np.random.default_rng(7)
    a, n, s, R0, R1 = 5, 3, 4, 2, 3
    x0c = rng.standard_normal((a, n, 1, s))
    x1c = rng.standard_normal((s, n, 1, a))
    A0 = rng.standard_normal((R0, n, n, R1))
    A1 = rng.standard_normal((R1, n, n, R0))
    op, sol = RTT([A0, A1]), RTT([x0c, x1c])
    Lp = rng.standard_normal((a, R0, a))
    Rn = rng.standard_normal((a, R0, a))
    Ls = rng.standard_normal((a, R0, a))
    Rs = rng.standard_normal((s, R1, s))
    sl, sr = [Lp, None], [None, Rn]
    getattr(rsle, '__construct_stack_left_op')(1, sl, op, sol)
    getattr(rsle, '__construct_stack_right_op')(0, sr, op, sol)
    M = getattr(rsle, '__construct_micro_matrix_als')(0, [Ls], [Rs], op, sol)
    out = dict(x0c=x0c, x1c=x1c, A0=A0, A1=A1, Lp=Lp, Rn=Rn, Ls=Ls, Rs=Rs, left=sl[1], right=sr[0], micro=M)
    np.savez_compressed(os.path.join(HERE, 'helpers.npz'), **out)
    print('helpers', M.shape)


def ttops_case():
    rng = np.random.default_rng(11)
    d = 5
    ranks = [1, 3, 4, 2, 3, 1]
    dims = [2, 3, 2, 3, 2]
    t = [rng.standard_normal((ranks[i], dims[i], 1, ranks[i + 1])) for i in range(d)]
    opr = [1, 2, 3, 2, 2, 1]
    A = [rng.standard_normal((opr[i], dims[i], dims[i], opr[i + 1])) for i in range(d)]
    At = RTT([c.copy() for c in A])
    tt_ = RTT([c.copy() for c in t])
    prod = At.dot(tt_)
    out = dict(norm=np.array(tt_.norm()), opnorm=np.array(At.norm()), full=tt_.full().reshape(-1),
               prod_full=prod.full().reshape(-1),
               left_full=RTT([c.copy() for c in t]).ortho_left().full().reshape(-1),
               right_full=RTT([c.copy() for c in t]).ortho_right().full().reshape(-1))
    pack('t', t, out)
    pack('A', A, out)
    np.savez_compressed(os.path.join(HERE, 'ttops.npz'), **out)
    print('ttops norm', out['norm'])


def struct_case():
    """The TT container's host-side helpers: rank-sum addition and subtraction,
    scalar products, (partial) transposes, element access, full/matricize,
    the 1-norm, the HOSVD constructor and the constructors of
    tensor_train.py:1806-2032, 2144-2262."""
    rng = np.random.default_rng(21)
    rows, cols = [2, 3, 2, 3], [3, 2, 2, 2]

    def cores(rk, rd, cd, fn=rng.standard_normal):
        return [fn((rk[i], rd[i], cd[i], rk[i + 1])) for i in range(len(rd))]

    t = cores([1, 2, 3, 2, 1], rows, [1] * 4)
    u = cores([1, 3, 2, 2, 1], rows, [1] * 4)
    A = cores([1, 2, 2, 3, 1], rows, cols)
    P = cores([1, 2, 3, 2, 1], rows, [1] * 4, lambda s: rng.uniform(0.1, 1.0, s))
    Q = cores([1, 2, 2, 2, 1], rows, cols, lambda s: rng.uniform(0.1, 1.0, s))
    T, U, At = RTT([c.copy() for c in t]), RTT([c.copy() for c in u]), RTT([c.copy() for c in A])
    s = T + U
    full8 = s.full()
    h_thr = RTT(full8.copy(), threshold=1e-10)
    h_max = RTT(full8.copy(), max_rank=2)
    L = np.diag([2.0, 2.0, 2.0]) - np.diag([1.0, 1.0], 1) - np.diag([1.0, 1.0], -1)
    out = dict(
        add_full=s.full().reshape(-1), add_ranks=np.array(s.ranks),
        sub_full=(T - U).full().reshape(-1),
        rmul_full=(2.5 * T).full().reshape(-1), mul_full=(T * -0.75).full().reshape(-1),
        tr_full=At.copy().transpose().full().reshape(-1),
        tr_part_full=At.copy().transpose(cores=[0, 2]).full().reshape(-1),
        mat_A=At.matricize(), mat_t=T.matricize(),
        elem_A=np.array(At.element([1, 2, 0, 1, 2, 1, 1, 0])), elem_t=np.array(T.element([1, 0, 1, 2, 0, 0, 0, 0])),
        norm1_P=np.array(RTT([c.copy() for c in P]).norm(p=1)),
        norm1_Q=np.array(RTT([c.copy() for c in Q]).norm(p=1)),
        hosvd_thr_full=h_thr.full().reshape(-1), hosvd_thr_ranks=np.array(h_thr.ranks),
        hosvd_max_full=h_max.full().reshape(-1), hosvd_max_ranks=np.array(h_max.ranks),
        eye_full=rtt.eye([2, 3]).full().reshape(-1),
        ones_full=rtt.ones([2, 3], [1, 2], ranks=2).full().reshape(-1),
        unit_full=rtt.unit([2, 3, 2], [1, 2, 0]).full().reshape(-1),
        canonical_full=rtt.canonical([2, 3, 2, 2], 3).full().reshape(-1),
        uniform_full=rtt.uniform([2, 3, 2], ranks=2, norm=3.0).full().reshape(-1),
        core_nested=rtt.build_core([[np.eye(3), 0], [L, np.eye(3)]]),
        core_flat=rtt.build_core([L, np.eye(3), 2 * L]),
        L=L)
    pack('t', t, out)
    pack('u', u, out)
    pack('A', A, out)
    pack('P', P, out)
    pack('Q', Q, out)
    np.random.seed(5)                 # tt.rand draws from NumPy's global generator, in core order
    pack('rand', rtt.rand([2, 3, 4], [1, 2, 1], [1, 3, 2, 1]).cores, out)
    np.savez_compressed(os.path.join(HERE, 'ttops_struct.npz'), **out)
    print('ttops_struct add ranks', s.ranks, 'hosvd ranks', h_thr.ranks, h_max.ranks)


def container_case():
    """The rest of the TT container (tensor_train.py:526-904, 1432-1804,
    2076-2142): tensordot in its four modes (partial and complete on either
    side), rank_tensordot, concatenate, rank_transpose, tt2qtt / qtt2tt, diag,
    squeeze, svd / pinv at a bond, build_core_vector."""
    rng = np.random.default_rng(31)

    def rt(rk, rd, cd):
        return [rng.standard_normal((rk[i], rd[i], cd[i], rk[i + 1])) for i in range(len(rd))]

    a = rt([1, 2, 3, 2, 1], [2, 3, 2, 2], [1, 2, 1, 1])
    b = rt([1, 3, 2, 1], [2, 2, 3], [1, 1, 2])
    c = rt([1, 2, 2, 1], [2, 3, 2], [1, 2, 1])
    out = {}
    pack('a', a, out)
    pack('b', b, out)
    pack('c', c, out)
    A, B, Cc = (lambda: RTT([x.copy() for x in a])), (lambda: RTT([x.copy() for x in b])), \
        (lambda: RTT([x.copy() for x in c]))
    # (self, other, num_axes, mode) -- dims must match on the contracted ends
    e = rt([1, 1], [2], [1])
    pack('e', e, out)
    E = lambda: RTT([x.copy() for x in e])  # noqa: E731
    cases = {'lf2': (A, B, 0, 2, 'last-first'), 'fl1': (B, A, 0, 1, 'first-last'),
             'ff2': (A, Cc, 0, 2, 'first-first'), 'll1': (A, Cc, 0, 1, 'last-last'),
             'ff_full_self': (Cc, A, 0, 3, 'first-first'), 'lf_full_self': (E, A, 0, 1, 'last-first'),
             'fl_full_self': (E, A, 0, 1, 'first-last'), 'll_full_self': (E, A, 0, 1, 'last-last'),
             'full_both': (A, A, 0, 4, 'last-first'), 'bad': (A, B, 0, 1, 'last-last')}
    for key, (S, O, _, k, mode) in cases.items():
        try:
            r = S().tensordot(O(), k, mode=mode)
            out[f'td_{key}_cores_n'] = np.array(r.order)
            for i, core in enumerate(r.cores):
                out[f'td_{key}_cores_{i}'] = core
        except ValueError as e:
            out[f'td_{key}_error'] = np.array(str(e))
    out['m_last'], out['m_first'] = rng.standard_normal((1, 3)), rng.standard_normal((4, 1))
    out['rtd_last'] = np.asarray(A().rank_tensordot(out['m_last'], mode='last').cores[-1])
    out['rtd_first'] = np.asarray(A().rank_tensordot(out['m_first'], mode='first').cores[0])
    cat = A().concatenate(RTT([x.copy() for x in b]))
    out['cat_full'] = np.asarray(cat.full()).reshape(-1)
    out['rtr_full'] = np.asarray(A().rank_transpose().full()).reshape(-1)
    q = rt([1, 2, 3, 1], [4, 6, 2], [2, 1, 4])
    pack('q', q, out)
    qt = RTT([x.copy() for x in q]).tt2qtt([[2, 2], [2, 3], [2]], [[1, 2], [1, 1], [2, 2]])
    out['qtt_ranks'] = np.array(qt.ranks)
    out['qtt_full'] = np.asarray(qt.full()).reshape(-1)
    qt2 = RTT([x.copy() for x in q]).tt2qtt([[2, 2], [2, 3], [2]], [[1, 2], [1, 1], [2, 2]], threshold=0.6)
    out['qtt_thr_ranks'] = np.array(qt2.ranks)
    out['qtt_thr_full'] = np.asarray(qt2.full()).reshape(-1)
    back = qt.qtt2tt([2, 2, 1])
    out['back_full'] = np.asarray(back.full()).reshape(-1)
    out['back_rows'] = np.array(back.row_dims)
    dg = A().diag([0, 2])
    out['diag_full'] = np.asarray(dg.full()).reshape(-1)
    sq = rt([1, 2, 2, 3, 2, 1], [1, 3, 1, 1, 2], [1, 1, 1, 1, 2])
    pack('sq', sq, out)
    s_ = RTT([x.copy() for x in sq]).squeeze()
    out['sq_full'] = np.asarray(s_.full()).reshape(-1)
    out['sq_rows'] = np.array(s_.row_dims)
    v = rt([1, 3, 4, 3, 1], [3, 2, 3, 2], [1, 1, 1, 1])
    pack('v', v, out)
    u_, sv, w_ = RTT([x.copy() for x in v]).svd(2)
    out['svd_s'] = sv
    out['svd_u_full'] = np.tensordot(u_.cores[0], u_.cores[1], axes=(3, 0)).reshape(-1, u_.ranks[-1])
    u3, sv3, _ = RTT([x.copy() for x in v]).svd(2, max_rank=2)
    out['svd_s_r2'] = sv3
    pv = RTT([x.copy() for x in v]).pinv(2)
    out['pinv_full'] = np.asarray(pv.full()).reshape(-1)
    out['bcv'] = rtt.build_core_vector([np.arange(4.0).reshape(2, 2), 0, np.eye(2)])
    out['bcv_vec'] = rtt.build_core_vector([np.arange(3.0), 0])
    np.savez_compressed(os.path.join(HERE, 'ttops_container.npz'), **out)
    print('ttops_container', sorted(k for k in out if k.startswith('td_') and k.endswith('_n')),
          [k for k in out if k.endswith('_error')], out['qtt_ranks'], out['qtt_thr_ranks'], out['svd_s'])


def deflation_case():
    """evp.als with previous eigentensors and a shift (evp.py:376-381): the
    second-lowest Ising d=8 eigenpair, the first one deflated."""
    w = wl.ising_evp(d=8, x_rank=16, repeats=8)
    x0 = [c.copy() for c in RTT([c.copy() for c in w.x0]).ortho_right().cores]
    v0, t0, _ = revp.als(RTT([c.copy() for c in w.op]), RTT([c.copy() for c in x0]), repeats=8, sigma=w.sigma)
    t0 = (1.0 / t0.norm()) * t0
    v1, t1, its = revp.als(RTT([c.copy() for c in w.op]), RTT([c.copy() for c in x0]), previous=[t0.copy()],
                           shift=100.0, repeats=8, sigma=w.sigma)
    out = {'sigma': np.array(w.sigma), 'val0': np.array(v0), 'val': np.array(v1), 'its': np.array(its),
           'vec': np.asarray(t1.full()).reshape(-1)}
    pack('op', w.op, out)
    pack('x0', x0, out)
    pack('prev', [c.copy() for c in t0.cores], out)
    np.savez_compressed(os.path.join(HERE, 'evp_ising_d8_deflation.npz'), **out)
    print('evp_ising_d8_deflation', v0, v1, its)


def evp_block_case(name, op, x0, repeats, solver, sigma, number_ev, conv_eps=1e-10):
    """number_ev >= 1 on any operator: the eigenvalue list and one TT per eigenvector.

    The reference keeps the complex dtype of scipy's eig vectors; the wanted
    eigenpairs of these cases are real, so each eigentensor is stored as its
    full real vector (global phase removed)."""
    val, vec, its = revp.als(RTT([c.copy() for c in op]), RTT([c.copy() for c in x0]), repeats=repeats,
                             solver=solver, sigma=sigma, number_ev=number_ev, conv_eps=conv_eps)
    vecs = [vec] if number_ev == 1 else vec
    vals = np.atleast_1d(np.real(np.asarray(val)))
    out = {'repeats': np.array(repeats), 'solver': np.array(solver), 'sigma': np.array(sigma),
           'number_ev': np.array(number_ev), 'conv_eps': np.array(conv_eps), 'vals': vals, 'its': np.array(its)}
    pack('op', op, out)
    pack('x0', x0, out)
    for e, t in enumerate(vecs):
        # cores carry arbitrary complex phases (SVD of a complex-typed block);
        # the tensor itself is real up to one global phase: store it as a vector
        v = np.asarray(t.full()).reshape(-1)
        v = v * np.exp(-1j * np.angle(v[np.argmax(np.abs(v))]))
        assert np.abs(np.imag(v)).max() < 1e-10 * np.abs(v).max(), np.abs(np.imag(v)).max()
        out[f'vec{e}'] = np.real(v)
    np.savez_compressed(os.path.join(HERE, name + '.npz'), **out)
    print(name, 'vals', vals, 'its', its)


def evp_blocks():
    # nonsymmetric transfer operator (Arnoldi path): one and three eigenpairs near sigma = 1
    w = wl.markov_evp()
    x0 = [c.copy() for c in RTT([c.copy() for c in w.x0]).ortho_right().cores]
    evp_block_case('evp_markov_eig_k1', w.op, x0, 4, 'eig', 1.0, 1)
    evp_block_case('evp_markov_eig_k3', w.op, x0, 4, 'eig', 1.0, 3)
    evp_block_case('evp_markov_eigs_k3', w.op, x0, 4, 'eigs', 1.0, 3)
    # symmetric block of three (Lanczos with three Ritz pairs)
    w3 = wl.ising_evp(d=8, x_rank=8, repeats=4)
    x0 = [c.copy() for c in RTT([c.copy() for c in w3.x0]).ortho_right().cores]
    evp_block_case('evp_ising_d8_eigh_k3', w3.op, x0, 4, 'eigh', 1.0, 3)
    evp_block_case('evp_ising_d8_eig_k3', w3.op, x0, 4, 'eig', w3.sigma, 3)


def power_case(name, op, x0, gevp, repeats=10, sigma=0.999):
    """evp.power_method (inverse power iteration through sle.als) on a nonsymmetric operator."""
    A = RTT([c.copy() for c in op])
    M = rtt.eye(A.row_dims) if gevp else None
    val, vec = revp.power_method(A, RTT([c.copy() for c in x0]), operator_gevp=M, repeats=repeats, sigma=sigma)
    out = {'repeats': np.array(repeats), 'sigma': np.array(sigma), 'gevp': np.array(gevp), 'val': np.array(val),
           'vec0': np.asarray(vec.full()).reshape(-1)}
    pack('op', op, out)
    pack('x0', x0, out)
    np.savez_compressed(os.path.join(HERE, name + '.npz'), **out)
    print(name, 'val', val)


def power_cases():
    w = wl.markov_evp()
    x0 = [c.copy() for c in RTT([c.copy() for c in w.x0]).ortho_right().cores]
    power_case('evp_power_markov', w.op, x0, False)
    power_case('evp_power_markov_gevp', w.op, x0, True)


def ode_cases():
    """Implicit / explicit / trapezoidal / adaptive integrators on a Markov generator."""
    rng = np.random.default_rng(11)
    d, n = 4, 4
    gen = RTT(wl.markov_op(d, n, 0.2, rng)) - rtt.eye([n] * d)
    x0 = (1.0 / n ** d) * rtt.ones([n] * d, [1] * d)
    guess = RTT([np.abs(c) + 0.1 for c in wl.gaussian_tt(rng, d, n, 4)])
    out = {}
    pack('op', [c.copy() for c in gen.cores], out)
    pack('x0', [c.copy() for c in x0.cores], out)
    pack('guess', [c.copy() for c in guess.cores], out)
    steps = [0.1, 0.2, 0.4, 0.8]
    out['steps'] = np.array(steps)

    def store(prefix, sol):
        out[prefix + '_n'] = np.array(len(sol))
        for k, t in enumerate(sol):
            out[f'{prefix}_{k}'] = np.asarray(t.full()).reshape(-1)

    sol = rode.implicit_euler(gen, x0, guess, steps, progress=False)
    store('impl', sol)
    out['impl_err'] = np.array(rode.errors_impl_euler(gen, sol, steps))
    sol = rode.trapezoidal_rule(gen, x0, guess, steps, progress=False)
    store('trap', sol)
    out['trap_err'] = np.array(rode.errors_trapezoidal(gen, sol, steps))
    sol = rode.explicit_euler(gen, x0, [0.05, 0.05, 0.05], progress=False)
    store('expl', sol)
    out['expl_err'] = np.array(rode.errors_expl_euler(gen, sol, [0.05, 0.05, 0.05]))
    sol, times = rode.adaptive_step_size(gen, x0, guess, 2.0, step_size_first=0.05, progress=False)
    store('adapt', sol)
    out['adapt_times'] = np.array(times)
    np.savez_compressed(os.path.join(HERE, 'ode_markov.npz'), **out)
    print('ode_markov', 'adaptive steps', len(times), times[-1], 'impl err', out['impl_err'])


def hod_cases():
    """Higher-order differencing (ode.py:117-247) on a small Markov generator:
    order 2 and order 4 (operator powers), and a given previous value."""
    rng = np.random.default_rng(13)
    d, n = 3, 3
    gen = RTT(wl.markov_op(d, n, 0.2, rng)) - rtt.eye([n] * d)
    x0 = (1.0 / n ** d) * rtt.ones([n] * d, [1] * d)
    prev = RTT([np.abs(c) + 0.1 for c in wl.gaussian_tt(rng, d, n, 2)])
    out = {}
    pack('op', [c.copy() for c in gen.cores], out)
    pack('x0', [c.copy() for c in x0.cores], out)
    pack('prev', [c.copy() for c in prev.cores], out)

    def store(prefix, sol):
        out[prefix + '_n'] = np.array(len(sol))
        for k, t in enumerate(sol):
            out[f'{prefix}_{k}'] = np.asarray(t.full()).reshape(-1)

    store('o2', rode.hod(gen, x0, 0.1, 4, order=2, progress=False))
    store('o4', rode.hod(gen, x0, 0.1, 4, order=3, progress=False))
    store('o2p', rode.hod(gen, x0, 0.05, 3, order=2, previous_value=prev.copy(), normalize=2, progress=False))
    np.savez_compressed(os.path.join(HERE, 'ode_hod.npz'), **out)
    print('ode_hod', {k: v.shape for k, v in out.items() if k.endswith('_3')})


def trunc_cases():
    """ortho_left / ortho_right / ortho with threshold and max_rank (SVD truncation)."""
    rng = np.random.default_rng(21)
    d, n = 6, 3
    a = RTT(wl.gaussian_tt(rng, d, n, 2))
    b = RTT(wl.gaussian_tt(rng, d, n, 2))
    c = RTT(wl.gaussian_tt(rng, d, n, 4))
    t = a + b + 1e-9 * c          # rank 8 with a 1e-9 tail: truncates to rank <= 4
    out = {}
    pack('t', [x.copy() for x in t.cores], out)
    cases = {'left_thr': lambda x: x.ortho_left(threshold=1e-6),
             'right_max': lambda x: x.ortho_right(max_rank=3),
             'ortho_both': lambda x: x.ortho(threshold=1e-12, max_rank=4)}
    for key, fn in cases.items():
        r = fn(t.copy())
        out[key + '_ranks'] = np.array(r.ranks)
        out[key + '_full'] = np.asarray(r.full()).reshape(-1)
        print(key, r.ranks)
    np.savez_compressed(os.path.join(HERE, 'ttops_trunc.npz'), **out)


def mals_case(name, op, rhs, x0, repeats, threshold, max_rank, solver='solve'):
    sol = rsle.mals(RTT([c.copy() for c in op]), RTT([c.copy() for c in x0]), RTT([c.copy() for c in rhs]),
                    repeats=repeats, solver=solver, threshold=threshold, max_rank=max_rank)
    out = {'repeats': np.array(repeats), 'threshold': np.array(threshold),
           'max_rank': np.array(-1 if max_rank == np.inf else max_rank), 'solver': np.array(solver),
           'ranks': np.array(sol.ranks), 'full': np.asarray(sol.full()).reshape(-1)}
    pack('op', op, out)
    pack('rhs', rhs, out)
    pack('x0', x0, out)
    np.savez_compressed(os.path.join(HERE, name + '.npz'), **out)
    print(name, 'ranks', sol.ranks)


def mals_cases():
    w = wl.laplace_sle(d=6, n=4, rhs_rank=2, x_rank=2, repeats=2)
    mals_case('sle_mals_laplace_d6', w.op, w.rhs, w.x0, 2, 1e-12, np.inf)
    mals_case('sle_mals_laplace_d6_r4', w.op, w.rhs, w.x0, 2, 1e-12, 4)
    w2 = wl.coupled_sle(d=5, n=4, rhs_rank=3, x_rank=3, repeats=1)
    mals_case('sle_mals_coupled_d5_lu', w2.op, w2.rhs, w2.x0, 1, 1e-10, 8, 'lu')


def tdvp_case(name, fn, op, x0, step_size, steps, **kw):
    """One TDVP run; stores the full state after every step (real parts: the
    reference returns complex trains, which stay real for imaginary-time steps)."""
    sol = fn(RTT([c.copy() for c in op]), RTT([c.copy() for c in x0]), step_size, steps, **kw)
    out = {'step_im': np.array(np.imag(step_size)), 'steps': np.array(steps)}
    for key, val in kw.items():
        if key == 'local_solver':
            out['krylov_dim'] = np.array(0 if val['method'] == 'exact' else val.get('dimension', 5))
        else:
            out[key] = np.array(-1 if val == np.inf else val)
    pack('op', op, out)
    pack('x0', x0, out)
    imag = 0.0
    for k, t in enumerate(sol):
        full = np.asarray(t.full()).reshape(-1)
        imag = max(imag, float(np.max(np.abs(np.imag(full)))))
        out[f'full_{k}'] = np.real(full).copy()
        out[f'ranks_{k}'] = np.array(t.ranks)
    out['n_states'] = np.array(len(sol))
    assert imag < 1e-12, imag
    np.savez_compressed(os.path.join(HERE, name + '.npz'), **out)
    print(name, 'states', len(sol), 'final ranks', sol[-1].ranks, 'max imag', imag)


def tdvp_cases():
    """tdvp1site / tdvp2site in imaginary time on Ising chains (the setting of
    the reference's own TDVP test), with its local Krylov method and with the
    exact local exponential."""
    N = 5
    op = [c.copy() for c in rmodels.ising(N, J=1.0, h=1.2).cores]
    init = rtt.uniform(N * [2], ranks=15).ortho()
    init = (1 / init.norm()) * init
    x0 = [c.copy() for c in init.cores]
    h = -1j * 0.02
    tdvp_case('tdvp1_ising_d5_krylov', rode.tdvp1site, op, x0, h, 30, local_solver={'method': 'local_krylov'},
              normalize=2)
    tdvp_case('tdvp1_ising_d5_exact', rode.tdvp1site, op, x0, h, 30, local_solver={'method': 'exact'}, normalize=2)
    tdvp_case('tdvp2_ising_d5_krylov', rode.tdvp2site, op, x0, h, 30, local_solver={'method': 'local_krylov'},
              normalize=2)
    # a random initial value, rank capped at 3 (truncating two-site splits), no normalisation
    # (normalize=1 is the sum of all entries, meant for non-negative states)
    rng = np.random.default_rng(31)
    N2 = 6
    op2 = [c.copy() for c in rmodels.ising(N2, J=1.0, h=0.7).cores]
    t2 = RTT(wl.gaussian_tt(rng, N2, 2, 2)).ortho_right()
    t2 = (1 / t2.norm()) * t2
    x02 = [c.copy() for c in t2.cores]
    tdvp_case('tdvp2_ising_d6_exact_r3', rode.tdvp2site, op2, x02, -1j * 0.05, 8, local_solver={'method': 'exact'},
              threshold=1e-12, max_rank=3)
    tdvp_case('tdvp1_ising_d6_krylov4', rode.tdvp1site, op2, x02, -1j * 0.05, 8,
              local_solver={'method': 'krylov', 'dimension': 4}, normalize=0)


def kuramoto_data(d=10, m=1000, seed=3):
    """The Kuramoto setting of the reference's tests/test_regression.py:24-71
    (oscillator phases from solve_ivp, derivatives as outputs), seeded."""
    import scipy.integrate as spint
    rng = np.random.default_rng(seed)
    x0 = 2 * np.pi * rng.random(d) - np.pi
    w = np.linspace(-5, 5, d)

    def rhs(_, theta):
        ti, tj = np.meshgrid(theta, theta)
        return w + 2 / d * np.sin(tj - ti).sum(0) + 0.2 * np.sin(theta)

    sol = spint.solve_ivp(rhs, [0, 100], x0, method='BDF', t_eval=np.linspace(0, 100, m))
    x = sol.y
    y = np.zeros((d, m))
    for j in range(m):
        y[:, j] = rhs(0, x[:, j])
    return x, y, w


def arr_case(name, x, y, basis, x0, repeats, rcond):
    import scikit_tt.data_driven.regression as rreg
    sol = rreg.arr(x, y, basis, RTT([c.copy() for c in x0]), repeats=repeats, rcond=rcond, progress=False)
    theta = [np.array([[f(x[:, j]) for j in range(x.shape[1])] for f in funcs]) for funcs in basis]
    out = {'repeats': np.array(repeats), 'rcond': np.array(rcond), 'x': x, 'y': y, 'n_out': np.array(len(sol))}
    for i, t in enumerate(theta):
        out[f'theta_{i}'] = t
    out['theta_n'] = np.array(len(theta))
    pack('x0', x0, out)
    for k, t in enumerate(sol):
        pack(f'sol{k}', [np.asarray(c) for c in t.cores], out)
    np.savez_compressed(os.path.join(HERE, name + '.npz'), **out)
    print(name, 'outputs', len(sol), 'ranks', sol[0].ranks)


def arr_cases():
    """regression.arr on the Kuramoto data of the reference's own test (sine and
    cosine bases of 11 functions, rank 11), and a three-mode fit with ranks 3, 2."""
    import scikit_tt.data_driven.transform as rtdt
    x, y, w = kuramoto_data()
    basis = [[rtdt.ConstantFunction(0)] + [rtdt.Sin(i, 1) for i in range(10)],
             [rtdt.ConstantFunction(0)] + [rtdt.Cos(i, 1) for i in range(10)]]
    x0 = [c.copy() for c in rtt.ones([11, 11], [1, 1], 11).cores]
    arr_case('arr_kuramoto_rcond12', x, y, basis, x0, 3, 1e-12)
    # exact coefficient tensor of the Kuramoto right-hand side (tests/test_regression.py:36, 116-137)
    z = dict(np.load(os.path.join(HERE, 'arr_kuramoto_rcond12.npz')))
    z['xi_exact_full'] = np.asarray(rmodels.kuramoto_coefficients(10, w).full()).reshape(-1)
    np.savez_compressed(os.path.join(HERE, 'arr_kuramoto_rcond12.npz'), **z)
    arr_case('arr_kuramoto_rcond2', x, y, basis, x0, 2, 1e-2)
    rng = np.random.default_rng(41)
    xs = rng.uniform(-1, 1, (3, 400))
    ys = np.vstack([np.sin(2 * xs[0]) * xs[1] + 0.5 * xs[2] ** 2, np.exp(-xs[0] ** 2) - xs[1] * xs[2]])
    basis3 = [[rtdt.ConstantFunction(0), rtdt.Identity(0), rtdt.Monomial(0, 2), rtdt.Sin(0, 2)],
              [rtdt.ConstantFunction(1), rtdt.Identity(1), rtdt.Monomial(1, 2), rtdt.Monomial(1, 3),
               rtdt.GaussFunction(1, 0.0, 0.5)],
              [rtdt.ConstantFunction(2), rtdt.Identity(2), rtdt.Legendre(2, 2)]]
    x03 = [c.copy() for c in rtt.rand([4, 5, 3], [1, 1, 1], [1, 3, 2, 1]).cores]
    arr_case('arr_three_mode', xs, ys, basis3, x03, 3, 1e-10)


def fingerprint(cores):
    """Sum and sum of squares over all cores plus their shapes: the tests check
    that the seeded generator still yields the inputs the reference solved."""
    return np.array([sum(float(c.sum()) for c in cores), sum(float((c * c).sum()) for c in cores)])


def _timed_als(w):
    t0 = time.perf_counter()
    sol = rsle.als(RTT([c.copy() for c in w.op]), RTT([c.copy() for c in w.x0]),
                   RTT([c.copy() for c in w.rhs]), repeats=w.repeats, solver='solve')
    return sol, time.perf_counter() - t0


def headline_case():
    """The coupled-Laplacian SLE at full size (d=32, n=8, operator rank 4, RHS
    rank 8, guess rank 32, 4 sweeps, seed 0): the reference's own sle.als on
    the inputs ``workloads.coupled_sle(seed=0)`` builds, which are also the
    first instance of the benchmark's batch.  Inputs are regenerated by the
    tests from the seed (their fingerprints are stored); the solution cores,
    the wall time and the host's thread count are stored."""
    from oracle import tt_oracle as orc
    w = wl.coupled_sle(seed=0, d=32, n=8, rhs_rank=8, x_rank=32, repeats=4)
    sol, wall = _timed_als(w)
    res = orc.stable_residual(w.op, [np.asarray(c) for c in sol.cores], w.rhs)
    out = {'seed': np.array(0), 'repeats': np.array(w.repeats), 'wall_s': np.array(wall),
           'host_threads': np.array(os.cpu_count()), 'global_rel_residual': np.array(res),
           'fp_op': fingerprint(w.op), 'fp_rhs': fingerprint(w.rhs), 'fp_x0': fingerprint(w.x0)}
    pack('sol', sol.cores, out)
    np.savez_compressed(os.path.join(HERE, 'sle_coupled_d32_headline.npz'), **out)
    print('headline ranks', sol.ranks, 'wall %.1f s' % wall, 'global residual %.3e' % res)


def triple_well_case():
    """The reference's own eigenproblem known answer (tests/test_evp.py:16-150):
    the Ulam transfer operator of the triple-well data shipped with the
    reference (examples/data/triple_well_transitions.npz, coarse-grained as the
    test does) in TT format, built by the reference's ulam_2d; the rank-15 ones
    guess, right-orthonormalised; the reference's evp.als with eig, eigs and
    eigh (symmetrised operator), number_ev=3, 10 sweeps, eig with the identity
    operator_gevp, and power_method; and the dense eigs answers the test
    compares with.  Eigenvectors are stored as full vectors."""
    import scipy.sparse.linalg as splin
    import scikit_tt.data_driven.ulam as rulam
    tr = np.load(os.path.join(REF, 'examples', 'data', 'triple_well_transitions.npz'))['transitions']
    tr = np.int64(np.ceil(np.true_divide(tr, 2)))
    op = rulam.ulam_2d(tr, [25, 25], 2000)
    x0 = rtt.ones(op.row_dims, [1] * op.order, ranks=15).ortho_right()
    out = {}
    pack('op', [c.copy() for c in op.cores], out)
    pack('x0', [c.copy() for c in x0.cores], out)
    mat = op.matricize()
    vals, vecs = splin.eigs(mat, k=3)
    out['mat_vals'], out['mat_vecs'] = np.real(vals), np.real(vecs)
    sym = 0.5 * (op + op.transpose())
    symmat = 0.5 * (mat + mat.transpose())
    svals, svecs = splin.eigs(symmat, k=3)
    out['sym_vals'], out['sym_vecs'] = np.real(svals), np.real(svecs)
    pack('sym', [c.copy() for c in sym.cores], out)

    def cp(t):
        return RTT([c.copy() for c in t.cores])
    for solver in ('eig', 'eigs', 'eigh'):
        A = sym if solver == 'eigh' else op
        v, t, its = revp.als(cp(A), cp(x0), number_ev=3, repeats=10, solver=solver)
        out[f'{solver}_vals'] = np.array(v)
        out[f'{solver}_vecs'] = np.stack([t[k].matricize() for k in range(3)])
        out[f'{solver}_its'] = np.array(its)
        print('triple well', solver, v, its)
    v1, t1, _ = revp.als(cp(op), cp(x0), operator_gevp=rtt.eye(op.row_dims), repeats=10)
    out['gevp_val'] = np.array(v1)
    out['gevp_vec'] = t1.matricize()
    pv, pt = revp.power_method(cp(op), cp(x0))
    out['power_val'] = np.array(pv)
    out['power_vec'] = pt.matricize()
    print('triple well gevp', v1, 'power', pv)
    np.savez_compressed(os.path.join(HERE, 'evp_triple_well.npz'), **out)


BATCH_SUBSET = list(range(16))   # the 16 smallest-seed instances of the uneven batch


def gevp_case(name, op, gevp, x0, repeats, solver, sigma, conv_eps=1e-10):
    """evp.als with a non-identity operator_gevp (evp.py:272-287, 314-329, 367-368, 410-439)."""
    val, vec, its = revp.als(RTT([c.copy() for c in op]), RTT([c.copy() for c in x0]),
                             operator_gevp=RTT([c.copy() for c in gevp]), repeats=repeats, solver=solver,
                             sigma=sigma, conv_eps=conv_eps)
    out = {'repeats': np.array(repeats), 'solver': np.array(solver), 'sigma': np.array(sigma),
           'conv_eps': np.array(conv_eps), 'val': np.array(val), 'its': np.array(its)}
    pack('op', op, out)
    pack('gevp', gevp, out)
    pack('x0', x0, out)
    pack('vec', vec.cores, out)
    # the dense pencil's eigenvalues, for the eigenvalues the ALS approaches
    A = RTT([c.copy() for c in op]).matricize()
    B = RTT([c.copy() for c in gevp]).matricize()
    out['pencil_vals'] = np.sort(sla.eigh(A, B, eigvals_only=True))
    np.savez_compressed(os.path.join(HERE, name + '.npz'), **out)
    print(name, 'val', val, 'its', its, 'pencil ends', out['pencil_vals'][[0, -1]])


def gevp_cases():
    """Ising d=6 (g=1.2) against the SPD mass operator sum_i L_i + I (L = [[2,-1],[-1,2]]),
    right-orthonormal rank-4 guess: the lowest generalised eigenpair ('eig', sigma below the
    spectrum) and the largest ('eigh')."""
    d = 6
    op = wl.ising_op(d, 1.0, 1.2)
    gevp = wl.laplace_op(d, 2, h=1.0, shift=1.0)
    rng = np.random.default_rng(11)
    x0 = [c.copy() for c in RTT(wl.gaussian_tt(rng, d, 2, 4)).ortho_right().cores]
    gevp_case('evp_gevp_ising_d6_eig', op, gevp, x0, 4, 'eig', -3.0)
    gevp_case('evp_gevp_ising_d6_eigh', op, gevp, x0, 4, 'eigh', 1.0)


def batch_subset_case():
    """The 16 smallest-seed instances of the uneven batch (instance j from
    default_rng(1000 + j): d 8..32, n in {2,4,8}, ranks 4..48, 4 sweeps), each
    solved by the reference's sle.als.  Stores per instance the solution cores,
    the input fingerprints, the wall time and the global residual."""
    from oracle import tt_oracle as orc
    out = {'seeds': np.array(BATCH_SUBSET), 'host_threads': np.array(os.cpu_count())}
    walls = []
    for j in BATCH_SUBSET:
        w = wl.batch_instance(j)
        sol, wall = _timed_als(w)
        walls.append(wall)
        res = orc.stable_residual(w.op, [np.asarray(c) for c in sol.cores], w.rhs)
        out[f'j{j}_global_rel_residual'] = np.array(res)
        out[f'j{j}_fp_rhs'] = fingerprint(w.rhs)
        out[f'j{j}_fp_x0'] = fingerprint(w.x0)
        pack(f'j{j}_sol', sol.cores, out)
        print('batch instance', j, w.meta, 'wall %.2f s' % wall, 'residual %.3e' % res, flush=True)
    out['wall_s'] = np.array(walls)
    np.savez_compressed(os.path.join(HERE, 'sle_batch_subset.npz'), **out)


def main():
    # workload 1 (exact) with both local solvers
    w1 = wl.laplace_sle()
    sle_case('sle_laplace_d10', w1.op, w1.rhs, w1.x0, w1.repeats, 'solve')
    sle_case('sle_laplace_d10_lu', w1.op, w1.rhs, w1.x0, w1.repeats, 'lu')
    # workload 1 at rank 8, 4 sweeps (deeper convergence)
    w1b = wl.laplace_sle(x_rank=8, repeats=4)
    sle_case('sle_laplace_d10_r8', w1b.op, w1b.rhs, w1b.x0, w1b.repeats, 'solve')
    # reduced workload 2 (coupled operator, rank 4)
    w2 = wl.coupled_sle(d=8, n=4, rhs_rank=4, x_rank=8, repeats=3)
    sle_case('sle_coupled_d8', w2.op, w2.rhs, w2.x0, w2.repeats, 'solve')
    # the reference's own known-answer SLE test: Toeplitz(1..1024) as an order-10 TT
    # (the operator is rebuilt by the tests: its untruncated TT is 17 MB)
    mat = sla.toeplitz(np.arange(1, 2 ** 10 + 1), np.arange(1, 2 ** 10 + 1)).astype(float)
    op = RTT(mat.reshape([2] * 20))
    rhs = rtt.ones(op.row_dims, [1] * 10)
    x0 = rtt.ones(op.row_dims, [1] * 10, ranks=5).ortho_right()
    sle_case('sle_toeplitz', [c.copy() for c in op.cores], [c.copy() for c in rhs.cores],
             [c.copy() for c in x0.cores], 1, 'solve', store_op=False)
    # Ising EVP (lowest eigenpair) both ways the reference allows
    for d, r in [(12, 16), (16, 16)]:
        w3 = wl.ising_evp(d=d, x_rank=r, repeats=6)
        x0o = RTT([c.copy() for c in w3.x0]).ortho_right()
        evp_case(f'evp_ising_d{d}_eig', w3.op, [c.copy() for c in x0o.cores], 6, 'eig', w3.sigma)
        evp_case(f'evp_ising_d{d}_eigh', w3.op, [c.copy() for c in x0o.cores], 6, 'eigh', 1.0, negate=True)
    helpers_case()
    ttops_case()
    struct_case()
    container_case()
    deflation_case()
    evp_blocks()
    power_cases()
    ode_cases()
    hod_cases()
    trunc_cases()
    mals_cases()
    tdvp_cases()
    arr_cases()
    triple_well_case()
    headline_case()
    batch_subset_case()


if __name__ == '__main__':
    if len(sys.argv) > 1 and sys.argv[1] == 'evp_blocks':
        evp_blocks()
    elif len(sys.argv) > 1 and sys.argv[1] == 'power':
        power_cases()
    elif len(sys.argv) > 1 and sys.argv[1] == 'ode':
        ode_cases()
    elif len(sys.argv) > 1 and sys.argv[1] == 'trunc':
        trunc_cases()
    elif len(sys.argv) > 1 and sys.argv[1] == 'mals':
        mals_cases()
    elif len(sys.argv) > 1 and sys.argv[1] == 'tdvp':
        tdvp_cases()
    elif len(sys.argv) > 1 and sys.argv[1] == 'arr':
        arr_cases()
    elif len(sys.argv) > 1 and sys.argv[1] == 'struct':
        struct_case()
    elif len(sys.argv) > 1 and sys.argv[1] == 'deflation':
        deflation_case()
    elif len(sys.argv) > 1 and sys.argv[1] == 'hod':
        hod_cases()
    elif len(sys.argv) > 1 and sys.argv[1] == 'container':
        container_case()
    elif len(sys.argv) > 1 and sys.argv[1] == 'triple_well':
        triple_well_case()
    elif len(sys.argv) > 1 and sys.argv[1] == 'headline':
        headline_case()
    elif len(sys.argv) > 1 and sys.argv[1] == 'gevp':
        gevp_cases()
    elif len(sys.argv) > 1 and sys.argv[1] == 'batch_subset':
        batch_subset_case()
    else:
        main()
