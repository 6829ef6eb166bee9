"""Seeded synthetic ALS workloads (input construction only).

Five workloads, each a pure function of its seed:

1. ``laplace_sle``    shifted discrete Laplacian, d=10, n=4, operator rank 2,
                      RHS rank 3 / guess rank 5 (N(0,1), default_rng(0)), 2 sweeps.
2. ``coupled_sle``    Laplacian + nearest-neighbour coupling sum c_i D (x) D,
                      d=32, n=8, operator rank 4, RHS rank 8, guess rank 32,
                      4 sweeps.
3. ``ising_evp``      transverse-field Ising chain d=48, J=1, g=1 (rank 3),
                      guess ``rand`` rank 64 from RandomState(1), 6 sweeps.
4. ``batch_sle``      256 independent instances, instance j from
                      default_rng(1000 + j): d~U{8..32}, n in {2,4,8},
                      r~U{4..48}, shift~U(0.5,2), c_i~U(0,0.5), RHS rank 4.
5. ``serving_stream`` Poisson arrivals (rate 2000/s) mixing 80 % workload-4
                      SLE requests and 20 % Ising EVP requests.

Laplacian: ``L = tridiag(-1, 2, -1) / h^2`` with h = 1/5 (not rescaled with n).
Coupling matrix: ``D = diag(linspace(-1, 1, n))``.
"""

from __future__ import annotations

from dataclasses import dataclass, field
from typing import List

import numpy as np

from .tensor_train import build_core


def laplacian(n: int, h: float = 0.2) -> np.ndarray:
    return (2.0 * np.eye(n) - np.eye(n, k=1) - np.eye(n, k=-1)) / h ** 2


def laplace_op(d: int, n: int, h: float = 0.2, shift: float = 1.0) -> List[np.ndarray]:
    """``sum_i L_i + shift * I`` as a rank-2 TT operator; the shift is folded
    into the first core: ``[[L + shift I, I]]``, ``[[I, 0], [L, I]]``, ``[I, L]``."""
    L, I = laplacian(n, h), np.eye(n)
    cores = [build_core([[L + shift * I, I]])]
    cores += [build_core([[I, 0], [L, I]]) for _ in range(1, d - 1)]
    cores.append(build_core([I, L]))
    return cores


def coupled_op(d: int, n: int, coupling: np.ndarray, h: float = 0.2, shift: float = 1.0) -> List[np.ndarray]:
    """``sum_i L_i + shift * I + sum_i c_i D_i D_{i+1}`` as a rank-4 TT operator
    with states {before, D pending, Laplacian done, coupling done}."""
    L, I = laplacian(n, h), np.eye(n)
    D = np.diag(np.linspace(-1.0, 1.0, n))
    cores = [build_core([[I, coupling[0] * D, L + shift * I, 0]])]
    for i in range(1, d - 1):
        cores.append(build_core([[I, coupling[i] * D, L, 0], [0, 0, 0, D], [0, 0, I, 0], [0, 0, 0, I]]))
    cores.append(build_core([L, D, I, I]))
    return cores


def gaussian_tt(rng, d: int, n: int, r: int) -> List[np.ndarray]:
    ranks = [1] + [r] * (d - 1) + [1]
    return [rng.standard_normal((ranks[i], n, 1, ranks[i + 1])) for i in range(d)]


def ising_op(d: int, coupling: float, field_: float) -> List[np.ndarray]:
    S = -field_ * np.array([[0.0, 1.0], [1.0, 0.0]])
    Z = np.array([[1.0, 0.0], [0.0, -1.0]])
    I = np.eye(2)
    M = -coupling * Z
    cores = [build_core([[S, Z, I]])]
    cores += [build_core([[I, 0, 0], [M, 0, 0], [S, Z, I]]) for _ in range(1, d - 1)]
    cores.append(build_core([I, M, S]))
    return cores


def uniform_tt(state, d: int, n: int, r: int) -> List[np.ndarray]:
    """``tt.rand`` cores: U[0,1) in core order from a legacy RandomState."""
    ranks = [1] + [r] * (d - 1) + [1]
    return [state.rand(ranks[i], n, 1, ranks[i + 1]) for i in range(d)]


@dataclass
class SLEInstance:
    op: List[np.ndarray]
    rhs: List[np.ndarray]
    x0: List[np.ndarray]
    repeats: int
    meta: dict = field(default_factory=dict)


@dataclass
class EVPInstance:
    op: List[np.ndarray]
    x0: List[np.ndarray]
    repeats: int
    sigma: float
    meta: dict = field(default_factory=dict)


def laplace_sle(d=10, n=4, rhs_rank=3, x_rank=5, repeats=2, seed=0) -> SLEInstance:
    rng = np.random.default_rng(seed)
    rhs = gaussian_tt(rng, d, n, rhs_rank)
    x0 = gaussian_tt(rng, d, n, x_rank)
    return SLEInstance(laplace_op(d, n), rhs, x0, repeats, dict(d=d, n=n, rhs_rank=rhs_rank, x_rank=x_rank))


def coupled_sle(d=32, n=8, rhs_rank=8, x_rank=32, repeats=4, seed=0) -> SLEInstance:
    c = np.random.default_rng(seed).uniform(0.0, 0.5, d)
    rng = np.random.default_rng(seed)
    rhs = gaussian_tt(rng, d, n, rhs_rank)
    x0 = gaussian_tt(rng, d, n, x_rank)
    return SLEInstance(coupled_op(d, n, c), rhs, x0, repeats, dict(d=d, n=n, rhs_rank=rhs_rank, x_rank=x_rank))


def ising_evp(d=48, g=1.0, x_rank=64, repeats=6, seed=1) -> EVPInstance:
    x0 = uniform_tt(np.random.RandomState(seed), d, 2, x_rank)
    sigma = -(d - 1) - g * d - 1.0   # below the spectrum: lowest eigenpair
    return EVPInstance(ising_op(d, 1.0, g), x0, repeats, sigma, dict(d=d, g=g, x_rank=x_rank))


@dataclass
class TDVPInstance:
    op: List[np.ndarray]
    x0: List[np.ndarray]
    step_size: complex
    steps: int
    max_rank: int
    meta: dict = field(default_factory=dict)


def right_orthonormal(cores: List[np.ndarray]) -> List[np.ndarray]:
    """RQ sweep from the right (tensor_train.py:1262-1296 without truncation),
    then the first core scaled to unit norm."""
    cores = [c.copy() for c in cores]
    for i in range(len(cores) - 1, 0, -1):
        r, n, m, s = cores[i].shape
        q, rr = np.linalg.qr(cores[i].reshape(r, n * m * s).T)
        k = q.shape[1]
        cores[i] = q.T.reshape(k, n, m, s)
        cores[i - 1] = np.tensordot(cores[i - 1], rr.T, axes=(3, 0))
    cores[0] = cores[0] / np.linalg.norm(cores[0])
    return cores


def tdvp_ising(d=16, g=1.2, x_rank=4, max_rank=16, steps=5, dt=0.05, seed=7) -> TDVPInstance:
    """Imaginary-time two-site TDVP on the transverse-field Ising chain from a
    random right-orthonormal rank-``x_rank`` state (step_size = -1j * dt)."""
    x0 = right_orthonormal(gaussian_tt(np.random.default_rng(seed), d, 2, x_rank))
    return TDVPInstance(ising_op(d, 1.0, g), x0, -1j * dt, steps, max_rank,
                        dict(d=d, g=g, x_rank=x_rank, max_rank=max_rank, dt=dt))


@dataclass
class ARRInstance:
    x: np.ndarray            # samples (coordinates x samples)
    y: np.ndarray            # outputs x samples
    basis: list              # basis functions per mode
    x0: List[np.ndarray]     # initial guess (one per output, copied)
    repeats: int
    rcond: float
    meta: dict = field(default_factory=dict)


def kuramoto_arr(d=10, m=1000, repeats=10, rcond=1e-12, seed=3) -> ARRInstance:
    """Alternating ridge regression of the Kuramoto model's right-hand side
    from d oscillator phases (the setting of the reference's ARR test): m
    samples of one trajectory (scipy BDF), bases [1, sin x_1 .. sin x_d] and
    [1, cos x_1 .. cos x_d], rank d+1, one regression per oscillator."""
    import scipy.integrate as spint
    from .data_driven import transform as tdt
    rng = np.random.default_rng(seed)
    x0 = 2 * np.pi * rng.random(d) - np.pi
    w = np.linspace(-5, 5, d)

    def rhs(_, theta):
        ti, tj = np.meshgrid(theta, theta)
        return w + 2 / d * np.sin(tj - ti).sum(0) + 0.2 * np.sin(theta)

    sol = spint.solve_ivp(rhs, [0, 100], x0, method='BDF', t_eval=np.linspace(0, 100, m))
    x = sol.y
    y = np.stack([rhs(0, x[:, j]) for j in range(m)], axis=1)
    basis = [[tdt.ConstantFunction(0)] + [tdt.Sin(i, 1) for i in range(d)],
             [tdt.ConstantFunction(0)] + [tdt.Cos(i, 1) for i in range(d)]]
    guess = [np.ones((1, d + 1, 1, d + 1)), np.ones((d + 1, d + 1, 1, 1))]
    return ARRInstance(x, y, basis, guess, repeats, rcond, dict(d=d, m=m))


def reversible_markov(rng, n: int) -> np.ndarray:
    """Column-stochastic n x n transition matrix S D^-1 of a reversible chain
    (S symmetric positive, D its column sums): similar to the symmetric
    D^-1/2 S D^-1/2, so its spectrum is real, with the Perron root 1."""
    s = rng.uniform(0.05, 1.0, (n, n))
    s = s + s.T
    return s / s.sum(axis=0, keepdims=True)


def markov_op(d: int, n: int, eps: float, rng) -> List[np.ndarray]:
    """Nonsymmetric rank-2 TT operator (P_1 x ... x P_d + eps Q_1 x ... x Q_d) / (1 + eps)
    of reversible transition matrices: column-stochastic, dominant eigenvalue 1,
    the leading eigenvalues real (a small perturbation of a real spectrum); the
    shape of the Ulam transfer operators that evp.als is applied to."""
    ps = [reversible_markov(rng, n) for _ in range(d)]
    qs = [reversible_markov(rng, n) for _ in range(d)]
    cores = []
    for i in range(d):
        if i == 0:
            c = np.zeros((1, n, n, 2))
            c[0, :, :, 0] = ps[i] / (1.0 + eps)
            c[0, :, :, 1] = qs[i] * eps / (1.0 + eps)
        elif i == d - 1:
            c = np.zeros((2, n, n, 1))
            c[0, :, :, 0] = ps[i]
            c[1, :, :, 0] = qs[i]
        else:
            c = np.zeros((2, n, n, 2))
            c[0, :, :, 0] = ps[i]
            c[1, :, :, 1] = qs[i]
        cores.append(c)
    return cores


def markov_evp(d=4, n=4, eps=0.2, x_rank=6, repeats=4, seed=3) -> EVPInstance:
    """Leading eigenvalues of a nonsymmetric transfer operator ('eig' near sigma=1)."""
    rng = np.random.default_rng(seed)
    op = markov_op(d, n, eps, rng)
    x0 = [np.abs(c) + 0.1 for c in gaussian_tt(rng, d, n, x_rank)]
    return EVPInstance(op, x0, repeats, 1.0, dict(d=d, n=n, eps=eps, x_rank=x_rank))


def batch_instance(j: int, repeats: int = 4) -> SLEInstance:
    rng = np.random.default_rng(1000 + j)
    d = int(rng.integers(8, 33))
    n = int(rng.choice([2, 4, 8]))
    r = int(rng.integers(4, 49))
    shift = float(rng.uniform(0.5, 2.0))
    c = rng.uniform(0.0, 0.5, d)
    op = coupled_op(d, n, c, shift=shift)
    rhs = gaussian_tt(rng, d, n, 4)
    x0 = gaussian_tt(rng, d, n, r)
    return SLEInstance(op, rhs, x0, repeats, dict(j=j, d=d, n=n, r=r, shift=shift))


def batch_sle(count: int = 256, repeats: int = 4) -> List[SLEInstance]:
    return [batch_instance(j, repeats) for j in range(count)]


def serving_stream(rate: float = 2000.0, duration: float = 60.0, seed: int = 5, sle_fraction: float = 0.8,
                   max_requests: int = None):
    """Yields ``(arrival_time_s, kind, instance)`` in arrival order."""
    rng = np.random.default_rng(seed)
    t, k = 0.0, 0
    while True:
        t += float(rng.exponential(1.0 / rate))
        if t > duration or (max_requests is not None and k >= max_requests):
            return
        if rng.uniform() < sle_fraction:
            yield t, 'sle', batch_instance(int(rng.integers(0, 1 << 30)))
        else:
            d = int(rng.integers(16, 49))
            r = int(rng.integers(16, 65))
            g = float(rng.uniform(0.5, 1.5))
            inst = ising_evp(d=d, g=g, x_rank=r, repeats=6, seed=int(rng.integers(0, 1 << 30)))
            yield t, 'evp', inst
        k += 1
