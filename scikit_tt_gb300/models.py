"""Operator builders used as ALS inputs (scikit_tt/models.py)."""

from __future__ import annotations

import numpy as np

from .tensor_train import TT, build_core


def ising(d, J, h) -> TT:
    """Transverse-field Ising chain ``H = -J sum z_i z_{i+1} - h sum x_i`` as a
    rank-3 TT operator (scikit_tt/models.py:10-44): first core ``[[S, L, I]]``,
    middle ``[[I, 0, 0], [M, 0, 0], [S, L, I]]``, last ``[I, M, S]`` with
    ``S = -h sigma_x``, ``L = sigma_z``, ``M = -J sigma_z``."""
    S = -h * np.array([[0.0, 1.0], [1.0, 0.0]])
    L = np.array([[1.0, 0.0], [0.0, -1.0]])
    I = np.eye(2)
    M = -J * np.array([[1.0, 0.0], [0.0, -1.0]])
    cores = [build_core([[S, L, I]])]
    for _ in range(1, d - 1):
        cores.append(build_core([[I, 0, 0], [M, 0, 0], [S, L, I]]))
    cores.append(build_core([I, M, S]))
    return TT(cores)
