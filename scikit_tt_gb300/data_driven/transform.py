"""Basis functions R^d -> R for the data-driven solvers.

The call semantics of scikit_tt/data_driven/transform.py:15-470 for the
one-coordinate functions (``f(t)`` for a sample vector ``t``), which is all
``regression.arr`` evaluates (regression.py:323-326): constant, identity,
monomial, sine, cosine, Gaussian and Legendre polynomial of one coordinate.
Derivatives and the tensor-product transformations are not part of the
device path and are not provided.  Any callable ``f(t) -> float`` works as a
basis function as well.
"""

from __future__ import annotations

import numpy as np


class Function:
    """Function R^n -> R (transform.py:15-93): checks the input dimension on
    the first call when none was given."""

    def __init__(self, dimension: int = None):
        if dimension is None:
            self.dimension = 1
            self.initialized = False
        else:
            if dimension < 1:
                raise ValueError('dimension has to be >= 1')
            self.dimension = dimension
            self.initialized = True

    def check_call_input(self, t):
        if not self.initialized:
            self.dimension = len(t)
            self.initialized = True

    def __call__(self, t):
        self.check_call_input(t)
        return 0


class OneCoordinateFunction(Function):
    """Function depending on coordinate ``index`` only (transform.py:96-165)."""

    def __init__(self, index: int, dimension: int = None):
        super().__init__(dimension)
        if self.initialized and not 0 <= index < self.dimension:
            raise ValueError('index has to be >= 0 and < dimension')
        self.index = index

    def check_call_input(self, t):
        if not self.initialized:
            self.dimension = len(t)
            if not 0 <= self.index < self.dimension:
                raise ValueError('index has to be >= 0 and < dimension')
            self.initialized = True


class ConstantFunction(OneCoordinateFunction):
    """1 (transform.py:168-197)."""

    def __call__(self, t):
        self.check_call_input(t)
        if np.isscalar(t[self.index]):
            return 1.0
        return np.ones(np.shape(t[self.index]))


class Identity(OneCoordinateFunction):
    """t[index] (transform.py:229-253)."""

    def __call__(self, t):
        self.check_call_input(t)
        return t[self.index]


class Monomial(OneCoordinateFunction):
    """prefactor * t[index] ** exponent (transform.py:256-290)."""

    def __init__(self, index: int, exponent: int, prefactor=1, dimension: int = None):
        super().__init__(index, dimension)
        if exponent < 0:
            raise ValueError('exponent has to be >= 0')
        self.exponent = exponent
        self.prefactor = prefactor

    def __call__(self, t):
        self.check_call_input(t)
        return self.prefactor * t[self.index] ** self.exponent


class Sin(OneCoordinateFunction):
    """sin(alpha * t[index]) (transform.py:330-360)."""

    def __init__(self, index: int, alpha: float, dimension: int = None):
        super().__init__(index, dimension)
        self.alpha = alpha

    def __call__(self, t):
        self.check_call_input(t)
        return np.sin(self.alpha * t[self.index])


class Cos(OneCoordinateFunction):
    """cos(alpha * t[index]) (transform.py:363-393)."""

    def __init__(self, index: int, alpha: float, dimension: int = None):
        super().__init__(index, dimension)
        self.alpha = alpha

    def __call__(self, t):
        self.check_call_input(t)
        return np.cos(self.alpha * t[self.index])


class GaussFunction(OneCoordinateFunction):
    """exp(-(t[index] - mean)^2 / (2 variance)) (transform.py:396-435)."""

    def __init__(self, index: int, mean: float, variance: float, dimension: int = None):
        super().__init__(index, dimension)
        if variance <= 0:
            raise ValueError('variance has to be > 0')
        self.mean = mean
        self.variance = variance

    def __call__(self, t):
        self.check_call_input(t)
        return np.exp(-0.5 * (t[self.index] - self.mean) ** 2 / self.variance)


class Legendre(OneCoordinateFunction):
    """Legendre polynomial P_degree(t[index] / domain) (transform.py:293-327)."""

    def __init__(self, index: int, degree: int, domain: float = 1.0, dimension: int = None):
        super().__init__(index, dimension)
        if degree < 0:
            raise ValueError('degree has to be >= 0')
        self.degree = degree
        self.domain = domain
        self._coef = np.zeros(degree + 1)
        self._coef[degree] = 1.0

    def __call__(self, t):
        self.check_call_input(t)
        return np.polynomial.legendre.legval(t[self.index] / self.domain, self._coef)
