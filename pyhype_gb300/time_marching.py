"""Explicit Runge-Kutta tableaux with the reference's integrator names.

Rows follow ``ExplicitRungeKutta`` (``pyhype/time_marching/explicit_runge_kutta.py:
91-274``): ``len(a)`` stages, row s holds the weights of k_0..k_s for the state after
stage s, the last row being the step update.  Coefficients are the same Python float
expressions (``1/6`` etc.) so ``dt * a`` rounds identically.  ``SSPRK2`` is the
two-stage strong-stability-preserving method in this Butcher-row form
(``[[1], [0.5, 0.5]]``), which the reference has no name for.
``Generic2``/``Generic3`` read ``config.alpha``, an attribute the reference's
``SolverConfig`` does not define; here ``alpha`` is taken as an argument.
"""
from __future__ import annotations

from typing import List, Optional

import numpy as np

_ROWS = {
    "ExplicitEuler1": [[1]],
    "RK2": [[0.5], [0, 1]],
    "Ralston2": [[2 / 3], [1 / 4, 3 / 4]],
    "RK3": [[0.5], [-1, 2], [1 / 6, 2 / 3, 1 / 6]],
    "RK3SSP": [[1], [1 / 4, 1 / 4], [1 / 6, 1 / 6, 2 / 3]],
    "Ralston3": [[1 / 2], [0, 3 / 4], [2 / 9, 1 / 3, 4 / 9]],
    "RK4": [[0.5], [0, 0.5], [0, 0, 1], [1 / 6, 1 / 3, 1 / 3, 1 / 6]],
    "Ralston4": [
        [0.4],
        [0.29697761, 0.15875964],
        [0.21810040, -3.05096516, 3.83286476],
        [0.17476028, -0.55148066, 1.20553560, 0.17118478],
    ],
    "DormandPrince5": [
        [1 / 5],
        [3 / 40, 9 / 40],
        [44 / 45, -56 / 15, 32 / 9],
        [19372 / 6561, -25360 / 2187, 64448 / 6561, -212 / 729],
        [9017 / 3168, -355 / 33, 46732 / 5247, 49 / 176, -5103 / 18656],
        [35 / 384, 0, 500 / 1113, 125 / 192, -2187 / 6784, 11 / 84],
    ],
    "SSPRK2": [[1], [0.5, 0.5]],
}


def rows(name: str, alpha: Optional[float] = None) -> List[List[float]]:
    if name == "Generic2":
        if alpha is None:
            raise ValueError("Generic2 needs alpha")
        a = alpha
        return [[a], [1 - 1 / (2 * a), 1 / (2 * a)]]
    if name == "Generic3":
        if alpha is None:
            raise ValueError("Generic3 needs alpha")
        a = alpha
        if a in (0, 2 / 3, 1):
            raise ValueError("Value of alpha parameter is not allowd.")
        k = (1 - a) / a / (3 * a - 2)
        return [[a], [1 + k, -k], [0.5 - 1 / (6 * a), 1 / (6 * a * (1 - a)), (2 - 3 * a) / (6 * (1 - a))]]
    if name not in _ROWS:
        raise ValueError(f"Time marching scheme {name} is not available.")
    return _ROWS[name]


def square(a_rows) -> np.ndarray:
    n = len(a_rows)
    out = np.zeros((n, n))
    for i, r in enumerate(a_rows):
        out[i, : len(r)] = r
    return out


def tableau(name: str, alpha: Optional[float] = None) -> np.ndarray:
    """Square (S x S) lower-triangular array of the named integrator's rows."""
    return square(rows(name, alpha))


class ExplicitRungeKutta:
    """Reference-compatible constructor: ``ExplicitRungeKutta(config, a=[[...], ...])``."""

    def __init__(self, config=None, a=None):
        if a is None:
            raise ValueError("a Butcher row list is required")
        self.config = config
        self.a = a
        self.num_stages = len(a)

    def tableau(self) -> np.ndarray:
        return square(self.a)

    @classmethod
    def named(cls, config, name: str, alpha: Optional[float] = None):
        return cls(config, a=rows(name, alpha))


class TimeIntegratorFactory:
    @classmethod
    def create(cls, config, **kwargs):
        return ExplicitRungeKutta.named(config, config.time_integrator, getattr(config, "alpha", None))
