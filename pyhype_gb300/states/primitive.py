from __future__ import annotations

import numpy as np

from .base import State


class PrimitiveState(State):
    """(rho, u, v, p) per cell."""

    RHO_IDX, U_IDX, V_IDX, P_IDX = 0, 1, 2, 3

    @property
    def rho(self):
        return self._data[:, :, 0]

    @property
    def u(self):
        return self._data[:, :, 1]

    @property
    def v(self):
        return self._data[:, :, 2]

    @property
    def p(self):
        return self._data[:, :, 3]

    def Ek(self):
        u, v = self.u, self.v
        return 0.5 * (u * u + v * v)

    def ek(self):
        # (0.5 * rho) * (u*u + v*v), the grouping of pyhype/states/primitive.py:97-101
        W = self._data
        return 0.5 * W[:, :, 0] * (W[:, :, 1] * W[:, :, 1] + W[:, :, 2] * W[:, :, 2])

    def a(self):
        return np.sqrt(self.fluid.gamma() * self.p / self.rho)

    def realizability_conditions(self):
        return dict(rho_good=self.rho > 0, pressure_good=self.p > 0)
