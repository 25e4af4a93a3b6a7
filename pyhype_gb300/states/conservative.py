from __future__ import annotations

import numpy as np

from .base import State


class ConservativeState(State):
    """(rho, rho*u, rho*v, E) per cell."""

    RHO_IDX, RHOU_IDX, RHOV_IDX, E_IDX = 0, 1, 2, 3

    @property
    def rho(self):
        return self._data[:, :, 0]

    @property
    def rhou(self):
        return self._data[:, :, 1]

    @property
    def rhov(self):
        return self._data[:, :, 2]

    @property
    def e(self):
        return self._data[:, :, 3]

    @property
    def u(self):
        return self._data[:, :, 1] / self.rho

    @property
    def v(self):
        return self._data[:, :, 2] / self.rho

    def Ek(self):
        u, v = self.u, self.v
        return 0.5 * (u * u + v * v)

    def ek(self):
        return self.rho * self.Ek()

    @property
    def p(self):
        return self.fluid.gm1() * (self.e - self.ek())

    def a(self):
        return np.sqrt(self.fluid.gamma() * self.p / self.rho)

    def realizability_conditions(self):
        return dict(rho_good=self.rho > 0, energy_good=self.e > 0)
