"""Ideal-gas fluid description (host side).

Same interface and constants as ``pyhype/fluids/base.py:27-64`` and
``pyhype/fluids/air.py:24-28``: gamma = 1.4, far-field speed of sound and density used
for non-dimensionalisation.  ``gamma()-1``, ``g/(g-1)`` and ``1/(g-1)`` are formed by
the same double-precision operations, so the constants handed to the kernels are the
reference's own bit patterns (``0.3999999999999999`` for gamma-1, for instance).
"""
from __future__ import annotations

from collections import namedtuple

_FarField = namedtuple("far_field", ["a", "rho"])


class Fluid:
    gas_constant = 8314.0
    _molecular_mass = float("-inf")
    _gamma = None

    def __init__(self, a_inf: float = 1.0, rho_inf: float = 1.0):
        self._far_field = _FarField(a_inf, rho_inf)
        self._R = self.gas_constant / self.molecular_mass

    @property
    def far_field(self):
        return self._far_field

    @property
    def R(self):
        return self._R

    @property
    def molecular_mass(self):
        return self._molecular_mass

    def gamma(self, *args, **kwargs) -> float:
        if self._gamma is None:
            raise NotImplementedError("Fluid subclasses define gamma")
        return self._gamma

    def g_over_gm1(self, *args, **kwargs) -> float:
        g = self.gamma()
        return g / (g - 1.0)

    def one_over_gm1(self, *args, **kwargs) -> float:
        g = self.gamma()
        return 1.0 / (g - 1.0)

    def gm1(self) -> float:
        return self.gamma() - 1


class Air(Fluid):
    _molecular_mass = 28.97
    _gamma = 1.4
