"""Initial conditions of the reference's examples, for the benchmark configurations.

``ExplosionInitialCondition`` is the high-pressure square of
``examples/explosion/initial_condition.py:32-61`` (pressure 404400 / density 4.6968
inside ``lo <= x, y <= hi``, 101100 / 1.1742 outside, at rest, non-dimensionalised by
the fluid's far field); ``SupersonicFloodInitialCondition`` is
``pyhype/initial_conditions/supersonic_flood.py``.
"""
from __future__ import annotations

import numpy as np

from ..states import ConservativeState, PrimitiveState
from .base import InitialCondition


class ExplosionInitialCondition(InitialCondition):
    def __init__(self, lo: float = 3.0, hi: float = 7.0, rho_in: float = 4.6968, p_in: float = 404400.0,
                 rho_out: float = 1.1742, p_out: float = 101100.0, u: float = 0.0, v: float = 0.0):
        self.lo, self.hi = lo, hi
        self.inside = (rho_in, u, v, p_in)
        self.outside = (rho_out, u, v, p_out)

    def apply_to_block(self, block):
        fluid = block.config.fluid
        left = PrimitiveState(fluid=fluid, array=np.array(self.inside, dtype=float).reshape((1, 1, 4))).to_type(ConservativeState)
        right = PrimitiveState(fluid=fluid, array=np.array(self.outside, dtype=float).reshape((1, 1, 4))).to_type(ConservativeState)
        xc = np.logical_and(block.mesh.x >= self.lo, block.mesh.x <= self.hi)
        yc = np.logical_and(block.mesh.y >= self.lo, block.mesh.y <= self.hi)
        block.state.data = np.where(np.logical_and(xc, yc), left.data, right.data)
        block.state.make_non_dimensional()


class SupersonicFloodInitialCondition(InitialCondition):
    def __init__(self, fluid, rho: float, u: float, v: float, p: float):
        if rho <= 0 or p <= 0:
            raise ValueError(f"Unrealizable density (rho={rho}) or pressure (p={p}).")
        a = np.sqrt(fluid.gamma() * p / rho)
        if np.hypot(u, v) / a < 1.0:
            raise ValueError("The given set of conditions do not produce a supersonic flow")
        self._state = (rho, u, v, p)

    def apply_to_block(self, block):
        s = PrimitiveState(fluid=block.config.fluid,
                           array=np.array(self._state, dtype=float).reshape((1, 1, 4))).to_type(ConservativeState)
        block.state.data = s.data
        block.state.make_non_dimensional()
