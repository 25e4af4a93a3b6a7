"""Boundary conditions that run on the device.

The reference applies boundary conditions as host callables on a ghost ``State``
(``pyhype/boundary_conditions/base.py:26-44``, ``pyhype/blocks/ghost.py:128-158``).
Here a boundary condition is data: each ``DeviceBoundaryCondition`` resolves to a side
kind of ``include/euler2d.h`` plus the constant states the kernels need.  The built-in
string kinds ("Reflection", "Slipwall", "OutletDirichlet", ``None``) need no object.
"""
from __future__ import annotations

import numpy as np

from ..states import ConservativeState, PrimitiveState


class BoundaryCondition:
    """Base class with the reference's call interface; host-only subclasses are
    rejected when a solver is built (they cannot run inside the GPU time loop)."""

    def __call__(self, state, *args, **kwargs):
        self._apply_boundary_condition(state, *args, **kwargs)

    def _apply_boundary_condition(self, state, *args, **kwargs):
        raise NotImplementedError


class DeviceBoundaryCondition(BoundaryCondition):
    def side_spec(self, recon: int, fluid, geometry, side: str):
        raise NotImplementedError


def _dirichlet_vectors(primitive_nd: np.ndarray, recon: int, fluid):
    """Ghost (conservative) and outside-face (reconstruction variables) states of a
    fixed primitive state, converted the way the reference's ``State.from_state``
    would convert them for the ghost block and for the boundary face state."""
    w = PrimitiveState(fluid=fluid, array=np.asarray(primitive_nd, dtype=np.float64).reshape(1, 1, 4).copy())
    ghost = w.to_type(ConservativeState).data.reshape(4)
    if recon == 1:
        face = w.data.reshape(4).copy()
        # the reconstruction block converts the conservative ghost back to primitive
        ghost_recon_src = ghost
    else:
        face = ghost.copy()
        ghost_recon_src = ghost
    return ghost.copy(), face, ghost_recon_src


class PrimitiveDirichletBC(DeviceBoundaryCondition):
    """Fixed primitive state on a side (``pyhype/boundary_conditions/bc.py:26-35``).

    The reference's version raises on a uniform ``(1, 1, 4)`` state when applied to a
    ghost of a different shape (its ``from_state`` checks shapes); this one accepts the
    uniform state, which is what every reference example passes."""

    def __init__(self, primitive_state: PrimitiveState):
        if not isinstance(primitive_state, PrimitiveState):
            raise TypeError("primitive_array must be a PrimitiveState.")
        super().__init__()
        self._primitive_state = primitive_state
        self._primitive_state.make_non_dimensional()

    def side_spec(self, recon: int, fluid, geometry, side: str):
        from ..problem import SIDE_DIRICHLET, SideSpec

        ghost, face, _ = _dirichlet_vectors(self._primitive_state.data.reshape(4), recon, fluid)
        return SideSpec(SIDE_DIRICHLET, ghost=ghost, face=face)

    def _apply_boundary_condition(self, state, *args, **kwargs):
        state.data = np.broadcast_to(
            self._primitive_state.to_type(type(state)).data, state.shape).copy()


class SwitchedBC(DeviceBoundaryCondition):
    """Per-cell choice along one side between two kinds ("Reflection" or a primitive
    Dirichlet state), switched where the centroid coordinate along the side crosses
    ``x0 + speed * t`` (t = non-dimensional solver time).  Used for the
    double-Mach-reflection walls, inflow and exact-shock top boundary."""

    def __init__(self, x0: float, speed: float, below, above):
        self.x0, self.speed, self.below, self.above = float(x0), float(speed), below, above

    def _kind(self, spec, recon, fluid):
        from ..problem import SIDE_DIRICHLET, SIDE_REFLECT

        if isinstance(spec, str):
            if spec in ("Reflection", "Slipwall"):
                return SIDE_REFLECT, np.zeros(4), np.zeros(4)
            raise ValueError(spec)
        ghost, face, _ = _dirichlet_vectors(np.asarray(spec, dtype=np.float64), recon, fluid)
        return SIDE_DIRICHLET, ghost, face

    def side_spec(self, recon: int, fluid, geometry, side: str):
        from ..problem import SIDE_MIXED, SideSpec

        kb, gb, fb = self._kind(self.below, recon, fluid)
        ka, ga, fa = self._kind(self.above, recon, fluid)
        if side in ("N", "S"):
            coord = geometry.xc[-1 if side == "N" else 0, :]
        else:
            coord = geometry.yc[:, -1 if side == "E" else 0]
        return SideSpec(SIDE_MIXED, mixed=dict(
            x0=self.x0, speed=self.speed, kind_below=kb, kind_above=ka,
            ghost_below=gb, face_below=fb, ghost_above=ga, face_above=fa, coord=coord.copy()))
