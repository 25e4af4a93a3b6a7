from .base import BoundaryCondition, DeviceBoundaryCondition, PrimitiveDirichletBC, SwitchedBC

__all__ = ["BoundaryCondition", "DeviceBoundaryCondition", "PrimitiveDirichletBC", "SwitchedBC"]
