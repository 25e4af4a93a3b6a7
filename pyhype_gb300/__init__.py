"""GB300 (sm_103a) implementation of pyHype's 2D Euler MUSCL finite-volume residual
and explicit Runge-Kutta time stepping, behind pyHype's ``Euler2D`` API.

Reference-compatible entry points::

    from pyhype_gb300.solvers import Euler2D
    from pyhype_gb300.solver_config import SolverConfig
    from pyhype_gb300.fluids import Air
    from pyhype_gb300.states import ConservativeState, PrimitiveState
    from pyhype_gb300.mesh.rectangular import RectagularMeshGenerator
    from pyhype_gb300.initial_conditions.base import InitialCondition

The numerics run in libeuler2d.so (include/euler2d.h); there is no CPU fallback.
"""
__version__ = "0.1.0"


def __getattr__(name):
    if name == "Euler2D":
        from .solvers import Euler2D

        return Euler2D
    if name == "SolverConfig":
        from .solver_config import SolverConfig

        return SolverConfig
    raise AttributeError(name)
