"""Builders for the benchmark configurations (config + mesh, reference keyword API).

* ``explosion``            single block, [0,10]^2, Reflection walls (n x n cells)
* ``explosion_multiblock`` [0,10]x[0,20] as 2x4 blocks of n x n cells
* ``double_mach``          Mach-10 double-Mach reflection on [0,4]x[0,1] as a row of
                           blocks: post-shock inflow west and south for x < 1/6, wall
                           for x >= 1/6, exact moving-shock state on the north side,
                           outflow east; HLLL, Venkatakrishnan, SSP-RK2, CFL 0.4,
                           primitive reconstruction, unit far field (t is physical).
"""
from __future__ import annotations

import numpy as np

from .boundary_conditions import PrimitiveDirichletBC, SwitchedBC
from .fluids import Air
from .initial_conditions import ExplosionInitialCondition, InitialCondition
from .mesh import QuadMeshGenerator, RectagularMeshGenerator
from .solver_config import SolverConfig
from .states import ConservativeState, PrimitiveState

DMR_PRE = [1.4, 0.0, 0.0, 1.0]
DMR_POST = [8.0, 8.25 * np.cos(np.pi / 6), -8.25 * np.sin(np.pi / 6), 116.5]


def _config(nx, ny, ic, fluid, **kw):
    base = dict(
        fvm_type="MUSCL", fvm_spatial_order=2, fvm_num_quadrature_points=1, fvm_gradient_type="GreenGauss",
        fvm_flux_function_type="Roe", fvm_slope_limiter_type="Venkatakrishnan", time_integrator="RK4",
        interface_interpolation="arithmetic_average", reconstruction_type=ConservativeState, CFL=0.8,
        t_final=0.07, nghost=1,
    )
    base.update(kw)
    return SolverConfig(nx=nx, ny=ny, initial_condition=ic, fluid=fluid, **base)


def explosion(n: int = 100, **kw):
    air = Air(a_inf=343.0, rho_inf=1.0)
    blk = {
        "nBLK": 0, "NW": [0, 10], "NE": [10, 10], "SW": [0, 0], "SE": [10, 0],
        "NeighborE": None, "NeighborW": None, "NeighborN": None, "NeighborS": None,
        "NeighborNE": None, "NeighborNW": None, "NeighborSE": None, "NeighborSW": None,
        "BCTypeE": "Reflection", "BCTypeW": "Reflection", "BCTypeN": "Reflection", "BCTypeS": "Reflection",
        "BCTypeNE": None, "BCTypeNW": None, "BCTypeSE": None, "BCTypeSW": None,
    }
    return _config(n, n, ExplosionInitialCondition(), air, **kw), {0: blk}


def explosion_multiblock(n: int = 150, **kw):
    air = Air(a_inf=343.0, rho_inf=1.0)
    mesh = RectagularMeshGenerator.generate(["Reflection"], ["Reflection"], ["Reflection"], ["Reflection"],
                                            east=10.0, west=0.0, north=20.0, south=0.0,
                                            n_blocks_horizontal=2, n_blocks_vertical=4)
    return _config(n, n, ExplosionInitialCondition(), air, **kw), mesh


class DoubleMachInitialCondition(InitialCondition):
    """Post-shock state left of the 60-degree shock through (1/6, 0), pre-shock right."""

    def apply_to_block(self, block):
        fl = block.config.fluid
        post = PrimitiveState(fluid=fl, array=np.array(DMR_POST).reshape((1, 1, 4))).to_type(ConservativeState)
        pre = PrimitiveState(fluid=fl, array=np.array(DMR_PRE).reshape((1, 1, 4))).to_type(ConservativeState)
        block.state.data = np.where(block.mesh.x < 1 / 6 + block.mesh.y / np.sqrt(3), post.data, pre.data)
        block.state.make_non_dimensional()


def double_mach_bcs():
    """(west, south, north) boundary-condition factories of the double-Mach setup."""
    west = lambda: PrimitiveDirichletBC(PrimitiveState(Air(1.0, 1.0), array=np.array(DMR_POST).reshape(1, 1, 4)))  # noqa: E731
    south = lambda: SwitchedBC(1 / 6, 0.0, DMR_POST, "Reflection")  # noqa: E731
    north = lambda: SwitchedBC(1 / 6 + 1 / np.sqrt(3), 20 / np.sqrt(3), DMR_POST, DMR_PRE)  # noqa: E731
    return west, south, north


def double_mach(nx: int = 400, ny: int = 500, nblk: int = 5, **kw):
    fluid = Air(a_inf=1.0, rho_inf=1.0)
    west, south, north = double_mach_bcs()
    gen = QuadMeshGenerator(nx_blk=nblk, ny_blk=1, BCE=["OutletDirichlet"], BCW=[west()],
                            BCN=[north() for _ in range(nblk)], BCS=[south() for _ in range(nblk)],
                            SW=(0.0, 0.0), SE=(4.0, 0.0), NW=(0.0, 1.0), NE=(4.0, 1.0))
    opts = dict(fvm_flux_function_type="HLLL", reconstruction_type=PrimitiveState, time_integrator="SSPRK2",
                CFL=0.4, t_final=0.2)
    opts.update(kw)
    return _config(nx, ny, DoubleMachInitialCondition(), fluid, **opts), gen
