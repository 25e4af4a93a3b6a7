"""Generate the golden fixtures in this directory by running the pyHype reference itself.

The reference (pure Python + numba + mpi4py + matplotlib) is imported unmodified from
its source tree through the import shim in ``_refshim.py`` (identity ``njit``, a
one-rank MPI world, stub plotting).  Each case builds an ``Euler2D`` solver with the
reference's own ``SolverConfig``/mesh dictionaries/initial conditions, runs the
reference's own step loop (``Solver.get_dt`` -> ``ExplicitRungeKutta.integrate`` ->
``t += dt``; ``pyhype/solvers/Euler2D.py:175-216``) and records:

* the initial conservative state of every block (after ``_pre_process_solve``),
* the dt of every step and a fingerprint of the state after every step,
* full states after selected steps,
* for ``ops_*`` cases, the per-operator intermediates of one residual evaluation
  (gradients, limiter, the primitive L/R face states fed to the flux, the fluxes and
  dUdt) captured from the reference objects,
* the reference's mesh geometry (to pin the host geometry builder bit for bit).

Usage (in a container that holds the reference sources)::

    python tests/golden/make_golden.py            # every case
    python tests/golden/make_golden.py p100 m2x4_40

The fixtures are committed; this script is the record of how they were made.
"""
from __future__ import annotations

import hashlib
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import _refshim  # noqa: E402

_refshim.install()
sys.path.insert(0, _refshim.REFERENCE_ROOT)

from pyhype.solvers import Euler2D  # noqa: E402
from pyhype.solver_config import SolverConfig  # noqa: E402
from pyhype.fluids import Air  # noqa: E402
from pyhype.states import ConservativeState, PrimitiveState  # noqa: E402
from pyhype.mesh.rectangular import RectagularMeshGenerator  # noqa: E402
from pyhype.initial_conditions.base import InitialCondition  # noqa: E402
from pyhype.time_marching.explicit_runge_kutta import ExplicitRungeKutta  # noqa: E402
from pyhype.utils.utils import Direction  # noqa: E402


# --------------------------------------------------------------------------------------
# fingerprints (shared with the tests: a canonical +0.0 is added so -0.0 == +0.0)
# --------------------------------------------------------------------------------------
def fingerprint(arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(np.asarray(a, dtype=np.float64) + 0.0).tobytes())
    return h.hexdigest()[:32]


# --------------------------------------------------------------------------------------
# initial conditions (the explosion one is the reference example's, restated so the
# generator does not depend on the examples package layout)
# --------------------------------------------------------------------------------------
class ExplosionIC(InitialCondition):
    """examples/explosion/initial_condition.py:32-61 with an optional background flow."""

    def __init__(self, u0=0.0, v0=0.0, lo=3.0, hi=7.0, ylo=None, yhi=None):
        self.u0, self.v0, self.lo, self.hi = u0, v0, lo, hi
        self.ylo = lo if ylo is None else ylo
        self.yhi = hi if yhi is None else yhi

    def apply_to_block(self, block):
        left = PrimitiveState(
            fluid=block.config.fluid,
            array=np.array([4.6968, self.u0, self.v0, 404400.0]).reshape((1, 1, 4)),
        ).to_type(ConservativeState)
        right = PrimitiveState(
            fluid=block.config.fluid,
            array=np.array([1.1742, self.u0, self.v0, 101100.0]).reshape((1, 1, 4)),
        ).to_type(ConservativeState)
        xc = np.logical_and(block.mesh.x >= self.lo, block.mesh.x <= self.hi)
        yc = np.logical_and(block.mesh.y >= self.ylo, block.mesh.y <= self.yhi)
        block.state.data = np.where(np.logical_and(xc, yc), left.data, right.data)
        block.state.make_non_dimensional()


class DMRExampleIC(InitialCondition):
    """examples/dmr/initial_condition.py:32-59."""

    def apply_to_block(self, block):
        left = PrimitiveState(
            fluid=block.config.fluid,
            array=np.array([8, 8.25, 0.0, 116.5]).reshape((1, 1, 4)),
        ).to_type(ConservativeState)
        right = PrimitiveState(
            fluid=block.config.fluid,
            array=np.array([1.4, 0.0, 0.0, 1.0]).reshape((1, 1, 4)),
        ).to_type(ConservativeState)
        block.state.data = np.where(block.mesh.x <= 0.95, left.data, right.data)
        block.state.make_non_dimensional()


# ---- double-Mach-reflection boundary conditions as reference BoundaryCondition objects ----
from pyhype.boundary_conditions.base import BoundaryCondition  # noqa: E402
from pyhype.boundary_conditions.funcs import BoundaryConditionFunctions  # noqa: E402

HARNESS_CLOCK = [0.0]  # solver time at the start of the step the BC values are for


def clock_ghost_fills(solver, num_stages):
    """Ghost cells are filled at the end of every stage; the fill after a step's last
    stage serves the next step.  Set the clock so that every boundary evaluation made
    for step n (ghosts and boundary face states) sees t at the start of step n."""
    blocks = solver._blocks
    orig = blocks.apply_boundary_condition
    state = {"stage": 0, "t": 0.0, "dt": 0.0}

    def wrapped():
        state["stage"] += 1
        HARNESS_CLOCK[0] = state["t"] + state["dt"] if state["stage"] == num_stages else state["t"]
        orig()

    blocks.apply_boundary_condition = wrapped
    return state


def _prim_as(state, W):
    """A fixed primitive state converted to the type of ``state`` (same converter the
    reference's PrimitiveDirichletBC would use, at the ghost's shape)."""
    arr = np.broadcast_to(np.asarray(W, dtype=float).reshape(1, 1, 4), state.data.shape).copy()
    return PrimitiveState(fluid=state.fluid, array=arr).to_type(type(state)).data


class DirichletBC(BoundaryCondition):
    def __init__(self, W):
        self.W = W

    def _apply_boundary_condition(self, state, *args, **kwargs):
        state.data = _prim_as(state, self.W)


class SwitchBC(BoundaryCondition):
    """Per boundary cell: ``below`` where the centroid coordinate along the side is
    < x0 + speed * t, else ``above``; each is a primitive state or "Reflection"."""

    def __init__(self, x0, speed, below, above):
        self.x0, self.speed, self.below, self.above = x0, speed, below, above
        self.coord = self.angle = None

    def bind(self, block, side):
        m = block.mesh
        if side in ("N", "S"):
            row = -1 if side == "N" else 0
            self.coord = m.x[row, :, 0][None, :, None]
        else:
            col = -1 if side == "E" else 0
            self.coord = m.y[:, col, 0][:, None, None]
        d = {"E": Direction.east, "W": Direction.west, "N": Direction.north, "S": Direction.south}[side]
        self.angle = m.boundary_angle(direction=d)

    def _part(self, spec, state):
        if isinstance(spec, str):
            tmp = type(state)(fluid=state.fluid, array=state.data.copy())
            BoundaryConditionFunctions.reflection(tmp, self.angle)
            return tmp.data
        return _prim_as(state, spec)

    def _apply_boundary_condition(self, state, *args, **kwargs):
        mask = self.coord < self.x0 + self.speed * HARNESS_CLOCK[0]
        state.data = np.where(mask, self._part(self.below, state), self._part(self.above, state))


DMR_PRE = [1.4, 0.0, 0.0, 1.0]
DMR_POST = [8.0, 8.25 * np.cos(np.pi / 6), -8.25 * np.sin(np.pi / 6), 116.5]


class DMRIC(InitialCondition):
    """Mach-10 shock at 60 degrees through (1/6, 0): post-shock for x < 1/6 + y/sqrt(3)."""

    def apply_to_block(self, block):
        post = PrimitiveState(fluid=block.config.fluid, array=np.array(DMR_POST).reshape((1, 1, 4))).to_type(ConservativeState)
        pre = PrimitiveState(fluid=block.config.fluid, array=np.array(DMR_PRE).reshape((1, 1, 4))).to_type(ConservativeState)
        block.state.data = np.where(block.mesh.x < 1 / 6 + block.mesh.y / np.sqrt(3), post.data, pre.data)
        block.state.make_non_dimensional()


def dmr_mesh(nblk=5):
    """[0,4]x[0,1] as nblk blocks in a row: post-shock inflow on the west side and on
    the south side for x < 1/6, reflecting wall for x >= 1/6, the exact moving-shock
    state on the north side, outflow east."""
    from pyhype.mesh.base import QuadMeshGenerator

    south = [SwitchBC(1 / 6, 0.0, DMR_POST, "Reflection") for _ in range(nblk)]
    north = [SwitchBC(1 / 6 + 1 / np.sqrt(3), 20 / np.sqrt(3), DMR_POST, DMR_PRE) for _ in range(nblk)]
    gen = QuadMeshGenerator(nx_blk=nblk, ny_blk=1, BCE=["OutletDirichlet"], BCW=[DirichletBC(DMR_POST)],
                            BCN=north, BCS=south, SW=(0.0, 0.0), SE=(4.0, 0.0), NW=(0.0, 1.0), NE=(4.0, 1.0))
    gen._switch = {"N": north, "S": south}
    return gen


def single_block(x0, x1, y0, y1, bce="Reflection", bcw="Reflection", bcn="Reflection", bcs="Reflection"):
    return {
        0: {
            "nBLK": 0,
            "NW": [x0, y1],
            "NE": [x1, y1],
            "SW": [x0, y0],
            "SE": [x1, y0],
            "NeighborE": None,
            "NeighborW": None,
            "NeighborN": None,
            "NeighborS": None,
            "NeighborNE": None,
            "NeighborNW": None,
            "NeighborSE": None,
            "NeighborSW": None,
            "BCTypeE": bce,
            "BCTypeW": bcw,
            "BCTypeN": bcn,
            "BCTypeS": bcs,
            "BCTypeNE": None,
            "BCTypeNW": None,
            "BCTypeSE": None,
            "BCTypeSW": None,
        }
    }


def dmr_example_mesh():
    """examples/dmr/mesh.py:4-33 (skewed 4x1 block layout)."""
    from pyhype.mesh.base import QuadMeshGenerator

    k = 1
    a = 2 / np.sqrt(3)
    d = np.tan(30 * np.pi / 180)
    return QuadMeshGenerator(
        nx_blk=4,
        ny_blk=1,
        BCE=["OutletDirichlet"],
        BCW=["OutletDirichlet"],
        BCN=["OutletDirichlet"],
        BCS=["OutletDirichlet", "Slipwall", "Slipwall", "Slipwall"],
        top_x=[0, k, 2 * k, 3 * k, 4 * k],
        bot_x=[0, k, 2 * k, 3 * k, 4 * k],
        top_y=[a, a, a + d, a + 2 * d, a + 3 * d],
        bot_y=[0, 0, d, 2 * d, 3 * d],
        left_x=[0, 0],
        left_y=[0, a],
        right_x=[4 * k, 4 * k],
        right_y=[3 * d, a + 3 * d],
    )


def wedge_mesh():
    """examples/supersonic_wedge/mesh.py:6-77: a 2 x 2 square and a 15-degree wedge
    block, Mach-2 inlet on the west (the reference's PrimitiveDirichletBC state, made
    non-dimensional as that class does, applied through the harness Dirichlet BC).
    The example numbers its blocks 1 and 2, which the reference's block builder
    cannot read (blocks/base.py:531 looks blocks up from 0); they are 0 and 1 here."""
    W = PrimitiveState(fluid=AIR, array=np.array([1.0, 2.0, 0.0, 1 / AIR.gamma()]).reshape((1, 1, 4)))
    W.make_non_dimensional()
    inlet = DirichletBC(W.data.reshape(4).copy())
    tan15 = np.tan(15 * np.pi / 180)
    b1 = {"nBLK": 0, "NW": [0, 2], "NE": [2, 2], "SW": [0, 0], "SE": [2, 0],
          "NeighborE": 1, "NeighborW": None, "NeighborN": None, "NeighborS": None,
          "BCTypeE": None, "BCTypeW": inlet, "BCTypeN": "OutletDirichlet", "BCTypeS": "Reflection"}
    b2 = {"nBLK": 1, "NW": [2, 2], "NE": [4, 2 + 2 * tan15], "SW": [2, 0], "SE": [4, 2 * tan15],
          "NeighborE": None, "NeighborW": 0, "NeighborN": None, "NeighborS": None,
          "BCTypeE": "OutletDirichlet", "BCTypeW": None, "BCTypeN": "OutletDirichlet", "BCTypeS": "Reflection"}
    for b in (b1, b2):
        for c in ("NE", "NW", "SE", "SW"):
            b["Neighbor" + c] = None
            b["BCType" + c] = None
    return {0: b1, 1: b2}


def jet_mesh():
    """examples/jet/mesh.py:1-54: nine blocks stacked in y, the middle one's west side
    a subsonic Dirichlet inlet (non-dimensional, as the reference's class makes it),
    slip walls on the rest of the west side, outlets elsewhere."""
    from pyhype.mesh.base import QuadMeshGenerator

    W = PrimitiveState(fluid=AIR, array=np.array([1.0, 0.1, 0.0, 2.0 / AIR.gamma()]).reshape((1, 1, 4)))
    W.make_non_dimensional()
    inlet = DirichletBC(W.data.reshape(4).copy())
    bcw = ["Slipwall"] * 4 + [inlet] + ["Slipwall"] * 4
    return QuadMeshGenerator(nx_blk=1, ny_blk=9, BCE=["OutletDirichlet"] * 9, BCW=bcw, BCN=["OutletDirichlet"],
                             BCS=["OutletDirichlet"], NE=(1, 0.5), SW=(0, 0), NW=(0, 0.5), SE=(1, 0))


class FloodIC(InitialCondition):
    """initial_conditions/supersonic_flood.py:32-54 at the block's full shape."""

    def __init__(self, W):
        self.W = W

    def apply_to_block(self, block):
        s = PrimitiveState(fluid=block.config.fluid, array=np.array(self.W).reshape((1, 1, 4))).to_type(
            ConservativeState)
        block.state.data = np.broadcast_to(s.data, block.state.data.shape).copy()
        block.state.make_non_dimensional()


def rect_mesh(nbx, nby, east, north, bc="Reflection"):
    return RectagularMeshGenerator.generate(
        BCE=[bc], BCW=[bc], BCN=[bc], BCS=[bc],
        east=east, west=0.0, north=north, south=0.0,
        n_blocks_horizontal=nbx, n_blocks_vertical=nby,
    )


AIR = Air(a_inf=343.0, rho_inf=1.0)
AIR_UNIT = Air(a_inf=1.0, rho_inf=1.0)

BASE = dict(
    fvm_type="MUSCL",
    fvm_spatial_order=2,
    fvm_num_quadrature_points=1,
    fvm_gradient_type="GreenGauss",
    fvm_flux_function_type="Roe",
    fvm_slope_limiter_type="Venkatakrishnan",
    time_integrator="RK4",
    interface_interpolation="arithmetic_average",
    reconstruction_type=ConservativeState,
    CFL=0.8,
    t_final=1.0,
    nghost=1,
    use_JIT=True,
)

MOVING = dict(u0=120.0, v0=-80.0, lo=2.0, hi=5.0, ylo=3.0, yhi=6.5)

# name -> (config overrides, mesh factory, ic factory, steps, snapshot steps, ops step, custom tableau)
CASES = {
    "ops_explosion_cons": (dict(nx=24, ny=20), lambda: single_block(0, 10, 0, 10), lambda: ExplosionIC(), 6, "all", 3, None),
    "p100": (dict(nx=100, ny=100), lambda: single_block(0, 10, 0, 10), lambda: ExplosionIC(), 100, (1, 10, 100), None, None),
    "m2x4_40": (dict(nx=40, ny=40), lambda: rect_mesh(2, 4, 10.0, 20.0), lambda: ExplosionIC(), 12, (1, 4, 12), 2, None),
    "m2x4_150": (dict(nx=150, ny=150), lambda: rect_mesh(2, 4, 10.0, 20.0), lambda: ExplosionIC(), 10, (), None, None),
    "lim_bj": (dict(nx=20, ny=16, fvm_slope_limiter_type="BarthJespersen"), lambda: single_block(0, 10, 0, 8), lambda: ExplosionIC(**MOVING), 5, "all", 2, None),
    "lim_va": (dict(nx=20, ny=16, fvm_slope_limiter_type="VanAlbada"), lambda: single_block(0, 10, 0, 8), lambda: ExplosionIC(**MOVING), 5, "all", 2, None),
    "lim_vl": (dict(nx=20, ny=16, fvm_slope_limiter_type="VanLeer"), lambda: single_block(0, 10, 0, 8), lambda: ExplosionIC(**MOVING), 5, "all", 2, None),
    "hlll_cons": (dict(nx=20, ny=16, fvm_flux_function_type="HLLL"), lambda: single_block(0, 10, 0, 8), lambda: ExplosionIC(**MOVING), 5, "all", 2, None),
    "hlll_prim": (dict(nx=20, ny=16, fvm_flux_function_type="HLLL", reconstruction_type=PrimitiveState), lambda: single_block(0, 10, 0, 8), lambda: ExplosionIC(**MOVING), 5, "all", 2, None),
    "roe_prim": (dict(nx=20, ny=16, reconstruction_type=PrimitiveState), lambda: single_block(0, 10, 0, 8), lambda: ExplosionIC(**MOVING), 5, "all", 2, None),
    "bc_mixed": (dict(nx=20, ny=16), lambda: single_block(0, 10, 0, 8, bce="Slipwall", bcw="OutletDirichlet", bcn="Reflection", bcs=None), lambda: ExplosionIC(**MOVING), 6, "all", 2, None),
    "m2x2_prim_hlll": (dict(nx=16, ny=12, fvm_flux_function_type="HLLL", reconstruction_type=PrimitiveState, fvm_slope_limiter_type="VanAlbada"), lambda: rect_mesh(2, 2, 10.0, 8.0, bc="OutletDirichlet"), lambda: ExplosionIC(**MOVING), 5, "all", 2, None),
    "dmr_example": (dict(nx=12, ny=12, fvm_flux_function_type="HLLL", reconstruction_type=PrimitiveState, time_integrator="RK2", CFL=0.4), dmr_example_mesh, lambda: DMRExampleIC(), 5, "all", 2, None),
    "ssprk2_hlll": (dict(nx=20, ny=16, fvm_flux_function_type="HLLL", reconstruction_type=PrimitiveState, CFL=0.4), lambda: single_block(0, 10, 0, 8), lambda: ExplosionIC(**MOVING), 4, "all", None, [[1], [0.5, 0.5]]),
}
CASES["wedge"] = (dict(nx=16, ny=16, fvm_flux_function_type="HLLL", reconstruction_type=PrimitiveState,
                      time_integrator="RK2", CFL=0.3), wedge_mesh, lambda: FloodIC([1.0, 2.0, 0.0, 1 / AIR.gamma()]),
                  8, "all", 3, None)
CASES["jet"] = (dict(nx=24, ny=6, fvm_flux_function_type="HLLL", reconstruction_type=PrimitiveState,
                    time_integrator="RK2", CFL=0.4), jet_mesh, lambda: FloodIC([1.0, 0.0, 0.0, 1 / AIR.gamma()]),
                6, "all", 2, None)
CASES["qp2_roe"] = (dict(nx=20, ny=16, fvm_num_quadrature_points=2), lambda: single_block(0, 10, 0, 8),
                    lambda: ExplosionIC(**MOVING), 5, "all", None, None)
CASES["qp3_hlll_prim"] = (dict(nx=16, ny=12, fvm_num_quadrature_points=3, fvm_flux_function_type="HLLL",
                               reconstruction_type=PrimitiveState, fvm_slope_limiter_type="VanAlbada"),
                          lambda: rect_mesh(2, 2, 10.0, 8.0, bc="OutletDirichlet"), lambda: ExplosionIC(**MOVING), 5,
                          "all", None, None)
CASES["qp2_skew"] = (dict(nx=12, ny=12, fvm_num_quadrature_points=2, fvm_flux_function_type="HLLL",
                          reconstruction_type=PrimitiveState, time_integrator="RK2", CFL=0.4), dmr_example_mesh,
                     lambda: DMRExampleIC(), 4, "all", None, None)
# one-cell-wide and one-cell-high blocks (a shock tube along the block), and a 2 x 1
# layout of one-cell-wide blocks with an inter-block side
CASES["thin_x1"] = (dict(nx=1, ny=16), lambda: single_block(3, 4, 0, 8, bce="OutletDirichlet"),
                    lambda: ExplosionIC(**MOVING), 5, "all", 2, None)
CASES["thin_y1"] = (dict(nx=16, ny=1, fvm_flux_function_type="HLLL"), lambda: single_block(0, 8, 3, 4, bcs=None),
                    lambda: ExplosionIC(**MOVING), 5, "all", 2, None)
CASES["dmr5"] = (dict(nx=16, ny=20, fvm_flux_function_type="HLLL", reconstruction_type=PrimitiveState, CFL=0.4,
                     t_final=0.2, fluid=AIR_UNIT), lambda: dmr_mesh(5), lambda: DMRIC(), 8, "all", 3, [[1], [0.5, 0.5]])
for _ti in ("ExplicitEuler1", "RK2", "Ralston2", "RK3", "RK3SSP", "Ralston3", "Ralston4", "DormandPrince5"):
    CASES["ti_" + _ti] = (dict(nx=16, ny=16, time_integrator=_ti, CFL=0.4), lambda: single_block(0, 10, 0, 10), lambda: ExplosionIC(**MOVING), 3, "all", None, None)


def mesh_dict_of(mesh):
    return mesh.dict if hasattr(mesh, "dict") else mesh


def encode_mesh(mesh_cfg, out):
    """Store the mesh dictionary (corners, neighbours, string BC kinds) in arrays."""
    names = sorted(mesh_cfg.keys())
    out["blk_ids"] = np.array(names, dtype=np.int64)
    corners = np.zeros((len(names), 4, 2))
    nbr = np.full((len(names), 4), -1, dtype=np.int64)
    bc = np.empty((len(names), 4), dtype="U16")
    dirichlet = np.zeros((len(names), 4, 4))
    for k, n in enumerate(names):
        d = mesh_cfg[n]
        for c, key in enumerate(("SW", "SE", "NW", "NE")):
            corners[k, c] = d[key]
        for s, side in enumerate("EWNS"):
            v = d["Neighbor" + side]
            nbr[k, s] = -1 if v is None else v
            b = d["BCType" + side]
            if isinstance(b, SwitchBC):
                bc[k, s] = "Switch"
            elif isinstance(b, DirichletBC):
                bc[k, s] = "Dirichlet"
                dirichlet[k, s] = b.W
            else:
                bc[k, s] = "None" if b is None else str(b)
    out["corners"] = corners
    out["neighbors"] = nbr
    out["bc"] = bc
    out["dirichlet_W"] = dirichlet  # non-dimensional primitive states of Dirichlet sides


def record_geometry(solver, out):
    for bnum, blk in solver._blocks.blocks.items():
        m = blk.mesh
        p = f"geo{bnum}_"
        out[p + "nodes_x"] = m.nodes.x[:, :, 0]
        out[p + "nodes_y"] = m.nodes.y[:, :, 0]
        out[p + "xc"] = m.x[:, :, 0]
        out[p + "yc"] = m.y[:, :, 0]
        out[p + "A"] = m.A[:, :, 0]
        out[p + "dx"] = m.dx[:, :, 0]
        out[p + "dy"] = m.dy[:, :, 0]
        for side in "EWNS":
            f = m.face[getattr(Direction, {"E": "east", "W": "west", "N": "north", "S": "south"}[side])]
            out[p + f"L{side}"] = f.L[:, :, 0]
            out[p + f"th{side}"] = f.theta[:, :, 0]
            out[p + f"nx{side}"] = f.norm.x[:, :, 0]
            out[p + f"ny{side}"] = f.norm.y[:, :, 0]
            qps = blk.qp[getattr(Direction, {"E": "east", "W": "west", "N": "north", "S": "south"}[side])]
            out[p + f"qx{side}"] = qps[0].x[:, :, 0]
            out[p + f"qy{side}"] = qps[0].y[:, :, 0]
            if len(qps) > 1:  # every point of a multi-point rule, in the reference's order
                for k, q in enumerate(qps):
                    out[p + f"qx{side}_{k}"] = q.x[:, :, 0]
                    out[p + f"qy{side}_{k}"] = q.y[:, :, 0]
            # the run-time rotation evaluates np.sin/np.cos on numpy float64 scalars
            # (pyhype/utils/utils.py:75-85); record that scalar path for the theta arrays
            th = f.theta[:, :, 0]
            out[p + f"cos_scalar{side}"] = np.array([np.cos(v) for v in th.ravel()]).reshape(th.shape)
            out[p + f"sin_scalar{side}"] = np.array([np.sin(v) for v in th.ravel()]).reshape(th.shape)
        out[p + "is_cartesian"] = np.array(bool(blk.is_cartesian))


def capture_ops(solver, out, tag):
    """One residual evaluation per block, with every intermediate recorded."""
    for bnum, blk in solver._blocks.blocks.items():
        p = f"{tag}{bnum}_"
        recon = blk.recon_block
        fvm = recon.fvm
        recon.from_block(blk)
        out[p + "recon"] = recon.state.data.copy()
        for side in "EWNS":
            g = recon.ghost[getattr(Direction, {"E": "east", "W": "west", "N": "north", "S": "south"}[side])]
            out[p + f"ghost{side}"] = g.state.data.copy()
        fvm.gradient.compute(recon)
        out[p + "gx"] = recon.grad.x.copy()
        out[p + "gy"] = recon.grad.y.copy()
        fvm.compute_limiter()
        out[p + "phi"] = fvm.limiter.phi.copy()

        captured = {}

        def wrap(fn, key):
            def inner(WL, WR):
                captured[key + "L"] = WL.data.copy()
                captured[key + "R"] = WR.data.copy()
                res = fn(WL=WL, WR=WR)
                captured[key + "F"] = np.array(res, copy=True)
                return res

            return inner

        fx, fy = fvm.flux_function_x, fvm.flux_function_y
        fvm.flux_function_x = wrap(fx, "x")
        fvm.flux_function_y = wrap(fy, "y")
        try:
            fvm._evaluate_east_west_flux()
            fvm._evaluate_north_south_flux()
        finally:
            fvm.flux_function_x, fvm.flux_function_y = fx, fy
        ny, nx = blk.state.data.shape[:2]
        out[p + "xL"] = captured["xL"].reshape(ny, nx + 1, 4)
        out[p + "xR"] = captured["xR"].reshape(ny, nx + 1, 4)
        out[p + "xF"] = captured["xF"].reshape(ny, nx + 1, 4)
        out[p + "yL"] = captured["yL"].reshape(nx, ny + 1, 4)
        out[p + "yR"] = captured["yR"].reshape(nx, ny + 1, 4)
        out[p + "yF"] = captured["yF"].reshape(nx, ny + 1, 4)
        for side, key in (("E", Direction.east), ("W", Direction.west), ("N", Direction.north), ("S", Direction.south)):
            out[p + f"flux{side}"] = fvm.Flux[key][0].copy()
        out[p + "dUdt"] = blk.dUdt().copy()


def run_case(name):
    overrides, mesh_f, ic_f, steps, snaps, ops_step, tableau = CASES[name]
    cfg_kwargs = dict(BASE)
    cfg_kwargs.update(overrides)
    fluid = cfg_kwargs.pop("fluid", AIR)
    cfg = SolverConfig(initial_condition=ic_f(), fluid=fluid, **cfg_kwargs)
    mesh = mesh_f()
    solver = Euler2D(config=cfg, mesh_config=mesh)
    # bind position-dependent BCs to the blocks that own them
    for bnum, blk in solver._blocks.blocks.items():
        d = mesh_dict_of(mesh)[bnum]
        for side in "EWNS":
            bc = d["BCType" + side]
            if isinstance(bc, SwitchBC):
                bc.bind(blk, side)
    if tableau is not None:
        solver._time_integrator = ExplicitRungeKutta(cfg, a=tableau)
    out = {}
    encode_mesh(mesh_dict_of(mesh), out)
    out["nx"] = np.array(cfg.nx)
    out["ny"] = np.array(cfg.ny)
    out["cfl"] = np.array(cfg.CFL)
    out["nqp"] = np.array(cfg.fvm_num_quadrature_points)
    out["t_final"] = np.array(cfg.t_final)
    out["a_inf"] = np.array(cfg.fluid.far_field.a)
    out["flux"] = np.array(cfg.fvm_flux_function_type)
    out["limiter"] = np.array(cfg.fvm_slope_limiter_type)
    out["recon"] = np.array(cfg.reconstruction_type.__name__)
    out["integrator"] = np.array(cfg.time_integrator if tableau is None else "custom")
    a = solver._time_integrator.a
    tab = np.zeros((len(a), len(a)))
    for i, row in enumerate(a):
        tab[i, : len(row)] = row
    out["tableau"] = tab
    record_geometry(solver, out)
    HARNESS_CLOCK[0] = 0.0
    clock = clock_ghost_fills(solver, solver._time_integrator.num_stages)
    solver._pre_process_solve()
    bnums = sorted(solver._blocks.blocks.keys())
    out["ic"] = np.stack([solver._blocks[b].state.data.copy() for b in bnums])
    dts, fps, ts = [], [], []
    t0 = time.time()
    for step in range(1, steps + 1):
        if ops_step is not None and step == ops_step:
            HARNESS_CLOCK[0] = solver.t
            out["ops_t"] = np.array(solver.t)
            capture_ops(solver, out, "ops")
            out["ops_state"] = np.stack([solver._blocks[b].state.data.copy() for b in bnums])
        dt = solver.get_dt()
        HARNESS_CLOCK[0] = solver.t
        clock.update(stage=0, t=solver.t, dt=dt)
        solver._update_solution_blocks(dt)
        solver._realizability_check()
        solver.t += dt
        solver.num_time_step += 1
        dts.append(dt)
        ts.append(solver.t)
        st = [solver._blocks[b].state.data for b in bnums]
        fps.append(fingerprint(st))
        if snaps == "all" or step in snaps:
            out[f"state_{step}"] = np.stack([s.copy() for s in st])
        if step == steps:
            out["sums_final"] = np.array([[s[:, :, k].sum() for k in range(4)] for s in st])
    out["dts"] = np.array(dts)
    out["ts"] = np.array(ts)
    out["fingerprints"] = np.array(fps)
    out["steps"] = np.array(steps)
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **out)
    print(f"{name}: {steps} steps in {time.time() - t0:.1f}s -> {os.path.getsize(path) / 1e3:.0f} kB", flush=True)


if __name__ == "__main__":
    names = sys.argv[1:] or list(CASES)
    if len(names) > 1 and os.environ.get("GOLDEN_SERIAL") is None:
        import multiprocessing as mp

        with mp.get_context("spawn").Pool(min(len(names), os.cpu_count() or 1)) as pool:
            pool.map(run_case, names)
    else:
        for n in names:
            run_case(n)
