"""Batched ensembles: many independent problems of uneven sizes in one device problem.

Every instance is one block with its own size, initial condition and time step
(per-instance CFL dt, t and step count live in the device instance table), so a
single launch per stage kernel advances all of them, and whole steps replay from a
captured CUDA graph.  Blocks carry their instance id in the block table; nothing
couples two instances.

``explosion_ensemble`` draws the benchmark ensemble (seeded): sizes nx, ny uniform in
{64, 96, ..., 512}, domain nx/10 x ny/10, a square of high pressure (ratio
log-uniform in [2, 20]) and density (ratio 4) over the base state (1.1742, 101100),
half-width uniform in [0.1, 0.3] of the smaller domain side, centred uniformly
inside, Reflection on every side.

The reference scheme itself is not robust on every such instance: with the seed-0
ensemble, instance 265 (448 x 448, pressure ratio 4.2) reaches NaN at a corner of the
square in its 8th step in FP64, in the CPU oracle as on the GPU.  Such an instance is
halted and reported; the others continue.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import List, Optional

import numpy as np

from ._native import DeviceSolver, RealizabilityError
from .fluids import Air
from .problem import Problem, build_problem
from .states import ConservativeState, PrimitiveState
from .time_marching import tableau as named_tableau

BASE_RHO = 1.1742
BASE_P = 101100.0


@dataclass
class ExplosionInstance:
    nx: int
    ny: int
    lx: float
    ly: float
    cx: float
    cy: float
    half_width: float
    p_ratio: float
    rho_ratio: float = 4.0


def explosion_ensemble(count: int = 512, seed: int = 0, sizes=tuple(range(64, 513, 32))) -> List[ExplosionInstance]:
    rng = np.random.default_rng(seed)
    sizes = np.asarray(sizes)
    nx = rng.choice(sizes, count)
    ny = rng.choice(sizes, count)
    out = []
    for k in range(count):
        lx, ly = nx[k] / 10.0, ny[k] / 10.0
        hw = rng.uniform(0.1, 0.3) * min(lx, ly)
        cx = rng.uniform(hw, lx - hw)
        cy = rng.uniform(hw, ly - hw)
        r = float(np.exp(rng.uniform(np.log(2.0), np.log(20.0))))
        out.append(ExplosionInstance(int(nx[k]), int(ny[k]), lx, ly, cx, cy, hw, r))
    return out


def _block(k: int, inst: ExplosionInstance, bc="Reflection") -> dict:
    return {
        "nBLK": k, "SW": [0.0, 0.0], "SE": [inst.lx, 0.0], "NW": [0.0, inst.ly], "NE": [inst.lx, inst.ly],
        "NeighborE": None, "NeighborW": None, "NeighborN": None, "NeighborS": None,
        "NeighborNE": None, "NeighborNW": None, "NeighborSE": None, "NeighborSW": None,
        "BCTypeE": bc, "BCTypeW": bc, "BCTypeN": bc, "BCTypeS": bc,
        "BCTypeNE": None, "BCTypeNW": None, "BCTypeSE": None, "BCTypeSW": None,
    }


def ensemble_problem(instances: List[ExplosionInstance], precision: int = 0, flux: str = "Roe",
                     limiter: str = "Venkatakrishnan", recon: str = "ConservativeState",
                     cfl: float = 0.5) -> Problem:
    """One device problem holding every instance as an independent block."""
    air = Air(a_inf=343.0, rho_inf=1.0)
    mesh = {k: _block(k, inst) for k, inst in enumerate(instances)}
    sizes = {k: (inst.nx, inst.ny) for k, inst in enumerate(instances)}
    inst_of = {k: k for k in range(len(instances))}
    return build_problem(mesh, 0, 0, flux=flux, limiter=limiter, recon=recon, gamma=air.gamma(),
                         gm1=air.gamma() - 1, cfl=cfl, fluid=air, precision=precision,
                         instance_of=inst_of, sizes=sizes)


def instance_state(inst: ExplosionInstance, geometry, fluid) -> np.ndarray:
    """(ny, nx, 4) non-dimensional conservative initial state of one instance."""
    inside = PrimitiveState(fluid, array=np.array([BASE_RHO * inst.rho_ratio, 0.0, 0.0, BASE_P * inst.p_ratio],
                                                  dtype=float).reshape(1, 1, 4)).to_type(ConservativeState)
    outside = PrimitiveState(fluid, array=np.array([BASE_RHO, 0.0, 0.0, BASE_P]).reshape(1, 1, 4)).to_type(
        ConservativeState)
    xin = np.abs(geometry.xc - inst.cx) <= inst.half_width
    yin = np.abs(geometry.yc - inst.cy) <= inst.half_width
    s = ConservativeState(fluid, array=np.where((xin & yin)[:, :, None], inside.data, outside.data))
    s.make_non_dimensional()
    return s.data


def ensemble_state(problem: Problem, instances: List[ExplosionInstance]) -> np.ndarray:
    air = Air(a_inf=343.0, rho_inf=1.0)
    return problem.to_soa([instance_state(inst, g, air) for inst, g in zip(instances, problem.block_geometry)])


class EnsembleSolver:
    """All instances of an ensemble advanced together on one GPU."""

    def __init__(self, instances: List[ExplosionInstance], precision: int = 0, integrator: str = "SSPRK2",
                 cfl: float = 0.5, problem: Optional[Problem] = None):
        self.instances = instances
        self.problem = problem if problem is not None else ensemble_problem(instances, precision, cfl=cfl)
        if self.problem.cfg.precision != precision:
            self.problem = self.problem.with_precision(precision)
        self.device = DeviceSolver(self.problem, tableau=named_tableau(integrator))
        self.device.set_state(ensemble_state(self.problem, instances))

    def run(self, steps: int) -> List[int]:
        """``steps`` steps of every instance, each with its own CFL dt.  An instance whose
        state becomes unrealizable (rho <= 0 or E <= 0 after a step) is halted there while
        the others continue; returns the indices of the instances halted in this call."""
        try:
            self.device.run(0.0, float("inf"), max_steps=steps)
        except RealizabilityError:
            pass
        _, done = self.device.instance_times()
        return [k for k, n in enumerate(done) if n < steps]

    def states(self) -> List[np.ndarray]:
        return self.problem.from_soa(self.device.get_state())
