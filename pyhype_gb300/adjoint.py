"""Reverse-mode differentiation of the time loop behind ``torch.autograd.Function``.

The objective is the time integral of the pressure force on one block side,

    J = sum_n dt_n * P(U^{n+1}),   P(U) = sum over the side's cells of p * L_face,

with the dt schedule frozen from the recorded forward pass (so that finite
differences of J at that schedule are what the gradient describes).  The forward pass
runs the plain FP64 kernels and keeps the state every ``ckpt_every`` steps; the
backward pass recomputes each segment from its checkpoint (keeping stage states and
face states) and runs the hand-written reverse kernels (e2d_adjoint.cu) step by step
back to U^0.  Gradients with respect to initial-condition parameters follow from
torch autograd through the initial condition itself (``smoothed_explosion``).

Subgradients at the scheme's non-differentiable points: min/max take the operand
the forward selects, Harten's entropy fix differentiates the branch taken, |x| has
derivative 0 at x = 0, the limiter's davg == 0 branch (slope 1) is constant, and a
negative limiter value clipped to 0 passes nothing back.

The reference (momokhalil/pyHype) has no differentiation; this module is new.
"""
from __future__ import annotations

from typing import Optional

import numpy as np
import torch

from ._native import DeviceSolver
from .fluids import Air
from .problem import Problem, build_problem
from .time_marching import tableau as named_tableau

SIDE = {"E": 0, "W": 1, "N": 2, "S": 3}


def single_block_mesh(length: float = 10.0, bc: str = "Reflection") -> dict:
    """One square block [0, length]^2 with the same BC on every side."""
    return {0: {
        "nBLK": 0, "NW": [0.0, length], "NE": [length, length], "SW": [0.0, 0.0], "SE": [length, 0.0],
        "NeighborE": None, "NeighborW": None, "NeighborN": None, "NeighborS": None,
        "NeighborNE": None, "NeighborNW": None, "NeighborSE": None, "NeighborSW": None,
        "BCTypeE": bc, "BCTypeW": bc, "BCTypeN": bc, "BCTypeS": bc,
        "BCTypeNE": None, "BCTypeNW": None, "BCTypeSE": None, "BCTypeSW": None,
    }}


def adjoint_problem(n: int = 256, length: float = 10.0, limiter: str = "Venkatakrishnan",
                    recon: str = "ConservativeState", cfl: float = 0.5, bc: str = "Reflection",
                    flux: str = "Roe") -> Problem:
    air = Air(a_inf=343.0, rho_inf=1.0)
    return build_problem(single_block_mesh(length, bc), n, n, flux=flux, limiter=limiter, recon=recon,
                         gamma=air.gamma(), gm1=air.gamma() - 1, cfl=cfl, fluid=air)


def smoothed_explosion(problem: Problem, r, w, cx, cy=5.0, device="cuda") -> torch.Tensor:
    """Differentiable explosion IC on block 0: a square of half-width w centred at
    (cx, cy) with pressure ratio r and density ratio 4 over (1.1742, 0, 0, 101100),
    edges smoothed by tanh over one cell width on each side (a two-cell edge).
    Returns the non-dimensional conservative state as (4, ncell) FP64 planes."""
    air = Air(a_inf=343.0, rho_inf=1.0)
    g = problem.block_geometry[0]
    xc = torch.as_tensor(g.xc, dtype=torch.float64, device=device)
    yc = torch.as_tensor(g.yc, dtype=torch.float64, device=device)
    delta = float(np.mean(np.diff(g.nodes_x[0, :])))
    r = torch.as_tensor(r, dtype=torch.float64, device=device)
    w = torch.as_tensor(w, dtype=torch.float64, device=device)
    cx = torch.as_tensor(cx, dtype=torch.float64, device=device)
    chi = 0.25 * (1 + torch.tanh((w - torch.abs(xc - cx)) / delta)) * (1 + torch.tanh((w - torch.abs(yc - cy)) / delta))
    rho = 1.1742 * (1 + 3 * chi)
    p = 101100.0 * (1 + (r - 1) * chi)
    a_inf, rho_inf = air.far_field.a, air.far_field.rho
    E = p / (air.gamma() - 1) / (rho_inf * a_inf * a_inf)
    zero = torch.zeros_like(rho)
    U = torch.stack([rho / rho_inf, zero, zero, E]).reshape(4, -1)
    return U.contiguous()


class AdjointSolver:
    """A single-instance problem set up for the recorded forward / reverse pass, on the
    FP64 path or (``precision="fp32"``) the FP32 form, whose reverse kernels run in FP32
    (J, dt and the returned gradient are FP64 values)."""

    def __init__(self, problem: Problem, integrator: str = "RK4", block: int = 0, side: str = "N",
                 nsteps: int = 400, ckpt_every: int = 20, precision: str = "fp64"):
        if precision not in ("fp64", "fp32"):
            raise ValueError(f"precision must be 'fp64' or 'fp32', not {precision!r}")
        self.problem = problem if precision == "fp64" else problem.with_precision(1)
        self.device = DeviceSolver(self.problem, tableau=named_tableau(integrator))
        self.block, self.side = int(block), SIDE[side] if isinstance(side, str) else int(side)
        self.nsteps, self.ckpt_every = int(nsteps), int(ckpt_every)
        self._record = 0
        self.dts: Optional[np.ndarray] = None

    def forward(self, U0: torch.Tensor, dts: Optional[np.ndarray] = None) -> float:
        U0 = U0.detach().to(dtype=torch.float64, device="cuda").contiguous()
        torch.cuda.synchronize()
        self.device.set_state_device(U0.data_ptr())
        J, self.dts = self.device.adjoint_forward(self.nsteps, self.ckpt_every, self.block, self.side, 0.0, dts)
        self._record += 1
        return J

    def backward(self) -> torch.Tensor:
        return self.device.adjoint_backward()

    def objective(self, U0: torch.Tensor, dts: Optional[np.ndarray] = None) -> torch.Tensor:
        """J as a differentiable function of U0 (autograd calls the reverse pass)."""
        return PressureObjective.apply(U0, self, dts)


class PressureObjective(torch.autograd.Function):
    @staticmethod
    def forward(ctx, U0, solver: AdjointSolver, dts):
        J = solver.forward(U0, dts)
        ctx.solver = solver
        ctx.record = solver._record
        return torch.tensor(J, dtype=torch.float64, device=U0.device)

    @staticmethod
    def backward(ctx, gJ):
        s = ctx.solver
        if s._record != ctx.record:
            raise RuntimeError("another forward pass was recorded on this solver since; the reverse pass "
                               "needs its own recording")
        g = s.backward().reshape(4, -1)
        return gJ * g, None, None
