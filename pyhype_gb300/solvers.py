"""``Euler2D``: the reference's solver API, running its time loop on the GPU.

Same constructor and ``solve()`` as ``pyhype/solvers/Euler2D.py:46-216``:

* construction resolves the mesh dictionary / generator, builds every block's
  geometry on the host and creates the device solver (``e2d_create``);
* ``solve()`` applies the initial condition to host-side block proxies
  (``block.mesh.x/y``, ``block.state``, ``block.config``), uploads the state once and
  runs the loop ``dt -> clamp to t_final -> RK step -> realizability -> t += dt``
  entirely on the device (``e2d_run``), returning to the host only to log progress,
  write snapshots or finish;
* snapshots use the reference's layout ``{base}/{name}/{k}/{name}_blk_{n}.npy`` and
  ``{base}/{name}/mesh/mesh_{x,y}_blk_{n}.npy`` (``pyhype/solvers/base.py:139-172``),
  including its numbering (directory ``k`` holds the state after ``k + 1`` steps);
* an unrealizable state (rho <= 0 or E <= 0) raises ``RealizabilityException`` where
  the reference logs and calls ``MPI.Abort`` (``Euler2D.py:144-152``).

All blocks share one GPU; there is no MPI layer (``distribute_blocks_to_processes``
has nothing to distribute on one device).
"""
from __future__ import annotations

import logging
import pathlib
import time
from typing import Dict, Iterable, Union

import numpy as np

from ._native import DeviceSolver, RealizabilityError
from .mesh.base import MeshGenerator
from .mesh.quad_mesh import QuadMesh
from .problem import problem_from_config
from .states import ConservativeState, RealizabilityException
from .time_marching import TimeIntegratorFactory

_log = logging.getLogger("pyhype_gb300")


class HostBlock:
    """What an initial condition sees of a block: ``mesh``, ``state``, ``config``."""

    def __init__(self, config, global_block_num: int, geometry, vertices, neighbors: dict, bc: dict):
        self.config = config
        self.global_block_num = global_block_num
        self.mesh = QuadMesh(geometry, vertices)
        self.state = ConservativeState(fluid=config.fluid, shape=(geometry.ny, geometry.nx, 4))
        self.neighbors = neighbors
        self.bc = bc

    @property
    def is_cartesian(self) -> bool:
        return self.mesh.geometry.is_cartesian

    def realizable(self):
        return [self.state.realizable()]


class Euler2D:
    def __init__(self, config, mesh_config: Union[MeshGenerator, dict], precision: str = "fp64") -> None:
        """``precision="fp32"`` selects the FP32 form (FP32 state and flux arithmetic,
        Kahan-compensated step accumulation, FP64 dt reduction); the default is the
        FP64 path, equal to the reference value for value."""
        if precision not in ("fp64", "fp32"):
            raise ValueError(f"precision must be 'fp64' or 'fp32', not {precision!r}")
        self.precision = precision
        self.config = config
        self.fluid = config.fluid
        info = mesh_config.dict if isinstance(mesh_config, MeshGenerator) else mesh_config
        self.mesh_config: Dict[int, dict] = info
        self.problem = problem_from_config(config, info, precision=0 if precision == "fp64" else 1)
        self._blocks: Dict[int, HostBlock] = {}
        for k, blk in enumerate(self.problem.block_ids):
            d = info[blk]
            self._blocks[blk] = HostBlock(
                config, blk, self.problem.block_geometry[k], {c: d[c] for c in ("NE", "NW", "SE", "SW")},
                {s: d.get("Neighbor" + s) for s in "EWNS"}, {s: d.get("BCType" + s) for s in "EWNS"},
            )
        self._time_integrator = TimeIntegratorFactory.create(config=config)
        self.t = 0
        self.num_time_step = 0
        self.CFL = config.CFL
        self.t_final = config.t_final * self.fluid.far_field.a
        self.profile_data = None
        self.write_path = None
        if config.write_solution:
            self.write_path = pathlib.Path(config.write_solution_base) / config.write_solution_name
            self.write_path.mkdir(exist_ok=True, parents=True)
        self.device = DeviceSolver(self.problem, tableau=self._time_integrator.tableau())

    # ---- reference-shaped accessors --------------------------------------------------
    @property
    def blocks(self) -> Iterable[HostBlock]:
        return self._blocks.values()

    def __str__(self):
        c = self.config
        return (
            "\tA Solver of type Euler2D for solving the 2D Euler\n"
            "\tequations on structured grids using the Finite Volume Method.\n\n"
            f"\t{'Finite Volume Method: ':<40} {c.fvm_type}\n"
            f"\t{'Gradient Method: ':<40} {c.fvm_gradient_type}\n"
            f"\t{'Flux Function: ':<40} {c.fvm_flux_function_type}\n"
            f"\t{'Limiter: ':<40} {c.fvm_slope_limiter_type}\n"
            f"\t{'Time Integrator: ':<40} {c.time_integrator}"
        )

    def apply_initial_condition(self):
        for block in self.blocks:
            self.config.initial_condition.apply_to_block(block)

    def upload(self):
        self.device.set_state(self.problem.to_soa([b.state.data for b in self.blocks]))

    def download(self):
        for b, arr in zip(self.blocks, self.problem.from_soa(self.device.get_state())):
            b.state.data = arr

    def get_dt(self) -> float:
        """Global CFL time step clamped to t_final (``pyhype/solvers/base.py:114-136``)."""
        dt = float(self.device.compute_dt()[0])
        return self.t_final - self.t if self.t_final - self.t < dt else dt

    # ---- solve ------------------------------------------------------------------------
    def solve(self):
        self._pre_process_solve()
        self._solve()
        self._post_process_solve()

    def _pre_process_solve(self):
        self.apply_initial_condition()
        for b in self.blocks:
            r = b.state.realizable()
            if isinstance(r, RealizabilityException):
                raise r
        self.upload()
        if self.config.write_solution:
            self.write_mesh()

    def _next_stop(self) -> int:
        """Steps until the host must look at the solution (log / snapshot)."""
        n = 50 - self.num_time_step % 50
        if self.config.write_solution and self.config.write_solution_mode == "every_n_timesteps":
            m = self.config.write_every_n_timesteps
            # a snapshot is written after the step whose pre-increment count is k*m
            k = self.num_time_step % m
            n = min(n, (m - k) % m + 1)
        return max(1, n)

    def _solve(self):
        t0 = time.perf_counter()
        start_steps = self.num_time_step
        while self.t < self.t_final:
            if self.num_time_step % 50 == 0:
                _log.info(f"Simulation time: {self.t / self.fluid.far_field.a}, Timestep number: {self.num_time_step}")
            chunk = self._next_stop()
            try:
                t, steps = self.device.run(self.t, self.t_final, max_steps=chunk)
            except RealizabilityError as e:
                self.download()
                raise RealizabilityException(
                    f"ConservativeState has unrealizable values: block {e.info.block}, cell {e.info.cell}, "
                    f"{e.info.nbad} cells") from e
            if steps == 0:
                break
            self.t = t
            self.num_time_step += steps
            if self.config.write_solution:
                self.write_solution(self.num_time_step - 1)
        if self.config.profile:
            el = time.perf_counter() - t0
            ncell = self.problem.ncell
            stages = self._time_integrator.num_stages
            steps = self.num_time_step - start_steps
            _log.info(f"{steps} steps in {el:.3f} s, {ncell * stages * steps / max(el, 1e-12):.4e} cell-stage updates/s")

    def _post_process_solve(self):
        self.download()
        _log.info(f"Simulation time: {self.t / self.fluid.far_field.a}, Timestep number: {self.num_time_step}")

    # ---- output -----------------------------------------------------------------------
    def write_mesh(self):
        path = self.write_path / "mesh"
        path.mkdir(parents=True, exist_ok=True)
        for b in self.blocks:
            np.save(str(path / "mesh_x_blk_") + str(b.global_block_num), b.mesh.x)
            np.save(str(path / "mesh_y_blk_") + str(b.global_block_num), b.mesh.y)

    def write_solution(self, count: int):
        if self.config.write_solution_mode != "every_n_timesteps" or count % self.config.write_every_n_timesteps:
            return
        self.download()
        path = self.write_path / str(count)
        path.mkdir(parents=True, exist_ok=True)
        for b in self.blocks:
            np.save(str(path / self.config.write_solution_name) + "_blk_" + str(b.global_block_num), b.state.data)
