"""Solver configuration: the same keyword set and string choices as
``pyhype/solver_config.py:32-135`` so a reference user's config builds unchanged."""
from __future__ import annotations

from typing import List, Union

from .states import ConservativeState


class SolverConfig:
    __slots__ = [
        "fvm_type",
        "fvm_spatial_order",
        "fvm_num_quadrature_points",
        "fvm_gradient_type",
        "fvm_flux_function_type",
        "fvm_slope_limiter_type",
        "time_integrator",
        "initial_condition",
        "interface_interpolation",
        "reconstruction_type",
        "write_solution",
        "write_solution_mode",
        "write_solution_name",
        "write_solution_base",
        "write_every_n_timesteps",
        "plot_every",
        "plot_function",
        "CFL",
        "t_final",
        "realplot",
        "profile",
        "fluid",
        "nx",
        "ny",
        "n",
        "nghost",
        "use_JIT",
        "show_log_for_procs",
    ]

    def __init__(
        self,
        nx: int,
        ny: int,
        CFL: float,
        t_final: float,
        initial_condition,
        fvm_type: str,
        time_integrator: str,
        fvm_gradient_type: str,
        fvm_flux_function_type: str,
        fvm_slope_limiter_type: str,
        fvm_spatial_order: int,
        fvm_num_quadrature_points: int,
        fluid,
        nghost: int = 1,
        use_JIT: bool = True,
        profile: bool = False,
        realplot: bool = False,
        plot_every: int = 20,
        plot_function: str = "Density",
        write_solution: bool = False,
        write_solution_mode: str = "every_n_timesteps",
        write_solution_name: str = "nozzle",
        write_solution_base: str = None,
        reconstruction_type=ConservativeState,
        write_every_n_timesteps: int = 40,
        interface_interpolation: str = "arithmetic_average",
        show_log_for_procs: Union[List[int], str] = None,
    ) -> None:
        self.initial_condition = initial_condition
        self.nx = nx
        self.ny = ny
        self.n = nx * ny
        self.nghost = nghost
        self.CFL = CFL
        self.t_final = t_final
        self.fvm_type = fvm_type
        self.time_integrator = time_integrator
        self.fvm_gradient_type = fvm_gradient_type
        self.fvm_flux_function_type = fvm_flux_function_type
        self.fvm_slope_limiter_type = fvm_slope_limiter_type
        self.fvm_spatial_order = fvm_spatial_order
        self.fvm_num_quadrature_points = fvm_num_quadrature_points
        self.reconstruction_type = reconstruction_type
        self.interface_interpolation = interface_interpolation
        self.fluid = fluid
        self.use_JIT = use_JIT
        self.profile = profile
        self.realplot = realplot
        self.plot_every = plot_every
        self.plot_function = plot_function
        self.write_solution = write_solution
        self.write_solution_mode = write_solution_mode
        self.write_solution_name = write_solution_name
        self.write_solution_base = write_solution_base
        self.write_every_n_timesteps = write_every_n_timesteps
        if show_log_for_procs is None:
            self.show_log_for_procs = [0]
        else:
            self.show_log_for_procs = show_log_for_procs

    def __str__(self):
        return "".join(f"\t{atr}: {getattr(self, atr)}\n" for atr in self.__slots__)
