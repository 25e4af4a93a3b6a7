"""Time the pyHype reference itself on this machine's CPU (one process, one core),
under the same import shim as make_golden.py: identity ``njit`` (the numba loop bodies
run as pure Python), a one-rank MPI world, stub plotting.  This is the reference's
"pure-Python fallback" rate; numba and mpi4py are not installed here or on the GPU
box, and the reference's sources are not present on the GPU machine at all.

Cases: the plain explosion (one 100 x 100 block) and the multiblock correctness size
(2 x 4 blocks of 150 x 150), Roe / Venkatakrishnan / Green-Gauss / RK4, CFL 0.8.  One
untimed step, then ``steps`` timed steps of the reference's own loop
(``Solver.get_dt`` -> ``ExplicitRungeKutta.integrate`` -> realizability check).

Usage::

    python tests/golden/time_reference.py [steps]
"""
from __future__ import annotations

import json
import os
import platform
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import make_golden as M  # noqa: E402  (installs the shim and imports the reference)


def time_case(name: str, steps: int) -> dict:
    overrides, mesh_f, ic_f, _, _, _, _ = M.CASES[name]
    kw = dict(M.BASE)
    kw.update(overrides)
    fluid = kw.pop("fluid", M.AIR)
    cfg = M.SolverConfig(initial_condition=ic_f(), fluid=fluid, **kw)
    solver = M.Euler2D(config=cfg, mesh_config=mesh_f())
    solver._pre_process_solve()
    ncell = sum(b.state.data.shape[0] * b.state.data.shape[1] for b in solver._blocks.blocks.values())
    stages = solver._time_integrator.num_stages

    def step():
        dt = solver.get_dt()
        solver._update_solution_blocks(dt)
        solver._realizability_check()
        solver.t += dt

    step()  # untimed
    t0 = time.perf_counter()
    for _ in range(steps):
        step()
    el = time.perf_counter() - t0
    return {"case": name, "cells": ncell, "stages": stages, "steps": steps, "s_per_step": el / steps,
            "cell_stage_updates_per_s": ncell * stages * steps / el, "cores": 1,
            "host": platform.processor() or platform.machine()}


if __name__ == "__main__":
    steps = int(sys.argv[1]) if len(sys.argv) > 1 else 3
    for name in ("p100", "m2x4_150"):
        print(json.dumps(time_case(name, steps)), flush=True)
