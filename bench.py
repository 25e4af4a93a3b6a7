#!/usr/bin/env python
"""Benchmark: cell-stage updates/s of the GB300 FP64 MUSCL/RK4 path.

Workload (the multiblock explosion throughput configuration): domain [0,10]x[0,20] as
2x4 blocks of 1024x1024 cells (8,388,608 cells), ideal gas gamma 1.4, explosion
initial condition, MUSCL order 2 with Green-Gauss gradients, Venkatakrishnan limiter,
Roe flux, conservative reconstruction, reflecting walls, RK4 at CFL 0.8, FP64.
A step is one RK4 step (4 residual evaluations) of every block, CFL dt included.

  value   device-resident throughput: K steps of the device time loop (e2d_run),
          timed with CUDA events on the solver's stream.  Each stage streams
          ~2.5 GB (state, geometry, face arrays), so the working set exceeds the
          129 MB L2 between iterations without a flush.
  e2e     the same metric through the C ABI with host buffers: each step copies the
          state from pinned host memory (e2d_set_state), steps once (e2d_run) and
          copies the state back (e2d_get_state).
  roofline  the dominant kernel's algorithmic FP64 flops per launch divided by its
          CUDA-event duration, against this GPU's measured DFMA rate.
  cpu_baseline  the CPU oracle (a C restatement of the reference algorithm) on
          every host core, timed on one full step of the same workload.

``--impl reference`` times the reference algorithm's CPU implementation (the same C
restatement, all host threads) on the same workload and prints its own line.
Multi-GPU: replicas only (each rank advances its own copy of the workload; there is
no inter-GPU exchange in this single-GPU path); value sums the ranks' cells.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = ("multiblock explosion 2x4 blocks x 1024x1024 cells, Roe/Venkatakrishnan/Green-Gauss/RK4, CFL 0.8, "
            "explosion IC with seeded cell noise (seed 0)")
SEED = 0
METRIC = "cell-stage updates/s (FP64 plain, multiblock explosion 2x4x1024^2, RK4)"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n", "--cells-per-side", dest="n", type=int, default=1024, help="cells per block side")
    ap.add_argument("--cpu-steps", type=int, default=2, help="timed RK4 steps in the CPU-baseline sample")
    ap.add_argument("--skip-cpu-baseline", action="store_true", help="omit the CPU baseline (profiling runs)")
    ap.add_argument("--skip-ensemble", action="store_true", help="omit the batched-ensemble section")
    ap.add_argument("--skip-adjoint", action="store_true", help="omit the adjoint section")
    ap.add_argument("--skip-dmr", action="store_true", help="omit the double-Mach-reflection section")
    ap.add_argument("--stage-form", default="default", choices=["default", "split", "fused28", "fused13"],
                    help="stage form of the --precision fp32 profiling run")
    ap.add_argument("--precision", default="fp64", choices=["fp64", "fp32"],
                    help="arithmetic of the timed multiblock run (fp32: the FP32 form; for profiling)")
    ap.add_argument("--workload", default="multiblock",
                    choices=["multiblock", "ensemble", "adjoint", "adjoint-study", "dmr"],
                    help="'ensemble' runs the full 512-instance, 200-step batched comparison instead; "
                         "'dmr' the double-Mach case with the FP64 scheme's one-ulp sensitivity; "
                         "'adjoint' one recorded forward + reverse pass on an n x n block for --steps steps; "
                         "'adjoint-study' the finite-difference convergence study of the reverse pass")
    return ap.parse_args()


def seeded_state(block, seed: int):
    """Explosion state with seeded per-cell noise on every primitive variable (density
    and pressure +-2 %, velocities +-0.01 of the far-field sound speed), so no region
    of the synthetic input is uniform."""
    import numpy as np

    from pyhype_gb300.states import ConservativeState, PrimitiveState

    fl = block.config.fluid
    W = ConservativeState(fl, array=block.state.data.copy()).to_type(PrimitiveState).data
    rng = np.random.default_rng(seed * 1000003 + block.global_block_num)
    n = W.shape[:2]
    W[:, :, 0] *= 1 + rng.uniform(-0.02, 0.02, n)
    W[:, :, 3] *= 1 + rng.uniform(-0.02, 0.02, n)
    W[:, :, 1] += rng.uniform(-0.01, 0.01, n)
    W[:, :, 2] += rng.uniform(-0.01, 0.01, n)
    block.state.data = PrimitiveState(fl, array=W).to_type(ConservativeState).data


def make_solver(n: int, device_solver: bool = True):
    """Euler2D for the workload with the initial condition applied (state on host)."""
    from pyhype_gb300.fluids import Air
    from pyhype_gb300.initial_conditions import ExplosionInitialCondition
    from pyhype_gb300.mesh import RectagularMeshGenerator
    from pyhype_gb300.solver_config import SolverConfig
    from pyhype_gb300.states import ConservativeState

    air = Air(a_inf=343.0, rho_inf=1.0)
    cfg = SolverConfig(
        fvm_type="MUSCL", fvm_spatial_order=2, fvm_num_quadrature_points=1, fvm_gradient_type="GreenGauss",
        fvm_flux_function_type="Roe", fvm_slope_limiter_type="Venkatakrishnan", time_integrator="RK4",
        initial_condition=ExplosionInitialCondition(), interface_interpolation="arithmetic_average",
        reconstruction_type=ConservativeState, CFL=0.8, t_final=0.07, fluid=air, nx=n, ny=n, nghost=1,
    )
    mesh = RectagularMeshGenerator.generate(["Reflection"], ["Reflection"], ["Reflection"], ["Reflection"],
                                            east=10.0, west=0.0, north=20.0, south=0.0,
                                            n_blocks_horizontal=2, n_blocks_vertical=4)
    if device_solver:
        from pyhype_gb300.solvers import Euler2D

        s = Euler2D(config=cfg, mesh_config=mesh)
        s.apply_initial_condition()
        for b in s.blocks:
            seeded_state(b, SEED)
        return s, cfg
    # host-only: problem + initial state for the CPU arm
    from pyhype_gb300.problem import problem_from_config
    from pyhype_gb300.solvers import HostBlock

    P = problem_from_config(cfg, mesh.dict)
    blocks = []
    for k, blk in enumerate(P.block_ids):
        d = mesh.dict[blk]
        hb = HostBlock(cfg, blk, P.block_geometry[k], {c: d[c] for c in ("NE", "NW", "SE", "SW")}, {}, {})
        cfg.initial_condition.apply_to_block(hb)
        seeded_state(hb, SEED)
        blocks.append(hb.state.data)
    return (P, P.to_soa(blocks)), cfg


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch
        import torch.distributed as dist

        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(x: float, ws: int) -> float:
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clock / throttle sampling while the timed region runs."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.lines = []
        if self.proc is not None:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()
                out = ""
            self.lines = [ln for ln in out.splitlines() if ln.strip()]

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in getattr(self, "lines", []):
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 8:
                continue
            try:
                sm.append(float(p[0]))
                smax = float(p[1])
            except ValueError:
                continue
            for nm, val in zip(names, p[4:8]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons), "samples": len(sm)}


def oracle_steps(P, U, warmup: int, steps: int, integrator: str = "RK4"):
    """The CPU oracle on every host core, run as the reference's loop body: per step the
    CFL dt, then one RK step advancing the state in place.  ``warmup`` untimed steps,
    then ``steps`` timed ones.  Returns (seconds, threads, (dt, state) after the first
    step or None when that step was timed)."""
    import numpy as np

    from oracle.oracle import Oracle, lib
    from pyhype_gb300.time_marching import tableau

    O = Oracle(P, threads=os.cpu_count() or 1)
    a = tableau(integrator) if isinstance(integrator, str) else integrator
    U = np.array(U, dtype=np.float64, copy=True, order="C").reshape(4, P.ncell)
    first = None
    t = 0.0
    t0 = time.perf_counter()
    for k in range(warmup + steps):
        if k == warmup:
            t0 = time.perf_counter()
        dt = float(O.dt(U)[0])
        O.step(U, a, dt, t, inplace=True)
        t += dt
        if k == 0 and warmup > 0:
            first = (dt, U.copy())
    el = time.perf_counter() - t0
    return el, int(lib().oracle_max_threads()), first


def cpu_baseline(n: int, steps: int):
    """The CPU oracle on every host core: one untimed step, then ``steps`` timed steps
    of the workload (the reference arm's loop body).  Also returns the initial state and
    the oracle's first step for the full-size parity check."""
    (P, U0), cfg = make_solver(n, device_solver=False)
    el, used, first = oracle_steps(P, U0, warmup=1, steps=steps)
    return {
        "value": P.ncell * 4 * steps / el,
        "unit": "cell-stage updates/s",
        "cores": used,
        "kind": "port",
        "sample": f"{steps} timed RK4 step(s) of the full {P.ncell}-cell workload after 1 untimed step, each the "
                  f"CFL dt plus one step in place, {el:.2f} s wall on {used} threads",
    }, U0, first


def step_parity(P, U0, tableau_a, dt_ref, U1_ref, t: float = 0.0):
    """One step of the device FP64 path from U0 against the oracle's step (dt and
    state, value for value)."""
    import numpy as np

    from pyhype_gb300._native import DeviceSolver

    S = DeviceSolver(P, tableau=tableau_a)
    try:
        S.set_state(U0)
        dt = float(S.compute_dt()[0])
        S.step(dt, t)
        G1 = S.get_state()
    finally:
        S.close()
    diff = np.abs(G1 - U1_ref)
    return {"dt_equal": dt == dt_ref, "max_abs_diff": float(np.max(diff)),
            "max_rel_diff": float(np.max(diff / np.maximum(np.abs(U1_ref), 1e-300))),
            "bitwise": bool(dt == dt_ref and np.array_equal(G1, U1_ref)), "cells": int(P.ncell)}


def ensemble_section(stream, full: bool = False, autotune: bool = True):
    """512 seeded explosion instances of uneven sizes (64..512 per side), Roe/Venkat,
    SSP-RK2, CFL 0.5, per-instance dt: FP32 batched vs FP64 batched vs FP64 instances
    solved one after another, and the FP32 L1 density difference at equal steps."""
    import numpy as np
    import torch

    from pyhype_gb300.batch import EnsembleSolver, ensemble_problem, explosion_ensemble

    inst = explosion_ensemble(512, seed=0)
    P = ensemble_problem(inst, precision=0, cfl=0.5)
    cells = P.ncell
    stages = 2
    k32, w = (200, 3) if full else (20, 3)
    k64 = 200 if full else 10
    out = {"workload": "512 instances, nx,ny in {64..512} (seed 0), explosion IC, Roe/Venkatakrishnan, SSP-RK2, "
                       "CFL 0.5, per-instance dt", "cells": cells}

    halted = {"fp32": set(), "fp64": set()}

    def timed(solver, steps, key=None):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        bad = solver.run(steps)
        e1.record(stream)
        torch.cuda.synchronize()
        if key:
            halted[key].update(bad)
        return e0.elapsed_time(e1)

    E32 = EnsembleSolver(inst, precision=1, problem=P)
    E32.device.set_stream(stream.cuda_stream)
    T0 = {"fp32": E32.device.totals()}
    if autotune:
        out["fp32_autotune"] = E32.device.autotune(reps=2)
    halted["fp32"].update(E32.run(w))
    ms32 = timed(E32, k32, "fp32")
    out["fp32_batched"] = {"value": cells * stages * k32 / (ms32 * 1e-3), "unit": "cell-stage updates/s",
                           "steps": k32, "ms_per_step": ms32 / k32}
    E64 = EnsembleSolver(inst, precision=0, problem=P)
    E64.device.set_stream(stream.cuda_stream)
    T0["fp64"] = E64.device.totals()
    halted["fp64"].update(E64.run(w))
    ms64 = timed(E64, k64, "fp64")
    out["fp64_batched"] = {"value": cells * stages * k64 / (ms64 * 1e-3), "unit": "cell-stage updates/s",
                           "steps": k64, "ms_per_step": ms64 / k64}
    if w + k64 < w + k32:
        halted["fp64"].update(E64.run(k32 - k64))
    a, b = E64.states(), E32.states()
    bad = halted["fp32"] | halted["fp64"]
    l1 = [float(np.sum(np.abs(y[:, :, 0] - x[:, :, 0])) / np.sum(np.abs(x[:, :, 0])))
          for k, (x, y) in enumerate(zip(a, b)) if k not in bad]
    out["fp32_l1_density_rel_vs_fp64"] = {"after_steps": w + k32, "mean": float(np.mean(l1)), "max": float(np.max(l1)),
                                           "median": float(np.median(l1)), "instances": len(l1)}
    # conservation (single reflecting blocks conserve mass and energy up to rounding):
    # relative drift of each instance's FP64 totals over the run, largest over instances
    keep = [k for k in range(len(inst)) if k not in bad]
    drift = {}
    for key, E in (("fp32", E32), ("fp64", E64)):
        T1 = E.device.totals()
        with np.errstate(divide="ignore", invalid="ignore"):  # momentum totals are 0
            d = np.abs(T1[keep] - T0[key][keep]) / np.abs(T0[key][keep])
        drift[key] = {"mass_max": float(d[:, 0].max()), "energy_max": float(d[:, 3].max())}
    out["conservation_drift"] = dict(drift, after_steps=w + k32)
    out["halted_unrealizable"] = {"fp32": sorted(halted["fp32"]), "fp64": sorted(halted["fp64"]),
                                  "note": "the reference scheme reaches NaN on these instances (checked in the CPU "
                                          "oracle for instance 265); they are excluded from the L1 statistics"}
    if full:
        # the FP64 scheme's own sensitivity to round-off: the same run from an initial
        # state whose densities and energies are one ulp larger
        from pyhype_gb300.batch import ensemble_state

        E64p = EnsembleSolver(inst, precision=0, problem=P)
        E64p.device.set_stream(stream.cuda_stream)
        U = ensemble_state(P, inst)
        U[0] = np.nextafter(U[0], np.inf)
        U[3] = np.nextafter(U[3], np.inf)
        E64p.device.set_state(U)
        bad_p = set(E64p.run(w)) | set(E64p.run(k32))
        c = E64p.states()
        l1p = [float(np.sum(np.abs(y[:, :, 0] - x[:, :, 0])) / np.sum(np.abs(x[:, :, 0])))
               for k, (x, y) in enumerate(zip(a, c)) if k not in bad | bad_p]
        out["fp64_one_ulp_initial_change_l1_density"] = {
            "after_steps": w + k32, "mean": float(np.mean(l1p)), "max": float(np.max(l1p)),
            "median": float(np.median(l1p)),
            "note": "FP64 run from densities and energies one ulp larger, against the FP64 run: the scheme's "
                    "own round-off sensitivity (the reference limiter switches psi between 0.75 and ~1 on "
                    "round-off-sized face differences)"}
        E64p.device.close()
    # FP64 instances one after another (each its own device problem)
    nseq = 512 if full else 16
    seq_ms, seq_cells = 0.0, 0
    for one in inst[:nseq]:
        S = EnsembleSolver([one], precision=0)
        S.device.set_stream(stream.cuda_stream)
        S.run(1)
        seq_ms += timed(S, k64)
        seq_cells += S.problem.ncell
        S.device.close()
    out["fp64_sequential"] = {"value": seq_cells * stages * k64 / (seq_ms * 1e-3), "unit": "cell-stage updates/s",
                              "instances_timed": nseq, "steps": k64}
    out["fp32_batched_over_fp64_sequential"] = out["fp32_batched"]["value"] / out["fp64_sequential"]["value"]
    E32.device.close()
    E64.device.close()
    return out


def adjoint_section(stream, nsteps: int = 400, ckpt: int = 20, n: int = 256, fd: bool = True,
                    precision: str = "fp64"):
    """Adjoint configuration: one 256 x 256 block on [0,10]^2, Reflection sides,
    Roe/Venkatakrishnan, RK4 at CFL 0.5, 400 steps; tanh-edged explosion with
    (r, w, cx) = (4, 2, 5); J = sum_n dt_n * (pressure integral along the north wall).
    Times the recorded forward pass, the reverse pass (segment recompute + reverse
    kernels) and a plain forward run of the same steps; checks dJ/d(r, w, cx) against
    central differences (h = 1e-6 and 1e-3) at the frozen dt schedule."""
    import numpy as np
    import torch

    from pyhype_gb300.adjoint import AdjointSolver, adjoint_problem, smoothed_explosion

    P = adjoint_problem(n=n)
    A = AdjointSolver(P, "RK4", side="N", nsteps=nsteps, ckpt_every=ckpt, precision=precision)
    A.device.set_stream(stream.cuda_stream)
    theta = torch.tensor([4.0, 2.0, 5.0], dtype=torch.float64, device="cuda", requires_grad=True)
    with torch.cuda.stream(stream):
        U0 = smoothed_explosion(P, theta[0], theta[1], theta[2])
    U0d = U0.detach().clone()
    # warm-up (first-touch allocations of the checkpoint and segment storage)
    A.forward(U0d)
    A.backward()

    def ev():
        return torch.cuda.Event(enable_timing=True)

    e0, e1, e2 = ev(), ev(), ev()
    torch.cuda.synchronize()
    e0.record(stream)
    J = A.forward(U0d)
    e1.record(stream)
    A.backward()
    e2.record(stream)
    torch.cuda.synchronize()
    t_fwd, t_bwd = e0.elapsed_time(e1), e1.elapsed_time(e2)
    # plain forward of the same steps (captured-graph device loop)
    A.device.set_state_device(U0d.data_ptr())
    f0, f1 = ev(), ev()
    f0.record(stream)
    A.device.run(0.0, float("inf"), max_steps=nsteps)
    f1.record(stream)
    torch.cuda.synchronize()
    t_plain = f0.elapsed_time(f1)
    out = {"workload": f"{n}x{n} block on [0,10]^2, Reflection, Roe/Venkatakrishnan, RK4, CFL 0.5, {nsteps} steps, "
                       f"checkpoints every {ckpt}; tanh-edged explosion (r, w, cx) = (4, 2, 5); "
                       "J = sum dt * north-wall pressure integral",
           "J": J, "forward_recorded_ms": t_fwd, "backward_ms": t_bwd, "plain_forward_ms": t_plain,
           "adjoint_cost_over_forward": t_bwd / t_plain,
           "adjoint_cost_over_recorded_forward": t_bwd / t_fwd, "precision": precision}
    if fd:
        J1 = A.objective(smoothed_explosion(P, theta[0], theta[1], theta[2]))
        J1.backward()
        grad = theta.grad.cpu().numpy()
        dts = A.dts.copy()
        gnorm = float(np.linalg.norm(grad))
        res = {}
        for k, name in enumerate(("r", "w", "cx")):
            row = {"adjoint": float(grad[k]), "central_difference": {}, "err_over_grad_norm": {}}
            for h in (1e-6, 1e-3):
                tp, tm = theta.detach().clone(), theta.detach().clone()
                tp[k] += h
                tm[k] -= h
                Jp = A.forward(smoothed_explosion(P, tp[0], tp[1], tp[2]), dts)
                Jm = A.forward(smoothed_explosion(P, tm[0], tm[1], tm[2]), dts)
                fdv = (Jp - Jm) / (2 * h)
                row["central_difference"][f"h={h:g}"] = fdv
                row["err_over_grad_norm"][f"h={h:g}"] = abs(fdv - grad[k]) / gnorm
            res[name] = row
        out["fd_check"] = res
        out["fd_check_note"] = (
            "frozen dt schedule; errors relative to |dJ/d(r,w,cx)|. cx = 5 is the mirror-symmetry point "
            "(dJ/dcx = 0 exactly; the reverse pass gives the first-of-equals subgradient there). Over 400 steps "
            "with this limiter J jumps at round-off scale where the reference's slope rule switches "
            "(psi = 0.75 at davg == 0, about 1 one ulp away), so h = 1e-6 differences measure the jumps; "
            "h = 1e-3 differences track the derivative")
    A.device.close()
    return out


def adjoint_dmr_section(stream, nsteps: int = 200, ckpt: int = 20):
    """Adjoint at the double-Mach size: 5 blocks x 400 x 500 cells, HLLL, primitive
    reconstruction, SSP-RK2 at CFL 0.4 from the double-Mach initial state; J = sum dt *
    pressure integral along the south side of the middle block (the reflecting wall).
    Times the recorded forward pass, the reverse pass and a plain forward run of the
    same steps."""
    import torch

    from pyhype_gb300.adjoint import AdjointSolver
    from pyhype_gb300.configs import double_mach
    from pyhype_gb300.solvers import Euler2D

    cfg, gen = double_mach()
    sim = Euler2D(cfg, gen, precision="fp64")
    sim._pre_process_solve()
    U0 = torch.from_numpy(sim.device.get_state()).cuda()
    P = sim.problem
    sim.device.close()
    A = AdjointSolver(P, "SSPRK2", block=2, side="S", nsteps=nsteps, ckpt_every=ckpt)
    A.device.set_stream(stream.cuda_stream)
    A.forward(U0)  # first-touch allocations of the checkpoint and segment storage
    A.backward()

    def ev():
        return torch.cuda.Event(enable_timing=True)

    e0, e1, e2, f0, f1 = ev(), ev(), ev(), ev(), ev()
    torch.cuda.synchronize()
    e0.record(stream)
    J = A.forward(U0)
    e1.record(stream)
    g = A.backward()
    e2.record(stream)
    A.device.set_state_device(U0.data_ptr())
    f0.record(stream)
    A.device.run(0.0, float("inf"), max_steps=nsteps)
    f1.record(stream)
    torch.cuda.synchronize()
    t_plain = f0.elapsed_time(f1)
    out = {"workload": f"double-Mach reflection 5 x 400x500 cells, HLLL/Venkatakrishnan, primitive reconstruction, "
                       f"SSP-RK2, CFL 0.4, {nsteps} steps, checkpoints every {ckpt}; J = sum dt * south-wall "
                       "pressure integral of the middle block",
           "J": J, "forward_recorded_ms": e0.elapsed_time(e1), "backward_ms": e1.elapsed_time(e2),
           "plain_forward_ms": t_plain, "adjoint_cost_over_forward": e1.elapsed_time(e2) / t_plain,
           "grad_finite": bool(torch.isfinite(g).all().item())}
    A.device.close()
    return out


def adjoint_study(limiters=("Venkatakrishnan", "BarthJespersen"), steps=(100, 200, 400), n: int = 256):
    """Central differences of J against the reverse pass, for several step counts and
    difference steps h, on the adjoint configuration off its symmetry point
    ((r, w, cx) = (4, 2, 5.3)); prints one line per case."""
    import torch

    from pyhype_gb300.adjoint import AdjointSolver, adjoint_problem, smoothed_explosion

    res = {}
    for lim in limiters:
        P = adjoint_problem(n=n, limiter=lim)
        for nsteps in steps:
            A = AdjointSolver(P, "RK4", side="N", nsteps=nsteps, ckpt_every=20)
            theta = torch.tensor([4.0, 2.0, 5.3], dtype=torch.float64, device="cuda", requires_grad=True)
            J = A.objective(smoothed_explosion(P, theta[0], theta[1], theta[2]))
            J.backward()
            g = theta.grad.cpu().numpy()
            dts = A.dts.copy()
            row = {"J": J.item(), "adjoint": g.tolist(), "rel_err": {}}
            for h in (1e-2, 1e-3, 1e-4, 1e-5, 1e-6, 1e-7):
                errs = []
                for k in range(3):
                    tp, tm = theta.detach().clone(), theta.detach().clone()
                    tp[k] += h
                    tm[k] -= h
                    fd = (A.forward(smoothed_explosion(P, tp[0], tp[1], tp[2]), dts)
                          - A.forward(smoothed_explosion(P, tm[0], tm[1], tm[2]), dts)) / (2 * h)
                    errs.append(abs(fd - g[k]) / max(abs(g[k]), 1e-300))
                row["rel_err"][f"{h:g}"] = errs
            res[f"{lim} {n}x{n} {nsteps} steps"] = row
            print(json.dumps({f"{lim} {n}x{n} {nsteps} steps": row}), flush=True)
            A.device.close()
    return res


def dmr_section(stream, sensitivity: bool = False):
    """Mach-10 double-Mach reflection: [0,4] x [0,1] as 5 blocks of 400 x 500 cells
    (dx = dy = 0.002), HLLL/Venkatakrishnan/Green-Gauss, primitive reconstruction,
    SSP-RK2 at CFL 0.4 to t = 0.2, FP64 and FP32 through Euler2D; FP32 L1 density
    difference at t_final.  With ``sensitivity`` also FP64 runs (i) whose initial
    densities and energies are one ulp larger, (ii) from the initial state rounded to
    FP32 once, (iii) on the geometry planes rounded to FP32 once: the FP64 scheme's own
    response to the perturbations that any FP32 representation makes, beside the FP32
    form's difference."""
    import numpy as np
    import torch

    from pyhype_gb300.configs import double_mach
    from pyhype_gb300.solvers import Euler2D

    out = {"workload": "double-Mach reflection, 5 blocks x 400x500 cells, HLLL/Venkatakrishnan, primitive "
                       "reconstruction, SSP-RK2, CFL 0.4, t_final 0.2"}
    states = {}
    totals = {}
    start = None
    runs = ("fp64", "fp32") + (("fp64_ulp", "fp64_state32", "fp64_geometry32") if sensitivity else ())
    for prec in runs:
        cfg, gen = double_mach()
        sim = Euler2D(cfg, gen, precision=prec[:4])
        if prec == "fp64_geometry32":
            # the FP64 path on the geometry planes rounded to FP32 once (the FP32 form's
            # geometry, nothing else rounded): round the host planes, upload again
            from pyhype_gb300._native import DeviceSolver

            Pr = sim.problem
            g = Pr.geometry
            planes = [(g.cell[q], Pr.ncell) for q in range(12)]
            planes += [(g.vface[q], Pr.nvface) for q in range(5)] + [(g.hface[q], Pr.nhface) for q in range(5)]
            for ptr, n in planes:
                arr = np.ctypeslib.as_array(ptr, shape=(n,))
                arr[:] = arr.astype(np.float32).astype(np.float64)
            sim.device.close()
            sim.device = DeviceSolver(Pr, tableau=sim._time_integrator.tableau())
        sim.device.set_stream(stream.cuda_stream)
        sim._pre_process_solve()
        if prec == "fp64":
            start = (sim.problem, sim.device.get_state(), sim._time_integrator.tableau())
        if prec == "fp64_ulp":
            U = sim.device.get_state()
            U[0] = np.nextafter(U[0], np.inf)
            U[3] = np.nextafter(U[3], np.inf)
            sim.device.set_state(U)
        if prec == "fp64_state32":  # the initial state rounded to FP32 once, FP64 after
            sim.device.set_state(sim.device.get_state().astype(np.float32).astype(np.float64))
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        sim._solve()
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        sim._post_process_solve()
        cells = sim.problem.ncell
        out[prec] = {"value": cells * 2 * sim.num_time_step / (ms * 1e-3), "unit": "cell-stage updates/s",
                     "steps": sim.num_time_step, "seconds": ms * 1e-3, "t_final_reached": sim.t >= sim.t_final}
        states[prec] = np.concatenate([b.state.data[:, :, 0].ravel() for b in sim.blocks])
        totals[prec] = sim.device.totals()[0]
        sim.device.close()
    a, b = states["fp64"], states["fp32"]
    out["fp32_l1_density_rel_vs_fp64"] = float(np.sum(np.abs(b - a)) / np.sum(np.abs(a)))
    if sensitivity:
        l1 = lambda k: float(np.sum(np.abs(states[k] - a)) / np.sum(np.abs(a)))  # noqa: E731
        out["fp64_one_ulp_initial_change_l1_density"] = l1("fp64_ulp")
        out["fp64_initial_state_rounded_to_fp32_l1_density"] = l1("fp64_state32")
        out["fp64_geometry_rounded_to_fp32_l1_density"] = l1("fp64_geometry32")
        for k in ("fp64_ulp", "fp64_state32", "fp64_geometry32"):
            out.pop(k, None)
    # inflow and outflow sides: the totals are not conserved; FP32 against FP64 at t_final
    out["fp32_totals_rel_vs_fp64"] = {
        "mass": float(abs(totals["fp32"][0] - totals["fp64"][0]) / abs(totals["fp64"][0])),
        "energy": float(abs(totals["fp32"][3] - totals["fp64"][3]) / abs(totals["fp64"][3]))}
    out["fp32_over_fp64"] = out["fp32"]["value"] / out["fp64"]["value"]
    # parity at full size: the first FP64 step on the device against the CPU oracle's
    P, U0, a = start
    _, _, first = oracle_steps(P, U0, warmup=1, steps=0, integrator=a)
    out["parity"] = step_parity(P, U0, a, *first)
    return out


def run_reference(args, ws, rank):
    """--impl reference: the reference algorithm's CPU implementation (C restatement,
    all host threads) on the same workload, through the same loop body as the CPU
    baseline of the GPU arm (CFL dt + one RK step in place per step); rank 0 only."""
    if rank != 0:
        return
    (P, U), cfg = make_solver(args.n, device_solver=False)
    el, used, _ = oracle_steps(P, U, warmup=args.warmup, steps=args.steps)
    value = P.ncell * 4 * args.steps / el
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "cell-stage updates/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "cells": P.ncell, "blocks": 8, "stages_per_step": 4,
                   "l2": "inputs larger than L2 (state 268 MB)", "parallelism": "host cores"},
        "cpu_baseline": {"value": value, "unit": "cell-stage updates/s", "cores": used, "kind": "port",
                         "sample": f"every step is the CFL dt plus one full RK4 step of the workload in place, "
                                   f"on {used} host threads"},
        "e2e": {"value": value, "unit": "cell-stage updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    ws, rank, local = dist_init()
    if args.impl == "reference":
        run_reference(args, ws, rank)
        return
    if args.warmup < 3:
        raise SystemExit("--warmup must be >= 3")
    if args.workload == "adjoint":
        import torch

        torch.cuda.set_device(local)
        if rank == 0:
            st = torch.cuda.Stream()
            res = adjoint_section(st, nsteps=args.steps, ckpt=max(1, args.steps // 2), n=args.n, fd=False,
                                  precision=args.precision)
            print(json.dumps({"metric": "adjoint cost", "adjoint": res}), flush=True)
        return
    if args.workload == "adjoint-study":
        import torch

        torch.cuda.set_device(local)
        if rank == 0:
            adjoint_study()
        return
    if args.workload == "dmr":
        import torch

        torch.cuda.set_device(local)
        st = torch.cuda.Stream()
        res = dmr_section(st, sensitivity=True)
        if rank == 0:
            print(json.dumps({"metric": "cell-stage updates/s, double-Mach reflection", "dmr": res}), flush=True)
        return
    if args.workload == "ensemble":
        import torch

        torch.cuda.set_device(local)
        st = torch.cuda.Stream()
        res = ensemble_section(st, full=True)
        if rank == 0:
            print(json.dumps({"metric": "cell-stage updates/s, batched ensemble", "ensemble": res}), flush=True)
        return
    import ctypes

    import numpy as np
    import torch

    from pyhype_gb300 import _native
    from pyhype_gb300.roofline import (BYTES_PER_CELL_STAGE_FP32, BYTES_PER_CELL_STAGE_FP64, FP64_INST_PER_CELL,
                                       FP64_INST_PER_SM_CLOCK, kernel_flops)

    # the CPU baseline first, while this process has done no GPU work: timed after the
    # GPU sections it ran up to 20 % slower than the same loop in a fresh process
    cpu = None
    if rank == 0 and ws == 1 and not args.skip_cpu_baseline and args.precision == "fp64":
        try:
            cpu = cpu_baseline(args.n, args.cpu_steps)
        except Exception as exc:  # the GPU number stands without it
            cpu = exc
    torch.cuda.set_device(local)
    solver, cfg = make_solver(args.n)
    dev = solver.device
    P = solver.problem
    if args.precision == "fp32":  # the FP32 form alone (profiling runs; the default line is FP64)
        S32 = _native.DeviceSolver(P.with_precision(1), tableau=solver._time_integrator.tableau())
        if args.stage_form != "default":
            S32.set_kernel_choice(3, {"split": 0, "fused28": 1, "fused13": 2}[args.stage_form])
        S32.set_state(P.to_soa([b.state.data for b in solver.blocks]))
        t32, _ = S32.run(0.0, 1e30, max_steps=args.warmup)
        g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        g0.record()
        S32.run(t32, 1e30, max_steps=args.steps)
        g1.record()
        torch.cuda.synchronize()
        ms32 = g0.elapsed_time(g1)
        if rank == 0:
            print(json.dumps({"metric": "cell-stage updates/s (FP32 form, multiblock explosion)", "value":
                              P.ncell * 4 * args.steps / (ms32 * 1e-3), "unit": "cell-stage updates/s",
                              "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
                              "ms_per_step": ms32 / args.steps, "dtype": "f32", "cells": P.ncell}), flush=True)
        return
    stream = torch.cuda.Stream()
    dev.set_stream(stream.cuda_stream)
    solver.upload()
    L = _native.load()
    L.e2d_bench_fp64_peak.argtypes = [ctypes.c_int32, ctypes.c_void_p]
    L.e2d_bench_kernels.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p]

    t = 0.0
    t_final = 1e30
    t, _ = dev.run(t, t_final, max_steps=args.warmup)
    torch.cuda.synchronize()
    barrier(ws)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        e0.record(stream)
        t, done = dev.run(t, t_final, max_steps=args.steps)
        e1.record(stream)
        torch.cuda.synchronize()
    assert done == args.steps
    ms = e0.elapsed_time(e1)
    ms = max_over_ranks(ms, ws)
    stages = 4
    value = ws * P.ncell * stages * args.steps / (ms * 1e-3)

    # e2e through the C ABI with host buffers (pinned), one step per call
    host = torch.empty((4, P.ncell), dtype=torch.float64, pin_memory=True)
    dev.get_state(host.numpy())
    e2e_steps = max(3, min(args.steps, 10))
    barrier(ws)
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    for _ in range(e2e_steps):
        L.e2d_set_state(dev.h, ctypes.c_void_p(host.data_ptr()))
        t, _ = dev.run(t, t_final, max_steps=1)
        L.e2d_get_state(dev.h, ctypes.c_void_p(host.data_ptr()))
    f1.record(stream)
    torch.cuda.synchronize()
    ms_e2e = max_over_ranks(f0.elapsed_time(f1), ws)
    e2e_value = ws * P.ncell * stages * e2e_steps / (ms_e2e * 1e-3)
    nbytes = 4 * P.ncell * 8

    # per-kernel event timing + measured FP64 rate -> roofline of the dominant kernel
    kms = np.zeros(6)
    kcnt = np.zeros(6, dtype=np.int64)
    code = L.e2d_bench_kernels(dev.h, 2, kms.ctypes.data, kcnt.ctypes.data)
    if code != 0:
        raise RuntimeError(L.e2d_last_error().decode())
    names = ["dt", "reconstruct", "flux", "update", "bookkeeping", "fused_stage"]
    share = kms * kcnt
    dom = int(np.argmax(share))
    # inter-block halo: reconstruction over the real tiles against the same number of
    # tiles with those along inter-block sides (and along any side) made interior
    halo = None
    try:
        L.e2d_bench_halo.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p]
        hms = np.zeros(3)
        hn = np.zeros(3, dtype=np.int64)
        if L.e2d_bench_halo(dev.h, 10, hms.ctypes.data, hn.ctypes.data) != 0:
            raise RuntimeError(L.e2d_last_error().decode())
        t, _ = dev.run(t, t_final, max_steps=1)  # face arrays rebuilt by a full step
        halo = {"reconstruct_ms": float(hms[0]), "inter_block_tiles_made_interior_ms": float(hms[1]),
                "all_side_tiles_made_interior_ms": float(hms[2]), "tiles": int(hn[0]),
                "inter_block_side_tiles": int(hn[1]), "side_tiles": int(hn[2]),
                "inter_block_halo_ms_per_stage": float(hms[0] - hms[1]),
                "halo_and_bc_ms_per_stage": float(hms[0] - hms[2]),
                "inter_block_halo_share_of_step": float((hms[0] - hms[1]) * stages / (ms / args.steps)),
                "note": "ghost cells and boundary face states are formed inside the reconstruction kernel's "
                        "side tiles; no separate halo pass or copy"}
    except Exception as exc:
        halo = {"error": str(exc)}
    peak_fma = ctypes.c_double(0.0)
    peak_add = ctypes.c_double(0.0)
    L.e2d_bench_fp64_peak(0, ctypes.byref(peak_fma))
    L.e2d_bench_fp64_peak(1, ctypes.byref(peak_add))
    flops = kernel_flops(names[dom], P.ncell, P.nvface, P.nhface)
    achieved = flops / (kms[dom] * 1e-3) / 1e12
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "traffic_per_cell.json")
    if os.path.exists(tpath):
        with open(tpath) as fh:
            tr = json.load(fh)
        if names[dom] in tr:
            traffic = tr[names[dom]] * P.ncell
    peaks = {}
    ppath = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(ppath):
        with open(ppath) as fh:
            peaks = json.load(fh)
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    step_ms = ms / args.steps
    hbm_achieved = P.ncell * stages * BYTES_PER_CELL_STAGE_FP64 / (step_ms * 1e-3) / 1e9

    # FP64 fused stage forms on the same workload (for comparison; the line's value is
    # the default form)
    fp64_fused = {}
    try:
        for form, name in ((1, "fused28"), (2, "fused13")):
            SF = _native.DeviceSolver(P, tableau=solver._time_integrator.tableau())
            SF.set_stream(stream.cuda_stream)
            SF.set_kernel_choice(3, form)
            SF.set_state(P.to_soa([b.state.data for b in solver.blocks]))
            tf_, _ = SF.run(0.0, t_final, max_steps=args.warmup)
            h0, h1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            h0.record(stream)
            SF.run(tf_, t_final, max_steps=args.steps)
            h1.record(stream)
            torch.cuda.synchronize()
            fms = h0.elapsed_time(h1) / args.steps
            fp64_fused[name] = {"ms_per_step": fms, "value": P.ncell * stages / (fms * 1e-3),
                                "speedup_vs_split": step_ms / fms}
            SF.close()
    except Exception as exc:
        fp64_fused = {"error": str(exc)}

    # FP32 form on the same workload and seeded state (same warm-up + timed steps), both
    # stage forms; the faster one is the form's number
    fp32 = None
    try:
        forms = {}
        for form, name in ((0, "split"), (1, "fused28"), (2, "fused13")):
            S32 = _native.DeviceSolver(P.with_precision(1), tableau=solver._time_integrator.tableau())
            S32.set_stream(stream.cuda_stream)
            S32.set_kernel_choice(3, form)
            S32.set_state(P.to_soa([b.state.data for b in solver.blocks]))
            t32, _ = S32.run(0.0, t_final, max_steps=args.warmup)
            g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            g0.record(stream)
            t32, _ = S32.run(t32, t_final, max_steps=args.steps)
            g1.record(stream)
            torch.cuda.synchronize()
            forms[name] = (max_over_ranks(g0.elapsed_time(g1), ws), S32.get_state(), S32)
        best = min(forms, key=lambda k: forms[k][0])
        ms32, U32, S32 = forms[best]
        forms_equal = all(bool(np.array_equal(forms["split"][1], v[1])) for v in forms.values())
        for k, v in forms.items():
            if k != best:
                v[2].close()
        # the FP64 solver has taken e2e steps more; rerun FP64 to the same step count
        S64b = _native.DeviceSolver(P, tableau=solver._time_integrator.tableau())
        S64b.set_stream(stream.cuda_stream)
        S64b.set_state(P.to_soa([b.state.data for b in solver.blocks]))
        tot0 = S64b.totals()[0]
        S64b.run(0.0, t_final, max_steps=args.warmup + args.steps)
        U64 = S64b.get_state()
        l1 = float(np.sum(np.abs(U32[0] - U64[0])) / np.sum(np.abs(U64[0])))
        tot64, tot32 = S64b.totals()[0], S32.totals()[0]
        conservation = {
            "totals_rel_vs_fp64": {"mass": float(abs(tot32[0] - tot64[0]) / abs(tot64[0])),
                                   "energy": float(abs(tot32[3] - tot64[3]) / abs(tot64[3]))},
            "drift_fp64": {"mass": float((tot64[0] - tot0[0]) / abs(tot0[0])),
                           "energy": float((tot64[3] - tot0[3]) / abs(tot0[3]))},
            "drift_fp32": {"mass": float((tot32[0] - tot0[0]) / abs(tot0[0])),
                           "energy": float((tot32[3] - tot0[3]) / abs(tot0[3]))},
            "note": "FP64 sums of A*U; the 2x4 layout is not conservative across blocks (the reference's "
                    "inter-block faces), so the drift includes the scheme's own"}
        # per-kernel timing advances the FP32 state further: after the comparison
        k32 = np.zeros(6)
        c32 = np.zeros(6, dtype=np.int64)
        L.e2d_bench_kernels(S32.h, 2, k32.ctypes.data, c32.ctypes.data)
        b32 = BYTES_PER_CELL_STAGE_FP32
        ach32 = P.ncell * stages * b32 / (ms32 / args.steps * 1e-3) / 1e9
        fp32 = {"value": ws * P.ncell * stages * args.steps / (ms32 * 1e-3), "unit": "cell-stage updates/s",
                "ms_per_step": ms32 / args.steps, "speedup_vs_fp64": ms / ms32, "stage_form": best,
                "forms_ms_per_step": {k: v[0] / args.steps for k, v in forms.items()},
                "forms_bitwise_equal": forms_equal,
                "l1_density_rel_vs_fp64": l1, "l1_after_steps": args.warmup + args.steps,
                "conservation": conservation,
                "kernel_ms": {n: float(x) for n, x in zip(names, k32)},
                "roofline": {"bound": "hbm", "achieved": ach32, "peak": hbm_peak, "unit": "GB/s",
                             "frac": ach32 / hbm_peak, "bytes_per_cell_stage": b32,
                             "note": "whole-step algorithmic bytes (stage program state values, geometry, "
                                     "CFL dt; pyhype_gb300/roofline.py) / ms per step; peak "
                                     + ("MEASURED_PEAKS.json hbm_gbs" if "hbm_gbs" in peaks else "fallback")}}
        S32.close()
        S64b.close()
    except Exception as exc:
        fp32 = {"error": str(exc)}

    ensemble = None
    if not args.skip_ensemble and ws == 1:
        try:
            ensemble = ensemble_section(stream)
            ensemble["fp32_batched_over_fp64_plain"] = ensemble["fp32_batched"]["value"] / value
        except Exception as exc:
            ensemble = {"error": str(exc)}

    adjoint = None
    if not args.skip_adjoint and ws == 1:
        try:
            adjoint = adjoint_section(stream)
            a32 = adjoint_section(stream, fd=False, precision="fp32")
            adjoint["fp32"] = {k: a32[k] for k in ("J", "backward_ms", "plain_forward_ms",
                                                   "adjoint_cost_over_forward")}
            adjoint["double_mach_hlll"] = adjoint_dmr_section(stream)
        except Exception as exc:
            adjoint = {"error": str(exc)}

    dmr = None
    parity = {}
    if not args.skip_dmr and ws == 1:
        try:
            dmr = dmr_section(stream)
            parity["dmr_ssprk2_step"] = dmr.pop("parity")
        except Exception as exc:
            dmr = {"error": str(exc)}

    clocks = clk.summary()
    # FP64 issue view of the dominant kernel: arithmetic FP64 instructions per second
    # against the pipe's issue limit at the sampled SM clock
    fp64_issue = None
    if names[dom] in FP64_INST_PER_CELL and clocks.get("sm_mhz"):
        nsm = torch.cuda.get_device_properties(0).multi_processor_count
        ipeak = FP64_INST_PER_SM_CLOCK * nsm * clocks["sm_mhz"] * 1e6
        iach = FP64_INST_PER_CELL[names[dom]] * P.ncell / (kms[dom] * 1e-3)
        fp64_issue = {"achieved_ginst_s": iach / 1e9, "peak_ginst_s": ipeak / 1e9, "frac": iach / ipeak,
                      "inst_per_cell": FP64_INST_PER_CELL[names[dom]],
                      "source": "DADD+DMUL+DFMA per cell counted by ncu; peak 2 per SM per clock at the "
                                "sampled SM clock"}
    line = {
        "metric": METRIC,
        "value": value,
        "unit": "cell-stage updates/s",
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": step_ms,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "cells": P.ncell, "blocks": P.nblocks, "stages_per_step": stages,
                   "l2": "inputs larger than L2 (state 268 MB, ~2.5 GB streamed per stage)",
                   "parallelism": "replicas" if ws > 1 else "single GPU"},
        "e2e": {"value": e2e_value, "unit": "cell-stage updates/s", "h2d_bytes_per_step": nbytes,
                "d2h_bytes_per_step": nbytes, "steps": e2e_steps},
        "roofline": {
            "bound": "fp64", "kernel": names[dom], "achieved": achieved, "peak": peak_fma.value,
            "unit": "TFLOP/s", "frac": achieved / peak_fma.value if peak_fma.value else None,
            # the parity build may not contract a*b+c, so every algorithmic flop takes at
            # least one FP64 instruction: against the unfused (DADD) rate
            "frac_unfused": achieved / peak_add.value if peak_add.value else None,
            "traffic": traffic,
            "peak_source": "measured in-run: DFMA chains over all SMs (2 flops per DFMA); DADD rate "
                           f"{peak_add.value:.3f} TFLOP/s",
            "kernel_ms": {n: float(x) for n, x in zip(names, kms)},
            "kernel_share": {n: float(s / share.sum()) for n, s in zip(names, share)},
            "halo": halo,
            "flops_per_launch": flops,
            "fp64_issue": fp64_issue,
            "hbm": {"achieved_gbs": hbm_achieved, "peak_gbs": hbm_peak,
                    "frac": hbm_achieved / hbm_peak, "bytes_per_cell_stage": BYTES_PER_CELL_STAGE_FP64,
                    "peak_source": "MEASURED_PEAKS.json hbm_gbs" if "hbm_gbs" in peaks else "fallback"},
        },
        "fp32": fp32,
        "fp64_fused_stage": fp64_fused,
        "ensemble": ensemble,
        "adjoint": adjoint,
        "dmr": dmr,
        "gpu_launches": int(args.steps * (3 + 3 * stages)),
        "clocks": clocks,
    }
    if cpu is not None:
        try:
            if isinstance(cpu, Exception):
                raise cpu
            line["cpu_baseline"], U0, first = cpu
            # full-size parity: the device's first FP64 step from the same seeded state
            if not np.array_equal(U0, P.to_soa([b.state.data for b in solver.blocks])):
                raise RuntimeError("CPU and GPU arms start from different states")
            parity["multiblock_rk4_step"] = step_parity(P, U0, solver._time_integrator.tableau(), *first)
        except Exception as exc:  # the GPU number stands without it
            line["cpu_baseline"] = {"value": None, "error": str(exc)}
    if parity:
        line["parity"] = {"bitwise": all(v.get("bitwise", False) for v in parity.values()),
                          "max_abs_diff": max(v.get("max_abs_diff", float("inf")) for v in parity.values()),
                          **parity}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
