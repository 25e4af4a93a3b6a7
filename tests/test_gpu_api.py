"""The Euler2D drop-in end to end: construction from a SolverConfig and a mesh
dictionary, initial condition on host block proxies, solve() on the device, the
reference's snapshot files, and the positivity abort."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _config(n, t_final, **kw):
    from pyhype_gb300.configs import explosion

    return explosion(n, t_final=t_final, **kw)


def test_solve_matches_oracle_and_writes_reference_snapshots(tmp_path):
    from oracle.oracle import Oracle
    from pyhype_gb300.solvers import Euler2D
    from pyhype_gb300.time_marching import tableau

    cfg, mesh = _config(40, 0.003, write_solution=True, write_solution_base=str(tmp_path),
                        write_solution_name="explosion", write_every_n_timesteps=4)
    sim = Euler2D(config=cfg, mesh_config=mesh)
    sim.solve()
    assert sim.t == sim.t_final
    steps = sim.num_time_step
    assert steps >= 8
    # the same run on the CPU oracle, snapshot numbering of the reference's write_solution
    P = sim.problem
    ic = Euler2D(config=cfg, mesh_config=mesh)
    ic.apply_initial_condition()
    U = P.to_soa([b.state.data for b in ic.blocks])
    O = Oracle(P)
    t = 0.0
    for k in range(steps):
        dt = float(O.dt(U)[0])
        if sim.t_final - t < dt:
            dt = sim.t_final - t
        U = O.step(U, tableau("RK4"), dt, t)
        t += dt
        if k % 4 == 0:
            snap = np.load(os.path.join(tmp_path, "explosion", str(k), "explosion_blk_0.npy"))
            assert np.array_equal(snap, P.from_soa(U)[0]), f"snapshot {k}"
    assert t == sim.t
    assert np.array_equal(next(iter(sim.blocks)).state.data, P.from_soa(U)[0])
    mx = np.load(os.path.join(tmp_path, "explosion", "mesh", "mesh_x_blk_0.npy"))
    assert mx.shape == (40, 40, 1)


def test_fp32_solve_close_to_fp64():
    from pyhype_gb300.solvers import Euler2D

    cfg, mesh = _config(64, 0.005)
    a = Euler2D(config=cfg, mesh_config=mesh)
    a.solve()
    cfg2, mesh2 = _config(64, 0.005)
    b = Euler2D(config=cfg2, mesh_config=mesh2, precision="fp32")
    b.solve()
    ra = next(iter(a.blocks)).state.data[:, :, 0]
    rb = next(iter(b.blocks)).state.data[:, :, 0]
    assert np.sum(np.abs(rb - ra)) / np.sum(np.abs(ra)) < 1e-3  # see test_gpu_fp32 for the bound


def test_unrealizable_state_raises():
    """A host-made bad input (pressure negative in one cell: kinetic energy above E)
    makes the device loop halt and the solver raise, as the reference aborts."""
    from pyhype_gb300.initial_conditions import InitialCondition
    from pyhype_gb300.solvers import Euler2D
    from pyhype_gb300.states import RealizabilityException

    class Bad(InitialCondition):
        def apply_to_block(self, block):
            from pyhype_gb300.initial_conditions import ExplosionInitialCondition

            ExplosionInitialCondition().apply_to_block(block)
            d = block.state.data
            d[5, 5, 1] = 50.0 * d[5, 5, 0]  # |u| = 50 a_inf: E < rho*u^2/2

    cfg, mesh = _config(24, 0.01)
    cfg.initial_condition = Bad()
    sim = Euler2D(config=cfg, mesh_config=mesh)
    with pytest.raises(RealizabilityException):
        sim.solve()


def test_host_rejects_negative_density_before_upload():
    from pyhype_gb300.initial_conditions import InitialCondition
    from pyhype_gb300.solvers import Euler2D
    from pyhype_gb300.states import RealizabilityException

    class Neg(InitialCondition):
        def apply_to_block(self, block):
            block.state.data = np.full(block.state.data.shape, 1.0)
            block.state.data[3, 3, 0] = -1.0

    cfg, mesh = _config(16, 0.01)
    cfg.initial_condition = Neg()
    with pytest.raises(RealizabilityException):
        Euler2D(config=cfg, mesh_config=mesh).solve()
