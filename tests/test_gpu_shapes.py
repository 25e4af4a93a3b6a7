"""Odd block shapes against the oracle: two-cell-wide and two-cell-high blocks (the
smallest the C ABI accepts; e2d_create rejects nx or ny below 2), sizes
that leave partial tiles in both directions, rows whose byte length rules out TMA
staging (odd nx) next to ones that allow it with partial tiles (nx = 34, 66), and
several blocks per side, for the FP64 path (value-exact, three RK4 steps with the
CFL dt) and the FP32 form (finite, close to FP64)."""
import numpy as np
import pytest

from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

SHAPES = [(17, 23, 2, 2), (2, 40, 1, 1), (40, 2, 1, 1), (34, 9, 1, 2), (66, 70, 3, 1), (33, 65, 2, 1)]


@pytest.mark.parametrize("nx,ny,bx,by", SHAPES)
@pytest.mark.parametrize("limiter", ["Venkatakrishnan", "VanLeer"])
def test_fp64_shapes_equal_oracle(nx, ny, bx, by, limiter):
    from test_gpu_slope_pick import _state
    from test_gpu_tma import _problem

    from pyhype_gb300._native import DeviceSolver
    from pyhype_gb300.time_marching import tableau

    P = _problem(nx, ny, bx, by)
    if limiter != "Venkatakrishnan":
        from pyhype_gb300.fluids import Air
        from pyhype_gb300.mesh import RectagularMeshGenerator
        from pyhype_gb300.problem import build_problem

        air = Air(a_inf=343.0, rho_inf=1.0)
        mesh = RectagularMeshGenerator.generate(["Reflection"], ["Reflection"], ["Reflection"], ["Reflection"],
                                                10.0, 0.0, 10.0, 0.0, bx, by)
        P = build_problem(mesh.dict, nx, ny, flux="Roe", limiter=limiter, recon="ConservativeState",
                          gamma=air.gamma(), gm1=air.gamma() - 1, cfl=0.8, fluid=air)
    U = _state(P, seed=nx + ny)
    a = tableau("RK4")
    S = DeviceSolver(P, tableau=a)
    O = Oracle(P)
    S.set_state(U)
    t = 0.0
    for _ in range(3):
        dt = float(S.compute_dt()[0])
        assert dt == float(O.dt(U)[0])
        S.step(dt, t)
        U = O.step(U, a, dt, t)
        t += dt
    assert np.array_equal(S.get_state(), U)
    S.close()


@pytest.mark.parametrize("nx,ny,bx,by", SHAPES)
def test_fp32_shapes_close_to_fp64(nx, ny, bx, by):
    from test_gpu_slope_pick import _state
    from test_gpu_tma import _problem

    from pyhype_gb300._native import DeviceSolver
    from pyhype_gb300.time_marching import tableau

    P = _problem(nx, ny, bx, by)
    U = _state(P, seed=nx + ny)
    a = tableau("RK4")
    out = []
    for prec in (0, 1):
        S = DeviceSolver(P.with_precision(prec), tableau=a)
        S.set_state(U)
        S.run(0.0, 1e30, max_steps=3)
        out.append(S.get_state())
        S.close()
    assert np.all(np.isfinite(out[1]))
    rel = np.sum(np.abs(out[1][0] - out[0][0])) / np.sum(np.abs(out[0][0]))
    assert rel < 1e-3, rel
