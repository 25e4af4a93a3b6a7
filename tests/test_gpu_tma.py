"""The reconstruction kernel stages interior tiles (halo inside the block) with one TMA
box load per tile where the block's layout allows it (row stride, plane stride and
base 16-byte aligned), and every other tile with plain loads.  Both stagings must give
the same values: FP64 (conservative and primitive reconstruction) and the FP32 form,
several RK steps with TMA on and off, bitwise; and a layout whose rows are not 16-byte
aligned (odd nx: plain loads everywhere) still equals the oracle."""
import ctypes

import numpy as np
import pytest

from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu


def _problem(nx, ny, nbx, nby, flux="Roe", recon="ConservativeState", precision=0):
    from pyhype_gb300.fluids import Air
    from pyhype_gb300.mesh import RectagularMeshGenerator
    from pyhype_gb300.problem import build_problem

    air = Air(a_inf=343.0, rho_inf=1.0)
    mesh = RectagularMeshGenerator.generate(["Reflection"], ["Reflection"], ["Reflection"], ["Reflection"],
                                            10.0, 0.0, 10.0, 0.0, nbx, nby)
    return build_problem(mesh.dict, nx, ny, flux=flux, limiter="Venkatakrishnan", recon=recon, gamma=air.gamma(),
                         gm1=air.gamma() - 1, cfl=0.8, fluid=air, precision=precision)


def _state(P, seed=0):
    from test_gpu_slope_pick import _state as st

    return st(P, seed)


def _run(P, U, tableau, steps, tma):
    from pyhype_gb300._native import DeviceSolver, load

    L = load()
    L.e2d_bench_set_tma.argtypes = [ctypes.c_void_p, ctypes.c_int32]
    S = DeviceSolver(P, tableau=tableau)
    assert L.e2d_bench_set_tma(S.h, 1 if tma else 0) == 0
    S.set_state(U)
    t, n = S.run(0.0, 1e30, max_steps=steps)
    assert n == steps
    out = S.get_state()
    S.close()
    return out


@pytest.mark.parametrize("flux,recon,precision", [("Roe", "ConservativeState", 0), ("HLLL", "PrimitiveState", 0),
                                                  ("Roe", "ConservativeState", 1)])
def test_tma_and_plain_loads_agree(flux, recon, precision):
    from pyhype_gb300.time_marching import tableau

    P = _problem(160, 96, 2, 2, flux=flux, recon=recon, precision=precision)
    U = _state(P)
    a = tableau("RK4")
    on = _run(P, U, a, 6, True)
    off = _run(P, U, a, 6, False)
    assert np.all(np.isfinite(on))
    assert np.array_equal(on, off)
    if precision == 0:
        O = Oracle(P)
        V = U.copy()
        t = 0.0
        for _ in range(6):
            dt = float(O.dt(V)[0])
            V = O.step(V, a, dt, t)
            t += dt
        assert np.array_equal(on, V)


def test_unaligned_rows_take_plain_loads():
    from pyhype_gb300.time_marching import tableau

    P = _problem(99, 70, 2, 1)  # 99 x 8 bytes per row: no tensor map for these blocks
    U = _state(P)
    a = tableau("RK4")
    got = _run(P, U, a, 3, True)
    O = Oracle(P)
    t = 0.0
    for _ in range(3):
        dt = float(O.dt(U)[0])
        U = O.step(U, a, dt, t)
        t += dt
    assert np.array_equal(got, U)
