"""The FP64 reconstruction kernel evaluates psi only at the faces that decide phi
(pyhype_gb300/csrc/e2d_slope_pick.cuh) and all four where it cannot tell.  On states
that exercise every branch of that choice - random cell noise (slopes spread widely),
smooth waves (many cells whose smallest slope is 2 or more, where both ends of the
slope range are candidates), exactly uniform patches (davg == 0), mirror-symmetric
patches (exact slope ties) - the CUDA path's phi, dUdt and states after RK4 steps
equal the CPU oracle's, which evaluates all four faces, for all four limiters and
both reconstruction types."""
import numpy as np
import pytest

from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

LIMITERS = ["Venkatakrishnan", "BarthJespersen", "VanAlbada", "VanLeer"]


def _problem(limiter, recon):
    from pyhype_gb300.fluids import Air
    from pyhype_gb300.mesh import RectagularMeshGenerator
    from pyhype_gb300.problem import build_problem

    air = Air(a_inf=343.0, rho_inf=1.0)
    mesh = RectagularMeshGenerator.generate(["Reflection"], ["Reflection"], ["Reflection"], ["Reflection"],
                                            10.0, 0.0, 10.0, 0.0, 2, 2)
    return build_problem(mesh.dict, 128, 96, flux="Roe", limiter=limiter, recon=recon, gamma=air.gamma(),
                         gm1=air.gamma() - 1, cfl=0.8, fluid=air)


def _state(P, seed):
    """Non-dimensional conservative state per block: smooth waves in the west half of
    the domain, cell noise in the south-east quarter, a uniform patch and a patch
    mirrored about its centre line in the north-east quarter."""
    from pyhype_gb300.fluids import Air
    from pyhype_gb300.states import ConservativeState, PrimitiveState

    air = Air(a_inf=343.0, rho_inf=1.0)
    rng = np.random.default_rng(seed)
    blocks = []
    for g in P.block_geometry:
        x, y = g.xc, g.yc
        rho = 1.2 + 0.3 * np.sin(0.9 * x) * np.cos(0.7 * y)
        u = 60.0 * np.sin(0.5 * y + 0.3 * x)
        v = 40.0 * np.cos(0.6 * x)
        p = 101100.0 * (1 + 0.2 * np.cos(0.8 * x + 0.4 * y))
        noisy = (x > 5) & (y < 5)
        n = x.shape
        rho = np.where(noisy, 1.2 * (1 + rng.uniform(-0.02, 0.02, n)), rho)
        p = np.where(noisy, 101100.0 * (1 + rng.uniform(-0.02, 0.02, n)), p)
        u = np.where(noisy, rng.uniform(-3.4, 3.4, n), u)
        v = np.where(noisy, rng.uniform(-3.4, 3.4, n), v)
        uni = (x > 5) & (y >= 5) & (x < 7.5)
        rho, u, v, p = (np.where(uni, c, a) for a, c in ((rho, 1.1742), (u, 0.0), (v, 0.0), (p, 101100.0)))
        mir = (x >= 7.5) & (y >= 5)
        bump = np.exp(-((x - 8.75) ** 2))
        rho = np.where(mir, 1.0 + 0.5 * bump, rho)
        p = np.where(mir, 101100.0 * (1 + bump), p)
        u = np.where(mir, 0.0, u)
        v = np.where(mir, 0.0, v)
        W = np.stack([rho, u, v, p], axis=-1)
        s = PrimitiveState(air, array=W).to_type(ConservativeState)
        s.make_non_dimensional()
        blocks.append(s.data)
    return P.to_soa(blocks)


@pytest.mark.parametrize("recon", ["ConservativeState", "PrimitiveState"])
@pytest.mark.parametrize("limiter", LIMITERS)
def test_phi_and_steps_equal_oracle(limiter, recon):
    from pyhype_gb300._native import DeviceSolver
    from pyhype_gb300.time_marching import tableau

    P = _problem(limiter, recon)
    U = _state(P, seed=LIMITERS.index(limiter))
    a = tableau("RK4")
    S = DeviceSolver(P, tableau=a)
    O = Oracle(P)
    S.set_state(U)
    dudt, dbg = S.residual(debug=True)
    ref, rdbg = O.residual(U, debug=True)
    for key in ("gx", "gy", "phi", "vL", "vR", "hL", "hR"):
        assert np.array_equal(dbg[key], rdbg[key]), f"{key}: max diff {np.max(np.abs(dbg[key] - rdbg[key]))}"
    assert np.array_equal(dudt, ref)
    t = 0.0
    for step in range(3):
        dt = float(S.compute_dt()[0])
        assert dt == float(O.dt(U)[0])
        S.step(dt, t)
        U = O.step(U, a, dt, t)
        t += dt
        assert np.array_equal(S.get_state(), U), f"step {step + 1}"
    S.close()
