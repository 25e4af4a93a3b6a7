"""The FP64 PyTorch transcription (oracle/torch_scheme.py), the checker of the reverse
kernels, reproduces the C oracle value for value, and its autograd gradient agrees
with central finite differences on a smooth initial condition."""
import numpy as np
import pytest
import torch

from oracle.oracle import Oracle
from oracle.torch_scheme import COPY, OUTLET, REFLECT, Geometry, Scheme
from pyhype_gb300.adjoint import adjoint_problem, single_block_mesh, smoothed_explosion
from pyhype_gb300.fluids import Air
from pyhype_gb300.problem import build_problem
from pyhype_gb300.time_marching import tableau


def _smooth_state(P, seed=0):
    U = smoothed_explosion(P, 4.0, 2.0, 5.0, device="cpu").numpy().copy()
    rng = np.random.default_rng(seed)
    g = P.block_geometry[0]
    # a smooth velocity field so that every flux and limiter branch is exercised
    xc, yc = g.xc.ravel(), g.yc.ravel()
    U[1] += U[0] * 0.05 * np.sin(0.7 * xc + 0.3 * yc)
    U[2] += U[0] * 0.04 * np.cos(0.5 * xc - 0.6 * yc)
    U[3] += 0.5 * (U[1] ** 2 + U[2] ** 2) / U[0]
    U *= 1 + 1e-3 * rng.standard_normal(U.shape)
    return U


def _scheme(P, limiter, recon, sides=None):
    air = Air(a_inf=343.0, rho_inf=1.0)
    return Scheme(Geometry(P.block_geometry[0]), air.gamma(), air.gamma() - 1, limiter, recon, sides)


@pytest.mark.parametrize("limiter", ["Venkatakrishnan", "BarthJespersen", "VanAlbada", "VanLeer"])
@pytest.mark.parametrize("recon", ["ConservativeState", "PrimitiveState"])
def test_transcription_residual_equals_oracle(limiter, recon):
    P = adjoint_problem(n=24, limiter=limiter, recon=recon)
    U = _smooth_state(P)
    S = _scheme(P, limiter, recon)
    ny, nx = 24, 24
    got = S.residual(torch.tensor(U.reshape(4, ny, nx))).numpy().reshape(4, -1)
    want = Oracle(P).residual(U)
    assert np.array_equal(got, want)


def test_transcription_non_cartesian_and_side_kinds():
    """A skewed block (rotated face frames) with outlet and copy sides."""
    air = Air(a_inf=343.0, rho_inf=1.0)
    mesh = single_block_mesh(10.0)
    mesh[0]["NE"] = [11.0, 10.5]
    mesh[0]["SE"] = [10.0, 0.5]
    mesh[0]["BCTypeE"] = "OutletDirichlet"
    P = build_problem(mesh, 20, 16, flux="Roe", limiter="Venkatakrishnan", recon="ConservativeState",
                      gamma=air.gamma(), gm1=air.gamma() - 1, cfl=0.5, fluid=air)
    assert not P.block_geometry[0].is_cartesian
    U = _smooth_state(P)
    S = _scheme(P, "Venkatakrishnan", "ConservativeState",
                {"E": OUTLET, "W": REFLECT, "N": REFLECT, "S": REFLECT})
    got = S.residual(torch.tensor(U.reshape(4, 16, 20))).numpy().reshape(4, -1)
    assert np.array_equal(got, Oracle(P).residual(U))


def test_transcription_steps_equal_oracle():
    P = adjoint_problem(n=20)
    U = _smooth_state(P)
    a = tableau("RK4")
    S = _scheme(P, "Venkatakrishnan", "ConservativeState")
    O = Oracle(P)
    Ut = torch.tensor(U.reshape(4, 20, 20))
    Uo = U.copy()
    for dt in (1e-3, 2e-3, 1.5e-3):
        Ut = S.step(Ut, dt, a)
        Uo = O.step(Uo, a, dt)
    assert np.array_equal(Ut.numpy().reshape(4, -1), Uo)


def test_transcription_gradient_vs_central_differences():
    """dJ/d(r, w, cx) by autograd against central differences (h = 1e-6) on a 16 x 16
    block, 3 RK4 steps at a fixed dt."""
    P = adjoint_problem(n=16)
    S = _scheme(P, "Venkatakrishnan", "ConservativeState")
    a = tableau("RK4")
    dts = [2e-3] * 3

    def J(theta):
        U0 = smoothed_explosion(P, theta[0], theta[1], theta[2], device="cpu").reshape(4, 16, 16)
        return S.objective(U0, dts, a)

    theta = torch.tensor([4.0, 2.0, 5.0], dtype=torch.float64, requires_grad=True)
    J(theta).backward()
    g = theta.grad.numpy()
    h = 1e-6
    for k in range(3):
        tp, tm = theta.detach().clone(), theta.detach().clone()
        tp[k] += h
        tm[k] -= h
        fd = (J(tp).item() - J(tm).item()) / (2 * h)
        assert abs(fd - g[k]) <= 1e-6 * max(abs(g[k]), 1e-12 * abs(J(theta).item())), (k, fd, g[k])


def test_multiblock_transcription_equals_oracle():
    from oracle.torch_scheme import MultiBlockScheme
    from pyhype_gb300.mesh.rectangular import RectagularMeshGenerator

    air = Air(a_inf=343.0, rho_inf=1.0)
    mesh = RectagularMeshGenerator.generate(["Reflection"], ["OutletDirichlet"], ["Reflection"], ["Reflection"],
                                            east=10.0, west=0.0, north=10.0, south=0.0,
                                            n_blocks_horizontal=2, n_blocks_vertical=2).dict
    P = build_problem(mesh, 14, 12, flux="Roe", limiter="VanAlbada", recon="ConservativeState",
                      gamma=air.gamma(), gm1=air.gamma() - 1, cfl=0.5, fluid=air)
    per = []
    for g in P.block_geometry:
        rho = 1.0 + 0.2 * np.sin(0.6 * g.xc) * np.cos(0.4 * g.yc)
        u, v = 0.1 * np.cos(0.3 * g.xc + 0.2 * g.yc), 0.08 * np.sin(0.5 * g.yc - 0.1 * g.xc)
        p = 0.6 + 0.1 * np.cos(0.07 * g.xc * g.yc)
        per.append(np.stack([rho, rho * u, rho * v, p / (air.gamma() - 1) + 0.5 * rho * (u * u + v * v)], axis=-1))
    U = P.to_soa(per)
    M = MultiBlockScheme(P, air.gamma(), air.gamma() - 1, "VanAlbada")
    assert np.array_equal(M.residual(torch.tensor(U)).numpy(), Oracle(P).residual(U))


def _flow_state(P, mach, seed=0):
    """The smooth state with a uniform stream of the given Mach number (of the far-field
    sound speed, 1 non-dimensional) added in x: supersonic streams put the HLL fluxes'
    vertical faces on their upwind branches."""
    U = _smooth_state(P, seed)
    u = mach * np.sqrt(1.4 * (0.4 * (U[3] - 0.5 * (U[1] ** 2 + U[2] ** 2) / U[0])) / U[0])
    U[3] += 0.5 * U[0] * ((U[1] / U[0] + u) ** 2 - (U[1] / U[0]) ** 2)
    U[1] += U[0] * u
    return U


@pytest.mark.parametrize("flux", ["HLLL", "HLLE"])
@pytest.mark.parametrize("recon", ["ConservativeState", "PrimitiveState"])
@pytest.mark.parametrize("mach", [0.0, 2.5, -2.5])
def test_transcription_hll_residual_equals_oracle(flux, recon, mach):
    """HLLL and HLLE (subsonic, and supersonic streams either way, so that every branch
    of the flux is taken) value for value against the C oracle."""
    air = Air(a_inf=343.0, rho_inf=1.0)
    P = build_problem(single_block_mesh(10.0), 20, 18, flux=flux, limiter="Venkatakrishnan", recon=recon,
                      gamma=air.gamma(), gm1=air.gamma() - 1, cfl=0.5, fluid=air)
    U = _flow_state(P, mach)
    S = Scheme(Geometry(P.block_geometry[0]), air.gamma(), air.gamma() - 1, "Venkatakrishnan", recon, None, flux)
    got = S.residual(torch.tensor(U.reshape(4, 18, 20))).numpy().reshape(4, -1)
    assert np.array_equal(got, Oracle(P).residual(U))


@pytest.mark.parametrize("flux", ["HLLL", "HLLE"])
def test_transcription_hll_gradient_vs_central_differences(flux):
    """Autograd of the HLLL / HLLE residual against central differences, on a smooth
    state with a Mach 0.6 stream: lam . R(U + h d) for a random direction d.  The
    perturbation moves every cell, so above h ~ 1e-6 (relative) it crosses the
    limiter's min/max switches somewhere (the Roe residual behaves the same); at
    h = 1e-7 the quotient agrees to ~1e-8."""
    air = Air(a_inf=343.0, rho_inf=1.0)
    P = build_problem(single_block_mesh(10.0), 12, 10, flux=flux, limiter="VanAlbada", recon="ConservativeState",
                      gamma=air.gamma(), gm1=air.gamma() - 1, cfl=0.5, fluid=air)
    U = _flow_state(P, 0.6, seed=4).reshape(4, 10, 12)
    S = Scheme(Geometry(P.block_geometry[0]), air.gamma(), air.gamma() - 1, "VanAlbada", "ConservativeState", None,
               flux)
    rng = np.random.default_rng(5)
    lam = torch.tensor(rng.standard_normal(U.shape))
    d = torch.tensor(rng.standard_normal(U.shape)) * torch.tensor(np.abs(U))
    Ut = torch.tensor(U, requires_grad=True)
    (S.residual(Ut) * lam).sum().backward()
    ad = float((Ut.grad * d).sum())
    h = 1e-7
    Jp = float((S.residual(torch.tensor(U) + h * d) * lam).sum())
    Jm = float((S.residual(torch.tensor(U) - h * d) * lam).sum())
    fd = (Jp - Jm) / (2 * h)
    assert abs(fd - ad) <= 1e-6 * abs(ad), (fd, ad)
