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
