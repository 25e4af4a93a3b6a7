"""Hand-written reverse kernels (e2d_residual_vjp, e2d_adjoint_forward/backward) against
torch autograd through the FP64 PyTorch transcription of the scheme
(oracle/torch_scheme.py) and against central finite differences."""
import numpy as np
import pytest
import torch

from oracle.torch_scheme import OUTLET, REFLECT, Geometry, Scheme
from pyhype_gb300.fluids import Air

pytestmark = pytest.mark.gpu

AIR = Air(a_inf=343.0, rho_inf=1.0)


def _smooth_state(P, seed=0):
    from pyhype_gb300.adjoint import smoothed_explosion

    U = smoothed_explosion(P, 4.0, 2.0, 5.0, device="cpu").numpy().copy()
    g = P.block_geometry[0]
    xc, yc = g.xc.ravel(), g.yc.ravel()
    U[1] += U[0] * 0.05 * np.sin(0.7 * xc + 0.3 * yc)
    U[2] += U[0] * 0.04 * np.cos(0.5 * xc - 0.6 * yc)
    U[3] += 0.5 * (U[1] ** 2 + U[2] ** 2) / U[0]
    U *= 1 + 1e-3 * np.random.default_rng(seed).standard_normal(U.shape)
    return U


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


@pytest.mark.parametrize("limiter", ["Venkatakrishnan", "BarthJespersen", "VanAlbada", "VanLeer"])
@pytest.mark.parametrize("recon", ["ConservativeState", "PrimitiveState"])
def test_residual_vjp_matches_autograd(limiter, recon):
    from pyhype_gb300._native import DeviceSolver
    from pyhype_gb300.adjoint import adjoint_problem
    from pyhype_gb300.time_marching import tableau

    n = 40
    P = adjoint_problem(n=n, limiter=limiter, recon=recon)
    U = _smooth_state(P)
    lam = np.random.default_rng(1).standard_normal(U.shape)
    S = Scheme(Geometry(P.block_geometry[0]), AIR.gamma(), AIR.gamma() - 1, limiter, recon)
    Ut = torch.tensor(U.reshape(4, n, n), requires_grad=True)
    R = S.residual(Ut)
    (R * torch.tensor(lam.reshape(4, n, n))).sum().backward()
    want = Ut.grad.numpy().reshape(4, -1)
    D = DeviceSolver(P, tableau=tableau("RK4"))
    D.set_state(U)
    assert np.array_equal(D.residual(), R.detach().numpy().reshape(4, -1))  # same forward values
    got = D.residual_vjp(torch.tensor(lam, device="cuda")).cpu().numpy()
    assert _rel(got, want) < 1e-11, _rel(got, want)


@pytest.mark.parametrize("flux", ["HLLL", "HLLE"])
@pytest.mark.parametrize("recon", ["ConservativeState", "PrimitiveState"])
@pytest.mark.parametrize("mach", [0.0, 2.5, -2.5])
def test_residual_vjp_hll_matches_autograd(flux, recon, mach):
    """The HLLL and HLLE reverse kernels against autograd of the transcription, on a
    smooth state at rest and with supersonic streams either way (every branch of the
    flux taken somewhere)."""
    from test_torch_scheme import _flow_state

    from pyhype_gb300._native import DeviceSolver
    from pyhype_gb300.adjoint import adjoint_problem
    from pyhype_gb300.time_marching import tableau

    n = 40
    P = adjoint_problem(n=n, limiter="Venkatakrishnan", recon=recon, flux=flux)
    U = _flow_state(P, mach)
    lam = np.random.default_rng(1).standard_normal(U.shape)
    S = Scheme(Geometry(P.block_geometry[0]), AIR.gamma(), AIR.gamma() - 1, "Venkatakrishnan", recon, None, flux)
    Ut = torch.tensor(U.reshape(4, n, n), requires_grad=True)
    R = S.residual(Ut)
    (R * torch.tensor(lam.reshape(4, n, n))).sum().backward()
    want = Ut.grad.numpy().reshape(4, -1)
    D = DeviceSolver(P, tableau=tableau("RK4"))
    D.set_state(U)
    assert np.array_equal(D.residual(), R.detach().numpy().reshape(4, -1))  # same forward values
    got = D.residual_vjp(torch.tensor(lam, device="cuda")).cpu().numpy()
    assert _rel(got, want) < 1e-11, _rel(got, want)


def test_time_loop_gradient_hlll_matches_autograd():
    """dJ/dU0 over 10 SSP-RK2 steps with HLLL and primitive reconstruction (the
    double-Mach scheme), checkpoints every 4, against autograd of the transcription."""
    from test_torch_scheme import _flow_state

    from pyhype_gb300.adjoint import AdjointSolver, adjoint_problem
    from pyhype_gb300.time_marching import tableau

    n = 32
    P = adjoint_problem(n=n, recon="PrimitiveState", flux="HLLL")
    U0 = torch.tensor(_flow_state(P, 0.8, seed=2))
    A = AdjointSolver(P, "SSPRK2", side="N", nsteps=10, ckpt_every=4)
    J = A.forward(U0.cuda())
    g = A.backward().cpu().numpy()
    S = Scheme(Geometry(P.block_geometry[0]), AIR.gamma(), AIR.gamma() - 1, "Venkatakrishnan", "PrimitiveState",
               None, "HLLL")
    Ut = U0.clone().reshape(4, n, n).requires_grad_(True)
    Jt = S.objective(Ut, A.dts, tableau("SSPRK2"), side="N")
    Jt.backward()
    assert abs(J - Jt.item()) <= 1e-13 * abs(J)
    want = Ut.grad.numpy().reshape(4, -1)
    assert _rel(g, want) < 1e-10, _rel(g, want)


@pytest.mark.parametrize("nx,ny", [(1, 12), (14, 1)])
def test_residual_vjp_thin_block(nx, ny):
    """A one-cell-wide (or -high) block: both ghost images of a side pair fall on the
    same cells."""
    from pyhype_gb300._native import DeviceSolver
    from pyhype_gb300.adjoint import single_block_mesh
    from pyhype_gb300.problem import build_problem
    from pyhype_gb300.time_marching import tableau

    mesh = single_block_mesh(10.0)
    mesh[0]["BCTypeE"] = "OutletDirichlet"
    P = build_problem(mesh, nx, ny, flux="HLLL", limiter="Venkatakrishnan", recon="ConservativeState",
                      gamma=AIR.gamma(), gm1=AIR.gamma() - 1, cfl=0.5, fluid=AIR)
    g = P.block_geometry[0]
    rho = 1.0 + 0.2 * np.sin(0.6 * g.xc + 0.5 * g.yc)
    u, v = 0.3 * np.cos(0.3 * g.yc), 0.2 * np.sin(0.4 * g.xc)
    p = 0.7 + 0.1 * np.cos(0.5 * g.xc - 0.3 * g.yc)
    U = P.to_soa([np.stack([rho, rho * u, rho * v, p / 0.4 + 0.5 * rho * (u * u + v * v)], axis=-1)])
    lam = np.random.default_rng(4).standard_normal(U.shape)
    S = Scheme(Geometry(g), AIR.gamma(), AIR.gamma() - 1, "Venkatakrishnan", "ConservativeState",
               {"E": OUTLET, "W": REFLECT, "N": REFLECT, "S": REFLECT}, "HLLL")
    Ut = torch.tensor(U.reshape(4, ny, nx), requires_grad=True)
    R = S.residual(Ut)
    (R * torch.tensor(lam.reshape(4, ny, nx))).sum().backward()
    D = DeviceSolver(P, tableau=tableau("RK4"))
    D.set_state(U)
    assert np.array_equal(D.residual(), R.detach().numpy().reshape(4, -1))
    got = D.residual_vjp(torch.tensor(lam, device="cuda")).cpu().numpy()
    assert _rel(got, Ut.grad.numpy().reshape(4, -1)) < 1e-11


def test_residual_vjp_non_cartesian_outlet():
    from pyhype_gb300._native import DeviceSolver
    from pyhype_gb300.adjoint import single_block_mesh
    from pyhype_gb300.problem import build_problem
    from pyhype_gb300.time_marching import tableau

    mesh = single_block_mesh(10.0)
    mesh[0]["NE"] = [11.0, 10.5]
    mesh[0]["SE"] = [10.0, 0.5]
    mesh[0]["BCTypeE"] = "OutletDirichlet"
    P = build_problem(mesh, 36, 28, flux="Roe", limiter="Venkatakrishnan", recon="ConservativeState",
                      gamma=AIR.gamma(), gm1=AIR.gamma() - 1, cfl=0.5, fluid=AIR)
    U = _smooth_state(P)
    lam = np.random.default_rng(2).standard_normal(U.shape)
    S = Scheme(Geometry(P.block_geometry[0]), AIR.gamma(), AIR.gamma() - 1,
               sides={"E": OUTLET, "W": REFLECT, "N": REFLECT, "S": REFLECT})
    Ut = torch.tensor(U.reshape(4, 28, 36), requires_grad=True)
    (S.residual(Ut) * torch.tensor(lam.reshape(4, 28, 36))).sum().backward()
    D = DeviceSolver(P, tableau=tableau("RK4"))
    D.set_state(U)
    got = D.residual_vjp(torch.tensor(lam, device="cuda")).cpu().numpy()
    assert _rel(got, Ut.grad.numpy().reshape(4, -1)) < 1e-11


def test_residual_vjp_multiblock_matches_autograd():
    """2 x 2 blocks with inter-block halos and an outlet side, against autograd of the
    multiblock transcription."""
    from oracle.torch_scheme import MultiBlockScheme
    from pyhype_gb300._native import DeviceSolver
    from pyhype_gb300.mesh.rectangular import RectagularMeshGenerator
    from pyhype_gb300.problem import build_problem
    from pyhype_gb300.time_marching import tableau

    mesh = RectagularMeshGenerator.generate(["Reflection"], ["OutletDirichlet"], ["Reflection"], ["Reflection"],
                                            east=10.0, west=0.0, north=10.0, south=0.0,
                                            n_blocks_horizontal=2, n_blocks_vertical=2).dict
    P = build_problem(mesh, 24, 20, flux="Roe", limiter="VanAlbada", recon="ConservativeState",
                      gamma=AIR.gamma(), gm1=AIR.gamma() - 1, cfl=0.5, fluid=AIR)
    per = []
    for g in P.block_geometry:
        rho = 1.0 + 0.2 * np.sin(0.6 * g.xc) * np.cos(0.4 * g.yc)
        u = 0.1 * np.cos(0.3 * g.xc + 0.2 * g.yc)
        v = 0.08 * np.sin(0.5 * g.yc - 0.1 * g.xc)
        p = 0.6 + 0.1 * np.cos(0.07 * g.xc * g.yc)
        E = p / (AIR.gamma() - 1) + 0.5 * rho * (u * u + v * v)
        per.append(np.stack([rho, rho * u, rho * v, E], axis=-1))
    U = P.to_soa(per)
    lam = np.random.default_rng(3).standard_normal(U.shape)
    M = MultiBlockScheme(P, AIR.gamma(), AIR.gamma() - 1, "VanAlbada")
    Ut = torch.tensor(U, requires_grad=True)
    R = M.residual(Ut)
    (R * torch.tensor(lam)).sum().backward()
    D = DeviceSolver(P, tableau=tableau("RK4"))
    D.set_state(U)
    assert np.array_equal(D.residual(), R.detach().numpy())
    got = D.residual_vjp(torch.tensor(lam, device="cuda")).cpu().numpy()
    assert _rel(got, Ut.grad.numpy()) < 1e-11, _rel(got, Ut.grad.numpy())


def test_time_loop_gradient_matches_autograd():
    """dJ/dU0 over 12 RK4 steps (checkpoints every 5: three segments) of a 64 x 64
    copy of the adjoint configuration, against torch autograd of the transcription at
    the same dt schedule."""
    from pyhype_gb300.adjoint import AdjointSolver, adjoint_problem, smoothed_explosion
    from pyhype_gb300.time_marching import tableau

    n = 64
    P = adjoint_problem(n=n)
    U0 = smoothed_explosion(P, 4.0, 2.0, 5.0, device="cpu")
    A = AdjointSolver(P, "RK4", side="N", nsteps=12, ckpt_every=5)
    J = A.forward(U0.cuda())
    g = A.backward().cpu().numpy()
    S = Scheme(Geometry(P.block_geometry[0]), AIR.gamma(), AIR.gamma() - 1)
    Ut = U0.clone().reshape(4, n, n).requires_grad_(True)
    Jt = S.objective(Ut, A.dts, tableau("RK4"), side="N")
    Jt.backward()
    assert abs(J - Jt.item()) <= 1e-13 * abs(J)
    want = Ut.grad.numpy().reshape(4, -1)
    assert _rel(g, want) < 1e-10, _rel(g, want)
    # replaying the recorded dt schedule from U0 repeats the forward pass exactly
    assert A.forward(U0.cuda(), A.dts.copy()) == J


@pytest.mark.parametrize("cx", [5.0, 5.3])
def test_ic_parameter_gradient_vs_central_differences(cx):
    """dJ/d(r, w, cx) through autograd of the IC and the reverse kernels, against
    central differences (h = 1e-6) of J at the frozen dt schedule, 64 x 64, 40 steps.
    At cx = 5 the problem is mirror-symmetric, dJ/dcx = 0, and the differences see a
    kink where the mirrored stencil values tie (the max/min subgradient takes the first
    of equal operands): only r and w are compared there."""
    from pyhype_gb300.adjoint import AdjointSolver, adjoint_problem, smoothed_explosion

    P = adjoint_problem(n=64)
    A = AdjointSolver(P, "RK4", side="N", nsteps=40, ckpt_every=20)
    theta = torch.tensor([4.0, 2.0, cx], dtype=torch.float64, device="cuda", requires_grad=True)
    J = A.objective(smoothed_explosion(P, theta[0], theta[1], theta[2]))
    J.backward()
    grad = theta.grad.cpu().numpy()
    dts = A.dts.copy()
    h = 1e-6
    for k in range(3 if cx != 5.0 else 2):
        tp = theta.detach().clone()
        tm = theta.detach().clone()
        tp[k] += h
        tm[k] -= h
        Jp = A.forward(smoothed_explosion(P, tp[0], tp[1], tp[2]), dts)
        Jm = A.forward(smoothed_explosion(P, tm[0], tm[1], tm[2]), dts)
        fd = (Jp - Jm) / (2 * h)
        print(f"cx {cx} param {k}: adjoint {grad[k]:.12e} fd {fd:.12e} rel {abs(fd - grad[k]) / abs(grad[k]):.2e}")
        # 1e-6 relative, plus the round-off of the difference quotient (J to ~1e-15)
        assert abs(fd - grad[k]) <= 1e-6 * abs(grad[k]) + 1e-15 * abs(J.item()) / h


def test_fp32_adjoint_close_to_fp64():
    """The FP32 form's reverse pass (FP32 state, face states and reverse kernels) at the
    FP64 pass's dt schedule.  Single Jacobian rows of a smooth state agree with FP64 to
    ~1e-5; dJ/dU0 as a whole does not, because the two maps differ where the state is
    uniform to round-off (the FP64 map resolves 1e-12-level differences of the tanh
    tails that the FP32 state rounds to exact uniformity, and the limiter's slope is
    very sensitive there).  The derivatives along smooth IC directions, dJ/d(r, w, cx),
    are stated against the FP64 ones."""
    from pyhype_gb300.adjoint import AdjointSolver, adjoint_problem, smoothed_explosion

    P = adjoint_problem(n=64)
    grads, Js = {}, {}
    dts = None
    for prec in ("fp64", "fp32"):
        A = AdjointSolver(P, "RK4", side="N", nsteps=40, ckpt_every=10, precision=prec)
        theta = torch.tensor([4.0, 2.0, 5.3], dtype=torch.float64, device="cuda", requires_grad=True)
        J = A.objective(smoothed_explosion(P, theta[0], theta[1], theta[2]), dts)
        J.backward()
        dts = A.dts.copy() if dts is None else dts
        grads[prec], Js[prec] = theta.grad.cpu().numpy(), J.item()
    rel_J = abs(Js["fp32"] - Js["fp64"]) / abs(Js["fp64"])
    rel = np.abs(grads["fp32"] - grads["fp64"]) / np.abs(grads["fp64"])
    print(f"FP32 adjoint: J rel {rel_J:.2e}; dJ/d(r, w, cx) fp64 {grads['fp64']} fp32 {grads['fp32']} rel {rel}")
    assert rel_J < 1e-5
    assert rel[0] < 1e-3 and rel[1] < 1e-3


@pytest.mark.parametrize("flux", ["Roe", "HLLL"])
def test_fp32_adjoint_fused_recompute_equals_split(flux):
    """The FP32 form's reverse pass recomputes each checkpoint segment with the fused
    stage kernel, which records the stage inputs and face states the reverse kernels
    read; with the three split kernels (stage form 0) instead, J and dJ/dU0 are the
    same bits."""
    from pyhype_gb300.adjoint import AdjointSolver, adjoint_problem, smoothed_explosion

    P = adjoint_problem(n=64, flux=flux)
    out = []
    for form in (2, 0):
        A = AdjointSolver(P, "RK4", side="N", nsteps=12, ckpt_every=5, precision="fp32")
        A.device.set_kernel_choice(3, form)
        U0 = smoothed_explosion(P, 4.0, 2.0, 5.3).detach().clone()
        J = A.forward(U0)
        g = A.backward().cpu().numpy()
        out.append((J, g))
    assert out[0][0] == out[1][0]
    assert np.array_equal(out[0][1], out[1][1])
