"""The FP32 form (FP32 state, geometry and flux arithmetic; Kahan-compensated step
accumulation; FP64 dt reduction) against the FP64 path on the same problems.

Stated results, not bit-exactness: the L1 density difference relative to the FP64
path stays below the bound written for each case.  The bounds differ by case because
the reference's limiter is discontinuous at round-off level (psi = 0.75 when a face
difference davg is exactly zero, ~1 when it is one ulp): on initial conditions with
uniform regions any change of operation order flips it in places.  The FP64 code
itself, compiled with fused multiply-add, already differs from the reference by
2.5e-5 after one step and 7e-5 after 100 steps of the 100x100 explosion
(tests/test_reference_sensitivity.py)."""
import numpy as np
import pytest

import _golden as G

pytestmark = pytest.mark.gpu


def _pair(z, tableau=None):
    from pyhype_gb300._native import DeviceSolver

    P64 = G.problem(z, precision=0)
    P32 = G.problem(z, precision=1)
    a = z["tableau"] if tableau is None else tableau
    return P64, DeviceSolver(P64, tableau=a), DeviceSolver(P32, tableau=a)


def _l1_rel(a, b):
    return float(np.sum(np.abs(a - b)) / np.sum(np.abs(b)))


@pytest.mark.parametrize("name,steps,bound", [("p100", 100, 1e-3), ("m2x4_40", 12, 3e-4), ("dmr5", 8, 1e-5),
                                              ("hlll_prim", 5, 1e-4), ("lim_vl", 5, 1e-5)])
def test_fp32_density_l1_vs_fp64(name, steps, bound):
    z = G.load(name)
    P, S64, S32 = _pair(z)
    U0 = P.to_soa(list(z["ic"]))
    S64.set_state(U0)
    S32.set_state(U0)
    tf = G.t_final(z)
    t64, n64 = S64.run(0.0, tf, max_steps=steps)
    t32, n32 = S32.run(0.0, tf, max_steps=steps)
    assert n64 == n32 == steps
    assert abs(t32 - t64) <= 2 * bound * t64  # CFL dt of states that differ by the same order
    U64, U32 = S64.get_state(), S32.get_state()
    err = _l1_rel(U32[0], U64[0])
    assert err < bound, f"L1 density error {err:.3e}"
    assert S32.check_realizable().ok == 1


def _seeded_problem(nx, ny, bx, by, flux="Roe", recon="ConservativeState", limiter="Venkatakrishnan"):
    """Reflecting multiblock square, smooth waves with seeded cell noise on every
    variable: no region is uniform, so the reference limiter's round-off switch
    (psi = 0.75 exactly at davg == 0) plays no part and the FP32 form's own rounding
    error shows."""
    from pyhype_gb300.fluids import Air
    from pyhype_gb300.mesh import RectagularMeshGenerator
    from pyhype_gb300.problem import build_problem
    from pyhype_gb300.states import ConservativeState, PrimitiveState

    air = Air(a_inf=343.0, rho_inf=1.0)
    mesh = RectagularMeshGenerator.generate(["Reflection"], ["Reflection"], ["Reflection"], ["Reflection"],
                                            10.0, 0.0, 10.0, 0.0, bx, by)
    P = build_problem(mesh.dict, nx, ny, flux=flux, limiter=limiter, recon=recon, gamma=air.gamma(),
                      gm1=air.gamma() - 1, cfl=0.8, fluid=air)
    rng = np.random.default_rng(nx * 31 + ny)
    blocks = []
    for g in P.block_geometry:
        x, y, n = g.xc, g.yc, g.xc.shape
        W = np.stack([1.2 * (1 + 0.3 * np.sin(0.9 * x) * np.cos(0.7 * y)) * (1 + rng.uniform(-0.02, 0.02, n)),
                      60.0 * np.sin(0.5 * y + 0.3 * x) + rng.uniform(-3.4, 3.4, n),
                      40.0 * np.cos(0.6 * x) + rng.uniform(-3.4, 3.4, n),
                      101100.0 * (1 + 0.2 * np.cos(0.8 * x + 0.4 * y)) * (1 + rng.uniform(-0.02, 0.02, n))], axis=-1)
        s = PrimitiveState(air, array=W).to_type(ConservativeState)
        s.make_non_dimensional()
        blocks.append(s.data)
    return P, P.to_soa(blocks)


@pytest.mark.parametrize("flux,recon", [("Roe", "ConservativeState"), ("HLLL", "PrimitiveState")])
def test_fp32_seeded_state_l1_vs_fp64(flux, recon):
    """On a state without uniform regions the FP32 form stays within 2e-6 (L1 density,
    relative) of the FP64 path over 20 RK4 steps of a 2 x 2 x 96^2 problem, and its
    conserved totals within 1e-6."""
    from pyhype_gb300._native import DeviceSolver
    from pyhype_gb300.time_marching import tableau

    P, U0 = _seeded_problem(96, 96, 2, 2, flux, recon)
    out, tot = [], []
    for prec in (0, 1):
        S = DeviceSolver(P.with_precision(prec), tableau=tableau("RK4"))
        S.set_state(U0)
        t, n = S.run(0.0, 1e30, max_steps=20)
        assert n == 20
        out.append(S.get_state())
        tot.append(S.totals()[0])
        S.close()
    err = _l1_rel(out[1][0], out[0][0])
    print(f"{flux}/{recon}: FP32 L1 density {err:.2e}, totals {np.abs(tot[1] - tot[0]) / np.abs(tot[0])}")
    assert err < 2e-6, err
    assert abs(tot[1][0] - tot[0][0]) <= 1e-6 * abs(tot[0][0])
    assert abs(tot[1][3] - tot[0][3]) <= 1e-6 * abs(tot[0][3])


def test_fp32_residual_close_to_fp64():
    z = G.load("ops_explosion_cons")
    P, S64, S32 = _pair(z)
    U = P.to_soa(list(z["ops_state"]))
    S64.set_state(U)
    S32.set_state(U)
    d64 = S64.residual()
    d32 = S32.residual()
    scale = np.max(np.abs(d64), axis=1, keepdims=True)
    assert np.max(np.abs(d32 - d64) / scale) < 1e-3


def _floats(rng, n, emin, emax):
    """Random float32 values with random sign, exponent uniform in [emin, emax] and
    random mantissa bits."""
    e = rng.integers(emin, emax + 1, n, dtype=np.int64)
    m = rng.integers(0, 1 << 23, n, dtype=np.int64)
    s = rng.integers(0, 2, n, dtype=np.int64) << 31
    return ((s | ((e + 127) << 23) | m).astype(np.uint32)).view(np.float32)


def test_div32_matches_ieee_division():
    """The FP32 form's division (reciprocal seed, one Newton step, residual correction;
    IEEE division outside |a|, |b| in 2^-60..2^61) against numpy's IEEE float32
    division: the same value for every sampled pair, zero quotients up to sign."""
    import ctypes

    import torch

    from pyhype_gb300 import _native

    L = _native.load()
    L.e2d_check_div32.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64]
    rng = np.random.default_rng(7)
    n = 1 << 21
    cases = {
        "fast path": (_floats(rng, n, -60, 60), _floats(rng, n, -60, 60)),
        "fast path, small divisors": (_floats(rng, n, -60, 60), _floats(rng, n, -60, -40)),
        "fallback operands": (_floats(rng, n, -126, 127), _floats(rng, n, -126, 127)),
        "zero numerators": (np.where(rng.random(n) < 0.3, np.float32(0), _floats(rng, n, -30, 30)).astype(np.float32),
                            _floats(rng, n, -30, 30)),
    }
    for name, (a, b) in cases.items():
        ad, bd = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
        qd = torch.empty_like(ad)
        assert L.e2d_check_div32(ad.data_ptr(), bd.data_ptr(), qd.data_ptr(), n) == 0
        q = qd.cpu().numpy()
        with np.errstate(all="ignore"):
            ref = a / b
        same = (q.view(np.uint32) == ref.view(np.uint32)) | ((q == 0) & (ref == 0)) | (np.isnan(q) & np.isnan(ref))
        assert same.all(), f"{name}: {int((~same).sum())} of {n} differ, e.g. {a[~same][:3]} / {b[~same][:3]}"


def test_rdiv_matches_ieee_division_inside_its_range():
    """rdiv (div32's sequence without the range test, for the state algebra's divisors)
    equals IEEE float32 division for operands within 2^-60..2^61 and zero numerators."""
    import ctypes

    import torch

    from pyhype_gb300 import _native

    L = _native.load()
    L.e2d_check_rdiv32.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64]
    rng = np.random.default_rng(8)
    n = 1 << 21
    cases = {
        "inside the range": (_floats(rng, n, -60, 60), _floats(rng, n, -60, 60)),
        "densities and pressures": (_floats(rng, n, -12, 12), np.abs(_floats(rng, n, -12, 12))),
        "zero numerators": (np.where(rng.random(n) < 0.3, np.float32(0), _floats(rng, n, -30, 30)).astype(np.float32),
                            _floats(rng, n, -30, 30)),
    }
    for name, (a, b) in cases.items():
        ad, bd = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
        qd = torch.empty_like(ad)
        assert L.e2d_check_rdiv32(ad.data_ptr(), bd.data_ptr(), qd.data_ptr(), n) == 0
        q = qd.cpu().numpy()
        ref = a / b
        same = (q.view(np.uint32) == ref.view(np.uint32)) | ((q == 0) & (ref == 0))
        assert same.all(), f"{name}: {int((~same).sum())} of {n} differ, e.g. {a[~same][:3]} / {b[~same][:3]}"


@pytest.mark.parametrize("limiter", [0, 2])  # Venkatakrishnan, van Albada
def test_paired_limiter_functions_equal_scalar(limiter):
    """The paired evaluation of min(psi(s_a), psi(s_b)) gives the two scalar
    evaluations' value bit for bit: slopes at 0, 1 (psi_s's exact value), the peaks,
    the cap and beyond, subnormal and random values."""
    import ctypes

    import torch

    from pyhype_gb300 import _native

    L = _native.load()
    L.e2d_check_psi_pair.argtypes = [ctypes.c_int32] + [ctypes.c_void_p] * 4 + [ctypes.c_int64]
    rng = np.random.default_rng(9 + limiter)
    special = np.array([0.0, 1e-45, 1e-30, 0.5, 1.0, 2.0, 1 + 2 ** 0.5, 2 + 2 * 2 ** 0.5, 10.0, 1e8, 1e15, 1e20,
                        np.inf], dtype=np.float32)
    n = 1 << 20
    sa = np.concatenate([np.repeat(special, special.size), np.abs(_floats(rng, n, -30, 30))]).astype(np.float32)
    sb = np.concatenate([np.tile(special, special.size), np.abs(_floats(rng, n, -30, 30))]).astype(np.float32)
    a, b = torch.from_numpy(sa).cuda(), torch.from_numpy(sb).cuda()
    p, q = torch.empty_like(a), torch.empty_like(a)
    assert L.e2d_check_psi_pair(limiter, a.data_ptr(), b.data_ptr(), p.data_ptr(), q.data_ptr(), sa.size) == 0
    pv, qv = p.cpu().numpy(), q.cpu().numpy()
    same = pv.view(np.uint32) == qv.view(np.uint32)
    assert same.all(), f"{int((~same).sum())} differ, e.g. s = {sa[~same][:3]}, {sb[~same][:3]}"

