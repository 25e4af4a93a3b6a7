"""HLLE on the GPU against the oracle, value for value.

The reference's FluxHLLE cannot be constructed (pyhype/flux/HLLE.py:25 passes the
solver config where the fluid belongs), so its recorded runs do not exist; the
fixtures' meshes, boundary conditions and initial states are reused with the flux
switched to HLLE and compared with the oracle's HLLE (its properties are pinned in
tests/test_hlle_oracle.py).  Covers the one-point flux kernel with its per-operator
outputs, the multi-point quadrature kernel, both reconstruction types, skewed blocks
and the supersonic double-Mach setup, where the upwind branches are taken."""
import numpy as np
import pytest

import _golden as G
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu


def _solver(z, **kw):
    from pyhype_gb300._native import DeviceSolver

    P = G.problem(z, flux="HLLE", **kw)
    return P, DeviceSolver(P, tableau=z["tableau"])


@pytest.mark.parametrize("name,recon", [("m2x4_40", None), ("m2x4_40", "PrimitiveState"), ("dmr5", None),
                                        ("wedge", None), ("hlll_cons", None), ("bc_mixed", "PrimitiveState")])
def test_hlle_residual_intermediates_vs_oracle(name, recon):
    z = G.load(name)
    P, S = _solver(z, recon=recon)
    U = P.to_soa(list(z["ops_state"]))
    S.set_state(U)
    t = float(z["ops_t"]) if "ops_t" in z.files else 0.0
    dudt, dbg = S.residual(debug=True, t=t)
    ref, rdbg = Oracle(P).residual(U, t=t, debug=True)
    for key in ("vL", "vR", "hL", "hR", "vflux_raw", "hflux_raw", "vflux", "hflux"):
        assert np.array_equal(dbg[key], rdbg[key]), f"{key}: max diff {np.max(np.abs(dbg[key] - rdbg[key]))}"
    assert np.array_equal(dudt, ref), f"dUdt: max diff {np.max(np.abs(dudt - ref))}"


@pytest.mark.parametrize("name,steps", [("p100", 10), ("m2x4_40", 6), ("dmr5", 8), ("wedge", 6), ("qp2_roe", 4),
                                        ("qp3_hlll_prim", 3), ("jet", 4)])
def test_hlle_steps_vs_oracle(name, steps):
    z = G.load(name)
    P, S = _solver(z)
    U = P.to_soa(list(z["ic"]))
    S.set_state(U)
    O = Oracle(P)
    a = z["tableau"]
    t = 0.0
    for step in range(1, steps + 1):
        dt = float(S.compute_dt()[0])
        assert dt == float(O.dt(U)[0]), f"step {step}: dt"
        S.step(dt, t)
        U = O.step(U, a, dt, t)
        t += dt
        G_ = S.get_state()
        assert np.array_equal(G_, U), f"step {step}: max diff {np.max(np.abs(G_ - U))}"


def test_hlle_device_loop_vs_oracle():
    """The graph-replayed device loop with HLLE reproduces the oracle's run."""
    z = G.load("dmr5")
    P, S = _solver(z)
    U0 = P.to_soa(list(z["ic"]))
    S.set_state(U0)
    tf = G.t_final(z)
    t, steps = S.run(0.0, tf, max_steps=8)
    Ut, t_or, dts = Oracle(P).run(U0, z["tableau"], 0.0, tf, 8)
    assert steps == len(dts) and t == t_or
    assert np.array_equal(S.get_state(), Ut)
