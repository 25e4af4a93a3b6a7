"""Conserved totals (FP64 sums of A * U per instance, e2d_totals) and the conservation
drift of the FP64 path and the FP32 form.

The totals are checked against exactly rounded host sums (math.fsum) of the same
products.  On a single block with reflecting walls the scheme conserves mass and
energy exactly up to rounding (the wall faces carry no mass or energy flux, every
interior face flux enters its two cells with opposite signs), so the drift over a
run measures the arithmetic alone.  Multiblock problems do not conserve: the
reference's inter-block faces take the neighbour's cell average on one side, so the
two blocks' fluxes through a shared face differ."""
import math

import numpy as np
import pytest

import _golden as G

pytestmark = pytest.mark.gpu


def _host_totals(P, U, fp32=False):
    """Exactly rounded sums of A * U_v per instance (values rounded to FP32 first for
    the FP32 form, whose state and areas are FP32)."""
    ninst = max(1, int(P.cfg.ninstances))
    terms = [[[] for _ in range(4)] for _ in range(ninst)]
    for b, arr in enumerate(P.from_soa(U)):
        A = np.asarray(P.block_geometry[b].A, dtype=np.float64)
        if fp32:
            A = A.astype(np.float32).astype(np.float64)
            arr = arr.astype(np.float32).astype(np.float64)
        q = int(P.blocks[b].instance)
        for v in range(4):
            terms[q][v].extend((A * arr[:, :, v]).ravel().tolist())
    return np.array([[math.fsum(terms[q][v]) for v in range(4)] for q in range(ninst)]), \
        np.array([[math.fsum(abs(x) for x in terms[q][v]) for v in range(4)] for q in range(ninst)])


@pytest.mark.parametrize("name,precision", [("p100", 0), ("m2x4_40", 0), ("dmr5", 0), ("m2x4_40", 1)])
def test_totals_are_the_exact_sums(name, precision):
    from pyhype_gb300._native import DeviceSolver

    z = G.load(name)
    P = G.problem(z, precision=precision)
    S = DeviceSolver(P, tableau=z["tableau"])
    U = P.to_soa(list(z["ic"]))
    S.set_state(U)
    got = S.totals()
    ref, mag = _host_totals(P, U, fp32=precision == 1)
    assert got.shape == ref.shape
    assert np.all(np.abs(got - ref) <= 1e-14 * mag), (got, ref)
    # reproducible: the same state gives the same bits
    assert np.array_equal(S.totals(), got)


def _drift(S, P, U0, tableau, steps):
    S.set_state(U0)
    T0 = S.totals()
    t, n = S.run(0.0, float("inf"), max_steps=steps)
    assert n == steps
    T1 = S.totals()
    with np.errstate(divide="ignore", invalid="ignore"):  # momentum totals may be 0
        return (T1 - T0) / np.abs(T0)


def test_reflecting_single_block_conserves_mass_and_energy():
    """100x100 explosion, Reflection on every side, RK4, 100 steps: relative drift of
    total mass and energy, FP64 path and FP32 form (Kahan-compensated steps)."""
    from pyhype_gb300._native import DeviceSolver

    z = G.load("p100")
    U0 = G.problem(z).to_soa(list(z["ic"]))
    out = {}
    for prec in (0, 1):
        P = G.problem(z, precision=prec)
        S = DeviceSolver(P, tableau=z["tableau"])
        d = _drift(S, P, U0, z["tableau"], 100)[0]
        out[prec] = (d[0], d[3])
        S.close()
    print(f"drift after 100 steps: FP64 mass {out[0][0]:.2e} energy {out[0][1]:.2e}; "
          f"FP32 mass {out[1][0]:.2e} energy {out[1][1]:.2e}")
    assert abs(out[0][0]) <= 1e-13 and abs(out[0][1]) <= 1e-13
    assert abs(out[1][0]) <= 1e-8 and abs(out[1][1]) <= 1e-8


def test_fp32_totals_track_fp64_on_multiblock():
    """2x4 blocks of 40^2 (not conservative across blocks): after 12 steps the FP32
    form's totals stay within 1e-6 of the FP64 path's."""
    from pyhype_gb300._native import DeviceSolver

    z = G.load("m2x4_40")
    U0 = G.problem(z).to_soa(list(z["ic"]))
    tots = []
    for prec in (0, 1):
        P = G.problem(z, precision=prec)
        S = DeviceSolver(P, tableau=z["tableau"])
        S.set_state(U0)
        S.run(0.0, float("inf"), max_steps=12)
        tots.append(S.totals()[0])
        S.close()
    rel = np.abs(tots[1] - tots[0]) / np.abs(tots[0])
    print("FP32 vs FP64 totals after 12 steps (mass, x-mom, y-mom, energy):", rel)
    assert rel[0] <= 1e-6 and rel[3] <= 1e-6
