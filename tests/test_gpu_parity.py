"""CUDA path (through the C ABI) against the CPU oracle and the reference fixtures.

The bar is value equality (bit-exact up to the sign of zero) for every per-operator
intermediate, the dt of every step and the state after every step."""
import numpy as np
import pytest

import _golden as G
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

CASES = G.cases()
OPS_CASES = [c for c in CASES if "ops_state" in G.load(c).files]


def _solver(z):
    from pyhype_gb300._native import DeviceSolver

    P = G.problem(z)
    return P, DeviceSolver(P, tableau=z["tableau"])


def _eq(a, b):
    return a.shape == b.shape and np.array_equal(a, b)


@pytest.mark.parametrize("name", OPS_CASES)
def test_residual_intermediates_vs_oracle(name):
    z = G.load(name)
    P, S = _solver(z)
    U = P.to_soa(list(z["ops_state"]))
    S.set_state(U)
    t = float(z["ops_t"]) if "ops_t" in z.files else 0.0
    dudt, dbg = S.residual(debug=True, t=t)
    ref, rdbg = Oracle(P).residual(U, t=t, debug=True)
    for key in ("gx", "gy", "phi", "vL", "vR", "hL", "hR", "vflux_raw", "hflux_raw", "vflux", "hflux"):
        assert _eq(dbg[key], rdbg[key]), f"{key}: max diff {np.max(np.abs(dbg[key] - rdbg[key]))}"
    assert _eq(dudt, ref), f"dUdt: max diff {np.max(np.abs(dudt - ref))}"
    # and against the reference's own dUdt
    for b in range(P.nblocks):
        assert _eq(P.from_soa(dudt)[b], z[f"ops{int(z['blk_ids'][b])}_dUdt"])


@pytest.mark.parametrize("name", OPS_CASES)
def test_ghost_layer_vs_reference(name):
    """e2d_ghost_layer (halo fill, boundary conditions, conversion) equals the
    reference's reconstruction-block ghosts and the oracle's layer."""
    from test_oracle_golden import ghost_pairs

    z = G.load(name)
    P, S = _solver(z)
    U = P.to_soa(list(z["ops_state"]))
    S.set_state(U)
    t = float(z["ops_t"]) if "ops_t" in z.files else 0.0
    layer = S.ghost_layer(t)
    assert _eq(layer, Oracle(P).ghost_layer(U, t=t))
    for key, mine, ref in ghost_pairs(P, z, layer):
        assert _eq(mine, ref), f"{key}: max diff {np.max(np.abs(mine - ref))}"


@pytest.mark.parametrize("name", CASES)
def test_steps_vs_reference(name):
    """Per-step: dt equal, state fingerprint equal to the reference's."""
    z = G.load(name)
    P, S = _solver(z)
    S.set_state(P.to_soa(list(z["ic"])))
    t, tf = 0.0, G.t_final(z)
    for step in range(1, int(z["steps"]) + 1):
        dt = float(S.compute_dt()[0])
        if tf - t < dt:
            dt = tf - t
        assert dt == z["dts"][step - 1], f"step {step}: dt {dt!r} vs {z['dts'][step - 1]!r}"
        S.step(dt, t)
        t += dt
        blocks = P.from_soa(S.get_state())
        if f"state_{step}" in z.files:
            ref = z[f"state_{step}"]
            assert np.array_equal(np.stack(blocks), ref), f"step {step}: max diff {np.max(np.abs(np.stack(blocks) - ref))}"
        assert G.fingerprint(blocks) == str(z["fingerprints"][step - 1]), f"fingerprint after step {step}"


@pytest.mark.parametrize("name", ["p100", "m2x4_40", "dmr_example", "dmr5", "ti_DormandPrince5", "bc_mixed",
                                  "wedge", "qp2_skew", "qp3_hlll_prim"])
def test_device_loop_vs_reference(name):
    """The device-resident time loop (dt, clamp, stages, t += dt on the GPU, replayed
    from a CUDA graph) reproduces the reference's whole run."""
    z = G.load(name)
    P, S = _solver(z)
    S.set_state(P.to_soa(list(z["ic"])))
    n = int(z["steps"])
    t, steps = S.run(0.0, G.t_final(z), max_steps=n)
    assert steps == n
    assert t == z["ts"][n - 1]
    assert G.fingerprint(P.from_soa(S.get_state())) == str(z["fingerprints"][n - 1])


def test_run_stops_at_t_final():
    """t_final clamp: the last step is shortened so t lands exactly on t_final."""
    z = G.load("ops_explosion_cons")
    P, S = _solver(z)
    U0 = P.to_soa(list(z["ic"]))
    S.set_state(U0)
    tf = 0.5 * float(z["ts"][2])
    t, steps = S.run(0.0, tf, max_steps=1000)
    Ut, t_or, dts = Oracle(P).run(U0, z["tableau"], 0.0, tf, 1000)
    assert t == tf == t_or
    assert steps == len(dts)
    assert np.array_equal(S.get_state(), Ut)


@pytest.mark.parametrize("kernel,variants", [(0, range(6)), (1, range(3)), (2, range(1)), (3, range(3))])
@pytest.mark.parametrize("persistent", [False, True])
def test_kernel_variants_bitwise(kernel, variants, persistent):
    """Every autotuner variant (tile height, occupancy target, persistent grid)
    computes the same values."""
    z = G.load("m2x4_40")
    for v in variants:
        P, S = _solver(z)
        S.set_kernel_choice(kernel, v, persistent)
        S.set_state(P.to_soa(list(z["ic"])))
        t, steps = S.run(0.0, G.t_final(z), max_steps=4)
        assert G.fingerprint(P.from_soa(S.get_state())) == str(z["fingerprints"][3]), (kernel, v, persistent)


def test_autotuned_run_bitwise():
    z = G.load("p100")
    P, S = _solver(z)
    S.set_state(P.to_soa(list(z["ic"])))
    choice = S.autotune(reps=2)
    assert set(choice) == {"reconstruct", "flux", "update", "stage"}
    t, steps = S.run(0.0, G.t_final(z), max_steps=10)
    assert G.fingerprint(P.from_soa(S.get_state())) == str(z["fingerprints"][9])
