"""The fused stage kernel (one launch per RK stage: tile + 2-cell halo staged in shared
memory, gradients and limiter of the tile and its ring, one flux per tile face, the
divergence and the stage's Butcher updates) against the reference fixtures, the CPU
oracle and the three-kernel form.

FP64 is value-exact against the reference (every step of every one-point fixture,
including time-dependent boundary sides, inter-block halos and skewed blocks); the FP32
form equals its three-kernel form bit for bit (both evaluate the same functions); TMA
and plain staging agree; odd block shapes (partial tiles, blocks narrower or shorter
than a tile and its halo, rows that rule out TMA) equal the oracle; batched instances
equal the same instances run split."""
import ctypes

import numpy as np
import pytest

import _golden as G
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

ONE_POINT = [c for c in G.cases() if int(G.load(c)["nqp"] if "nqp" in G.load(c).files else 1) == 1]
STAGE = 3
FORMS = [1, 2]  # the fused stage kernel with 28-row and 13-row tiles


def _fused_solver(P, tableau, form=1):
    from pyhype_gb300._native import DeviceSolver

    S = DeviceSolver(P, tableau=tableau)
    S.set_kernel_choice(STAGE, form)
    return S


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("name", ONE_POINT)
def test_fused_steps_vs_reference(name, form):
    """Per step: dt equal to the reference's, state fingerprint equal."""
    z = G.load(name)
    P = G.problem(z)
    S = _fused_solver(P, z["tableau"], form)
    S.set_state(P.to_soa(list(z["ic"])))
    t, tf = 0.0, G.t_final(z)
    for step in range(1, int(z["steps"]) + 1):
        dt = float(S.compute_dt()[0])
        if tf - t < dt:
            dt = tf - t
        assert dt == z["dts"][step - 1], f"step {step}"
        S.step(dt, t)
        t += dt
        assert G.fingerprint(P.from_soa(S.get_state())) == str(z["fingerprints"][step - 1]), f"step {step}"
    S.close()


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("name", ["p100", "m2x4_150", "dmr5", "wedge", "jet", "bc_mixed"])
def test_fused_device_loop_vs_reference(name, form):
    """The graph-replayed device loop with fused stages reproduces the reference's run."""
    z = G.load(name)
    P = G.problem(z)
    S = _fused_solver(P, z["tableau"], form)
    S.set_state(P.to_soa(list(z["ic"])))
    n = int(z["steps"])
    t, steps = S.run(0.0, G.t_final(z), max_steps=n)
    assert steps == n and t == z["ts"][n - 1]
    assert G.fingerprint(P.from_soa(S.get_state())) == str(z["fingerprints"][n - 1])
    S.close()


def _run(P, U, a, steps, form, tma=True):
    """``steps`` steps of the device loop at stage form ``form`` (0 split, 1 / 2 fused)."""
    from pyhype_gb300._native import DeviceSolver, load

    L = load()
    L.e2d_bench_set_tma.argtypes = [ctypes.c_void_p, ctypes.c_int32]
    S = DeviceSolver(P, tableau=a)
    S.set_kernel_choice(STAGE, int(form))
    assert L.e2d_bench_set_tma(S.h, 1 if tma else 0) == 0
    S.set_state(U)
    t, n = S.run(0.0, 1e30, max_steps=steps)
    assert n == steps
    out = S.get_state()
    S.close()
    return out


@pytest.mark.parametrize("name", [c for c in ONE_POINT if c != "m2x4_150"])
def test_fp32_fused_equals_split(name):
    """The FP32 form: fused (both tile shapes) and three-kernel stages give the same bits."""
    z = G.load(name)
    P = G.problem(z, precision=1)
    U = P.to_soa(list(z["ic"]))
    steps = min(int(z["steps"]), 6)
    b = _run(P, U, z["tableau"], steps, 0)
    for form in FORMS:
        a = _run(P, U, z["tableau"], steps, form)
        assert np.array_equal(a, b), f"form {form}: max diff {np.max(np.abs(a - b))}"


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("recon", ["ConservativeState", "PrimitiveState"])
def test_fused_tma_equals_plain_staging(precision, recon, form):
    """Interior tiles staged by one TMA box load and by plain loads agree bit for bit,
    on blocks large enough for interior tiles (2x2 blocks of 96 x 80)."""
    from test_gpu_tma import _problem, _state

    from pyhype_gb300.time_marching import tableau

    P = _problem(96, 80, 2, 2, recon=recon, precision=precision)
    U = _state(P, seed=7)
    a = tableau("RK4")
    on, off = _run(P, U, a, 3, form, tma=True), _run(P, U, a, 3, form, tma=False)
    assert np.array_equal(on, off)
    assert np.array_equal(on, _run(P, U, a, 3, 0))


SHAPES = [(17, 23, 2, 2), (2, 40, 1, 1), (40, 2, 1, 1), (34, 9, 1, 2), (66, 70, 3, 1), (33, 65, 2, 1),
          (100, 37, 1, 2), (31, 18, 2, 1), (1, 30, 2, 1), (45, 1, 1, 2), (70, 62, 1, 1)]


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("nx,ny,bx,by", SHAPES)
def test_fused_shapes_equal_oracle(nx, ny, bx, by, form):
    """Partial tiles, blocks thinner than the halo, odd row lengths: value-exact against
    the oracle over three RK4 steps (FP64), and the FP32 form equal to its split form."""
    from test_gpu_tma import _problem, _state

    from pyhype_gb300.time_marching import tableau

    P = _problem(nx, ny, bx, by)
    U = _state(P, seed=nx * 7 + ny)
    a = tableau("RK4")
    O = Oracle(P)
    S = _fused_solver(P, a, form)
    S.set_state(U)
    Uo = U
    t = 0.0
    for _ in range(3):
        dt = float(S.compute_dt()[0])
        assert dt == float(O.dt(Uo)[0])
        S.step(dt, t)
        Uo = O.step(Uo, a, dt, t)
        t += dt
    assert np.array_equal(S.get_state(), Uo)
    S.close()
    P32 = P.with_precision(1)
    assert np.array_equal(_run(P32, U, a, 3, form), _run(P32, U, a, 3, 0))


@pytest.mark.parametrize("precision", [0, 1])
def test_fused_batched_equals_split(precision):
    """Batched instances of uneven sizes with per-instance dt: fused = split, bitwise."""
    from pyhype_gb300.batch import EnsembleSolver, explosion_ensemble

    inst = explosion_ensemble(count=6, seed=3, sizes=(64, 96, 128))
    out = []
    for form in FORMS + [0]:
        B = EnsembleSolver(inst, precision=precision)
        B.device.set_kernel_choice(STAGE, form)
        B.run(10)
        out.append(np.concatenate([s.ravel() for s in B.states()]))
        B.device.close()
    assert np.array_equal(out[0], out[2]) and np.array_equal(out[1], out[2])


def test_explicit_euler_stays_split_and_exact():
    """A one-stage tableau writes its own input buffer; the stage runs split even with
    the fused form chosen, and stays value-exact."""
    z = G.load("ti_ExplicitEuler1")
    P = G.problem(z)
    S = _fused_solver(P, z["tableau"])
    S.set_state(P.to_soa(list(z["ic"])))
    n = int(z["steps"])
    S.run(0.0, G.t_final(z), max_steps=n)
    assert G.fingerprint(P.from_soa(S.get_state())) == str(z["fingerprints"][n - 1])
    S.close()


def test_fused_rejected_with_quadrature_points():
    from pyhype_gb300._native import E2D_ERR_UNSUPPORTED, DeviceSolver, E2DError

    z = G.load("qp2_roe")
    P = G.problem(z)
    S = DeviceSolver(P, tableau=z["tableau"])
    with pytest.raises(E2DError) as e:
        S.set_kernel_choice(STAGE, 1)
    assert e.value.code == E2D_ERR_UNSUPPORTED
    S.close()
