"""Batched ensembles: one device problem advancing independent instances of uneven
sizes with per-instance CFL dt must equal the same instances solved one by one."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _small_ensemble():
    from pyhype_gb300.batch import explosion_ensemble

    return explosion_ensemble(count=6, seed=3, sizes=(64, 96, 128))


def test_batched_fp64_equals_sequential_solves():
    from pyhype_gb300.batch import EnsembleSolver

    inst = _small_ensemble()
    B = EnsembleSolver(inst, precision=0)
    B.run(12)
    tb, sb = B.device.instance_times()
    assert list(sb) == [12] * len(inst)
    assert len(set(tb.tolist())) > 1  # per-instance dt really differs
    batched = B.states()
    for k, one in enumerate(inst):
        S = EnsembleSolver([one], precision=0)
        S.run(12)
        t1, _ = S.device.instance_times()
        assert t1[0] == tb[k]
        assert np.array_equal(S.states()[0], batched[k]), f"instance {k}"


def test_batched_fp64_equals_oracle_per_instance():
    """Every instance of the batched FP64 run against the CPU oracle run of that
    instance alone (its own CFL dt each step): time and state value for value."""
    from oracle.oracle import Oracle
    from pyhype_gb300.batch import EnsembleSolver, ensemble_problem, ensemble_state
    from pyhype_gb300.time_marching import tableau

    inst = _small_ensemble()
    B = EnsembleSolver(inst, precision=0)
    B.run(12)
    tb, sb = B.device.instance_times()
    batched = B.states()
    a = tableau("SSPRK2")
    for k, one in enumerate(inst):
        P1 = ensemble_problem([one])
        U, t, dts = Oracle(P1).run(ensemble_state(P1, [one]), a, 0.0, float("inf"), 12)
        assert len(dts) == 12 and t == tb[k], f"instance {k}: t {tb[k]!r} vs oracle {t!r}"
        assert np.array_equal(P1.from_soa(U)[0], batched[k]), f"instance {k}"


def test_batched_fp32_close_to_fp64():
    from pyhype_gb300.batch import EnsembleSolver

    inst = _small_ensemble()
    B64 = EnsembleSolver(inst, precision=0)
    B32 = EnsembleSolver(inst, precision=1, problem=B64.problem)
    B64.run(20)
    B32.run(20)
    for k, (a, b) in enumerate(zip(B64.states(), B32.states())):
        err = np.sum(np.abs(b[:, :, 0] - a[:, :, 0])) / np.sum(np.abs(a[:, :, 0]))
        assert err < 1e-3, f"instance {k}: {err:.2e}"  # uniform-region limiter flips, see test_gpu_fp32
