"""Failure detection without a GPU fault: every wait in the kernels is bounded.  The
reconstruction kernel's TMA tile staging waits on a shared-memory barrier for its box;
a wait that runs out is counted and reported by e2d_step / e2d_run instead of hanging.
Here the same bounded wait runs on a barrier phase that a transfer announced but
never delivered (nothing sets it): the wait must run out and return, the host must
read that status, and the context must stay usable for a solver step."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _check(complete, limit):
    from pyhype_gb300._native import load

    L = load()
    L.e2d_check_wait_bound.argtypes = [ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(ctypes.c_int32)]
    arrived = ctypes.c_int32(-1)
    assert L.e2d_check_wait_bound(complete, limit, ctypes.byref(arrived)) == 0
    return arrived.value


def test_wait_runs_out_and_context_stays_usable():
    assert _check(0, 1000) == 0     # nothing arrives: the bound ends the wait
    assert _check(1, 1000) == 1     # the phase completes: the wait sees it
    assert _check(0, 1) == 0        # a bound of one poll
    # the context still runs the solver
    import _golden as G
    from oracle.oracle import Oracle
    from pyhype_gb300._native import DeviceSolver

    z = G.load("p100")
    P = G.problem(z)
    S = DeviceSolver(P, tableau=z["tableau"])
    U = P.to_soa(list(z["ic"]))
    S.set_state(U)
    dt = float(S.compute_dt()[0])
    S.step(dt, 0.0)
    assert np.array_equal(S.get_state(), Oracle(P).step(U, z["tableau"], dt, 0.0))
