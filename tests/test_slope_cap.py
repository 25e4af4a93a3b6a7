"""The one deliberate deviation from the reference's arithmetic: the Venkatakrishnan
and van Albada slopes are capped at 1e30 (pyhype/limiters/limiters.py:31-56 forms s*s,
which overflows above 1.34e154 and returns inf/inf = NaN).  The cap changes no finite
value the reference produces, and it removes NaNs the reference reaches in practice."""
import warnings

import numpy as np

from oracle.oracle import Oracle
from pyhype_gb300.adjoint import adjoint_problem, smoothed_explosion
from pyhype_gb300.time_marching import tableau


def _venkat(s):
    s2 = s * s
    return (s2 + 2 * s) / (s2 + s + 2)


def _albada(s):
    s2 = s * s
    return (s2 + s) / (s2 + 1)


def test_cap_changes_no_finite_reference_value():
    s = np.concatenate([np.logspace(-3, 16, 20001), np.logspace(16, 153, 20001)])
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        for f in (_venkat, _albada):
            ref = f(s)
            capped = f(np.minimum(s, 1e30))
            assert np.all(np.isfinite(ref))
            assert np.array_equal(ref, capped)
            assert np.all(ref[s >= 1e17] == 1.0)
            big = np.array([2e154, 1e200, 1e300, np.inf])
            assert np.all(np.isnan(f(big)))                  # the reference's NaN
            assert np.all(f(np.minimum(big, 1e30)) == 1.0)   # the capped value


def test_capped_oracle_runs_where_the_reference_reaches_nan():
    """A smoothed 64 x 64 explosion off centre: the reference's slope overflows in the
    quiescent region near the south-east corner in step 25; with the cap every step is
    realizable."""
    P = adjoint_problem(n=64)
    U = smoothed_explosion(P, 4.0, 2.0, 5.3, device="cpu").numpy().copy()
    O = Oracle(P)
    a = tableau("RK4")
    for _ in range(30):
        U = O.step(U, a, float(O.dt(U)[0]))
        assert O.realizable(U).ok == 1
