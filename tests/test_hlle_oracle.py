"""Properties of the oracle's HLLE flux (the checker the GPU's HLLE is compared with).

The reference's FluxHLLE (pyhype/flux/HLLE.py:22-47) cannot be constructed (it passes
the solver config where the fluid belongs), so no recorded run pins it.  These tests
pin the oracle's restatement instead: against a numpy transcription of HLLE.py's
array code (Roe state of primitive.py:301-320, wave speeds and Harten correction of
flux/base.py:50-146, the HLL formula and the two np.where of HLLE.py:35-45), and
against the properties of the HLL flux with Einfeldt's bounds (Harten, Lax and van
Leer 1983; Einfeldt 1988; Toro, Riemann Solvers and Numerical Methods for Fluid
Dynamics, 3rd ed., 10.3 and 10.6): consistency F(W, W) = F(W), upwinding of
supersonic states, and mirror symmetry."""
import numpy as np

from oracle.oracle import face_flux

E2D_FLUX_HLLE = 2
GAMMA = 1.4
GM1 = 1.4 - 1


def _cons(W):
    ek = 0.5 * W[:, 0] * (W[:, 1] * W[:, 1] + W[:, 2] * W[:, 2])
    return np.stack([W[:, 0], W[:, 0] * W[:, 1], W[:, 0] * W[:, 2], W[:, 3] / GM1 + ek], axis=1)


def _phys(W, U):
    """PrimitiveState.F(U=...) (pyhype/states/primitive.py:203-209)."""
    return np.stack([U[:, 1], U[:, 1] * W[:, 1] + W[:, 3], U[:, 1] * W[:, 2], W[:, 1] * (U[:, 3] + W[:, 3])], axis=1)


def _hlle_numpy(WL, WR):
    """HLLE.py's compute_flux over arrays, in its operation order."""
    sqL, sqR = np.sqrt(WL[:, 0]), np.sqrt(WR[:, 0])
    inv = 1.0 / (sqL + sqR)
    Q = np.stack([np.sqrt(WL[:, 0] * WR[:, 0])] + [(WL[:, v] * sqL + WR[:, v] * sqR) * inv for v in (1, 2, 3)], axis=1)

    def speeds(W):
        a = np.sqrt(GAMMA * W[:, 3] / W[:, 0])
        return W[:, 1] - a, W[:, 1] + a

    L_p, L_m = speeds(WL)  # slow, fast (flux/base.py:50-74)
    R_p, R_m = speeds(WR)
    Roe_p, Roe_m = speeds(Q)
    tp = 2 * (R_p - L_p)
    tm = 2 * (R_m - L_m)
    tp = np.where(tp <= 0, 1e-8, tp)
    tm = np.where(tm <= 0, 1e-8, tm)
    _hlle_numpy.fired_slow = np.abs(Roe_p) < tp
    _hlle_numpy.fired_fast = np.abs(Roe_m) < tm
    _hlle_numpy.fired = _hlle_numpy.fired_slow | _hlle_numpy.fired_fast
    Roe_p = np.where(np.abs(Roe_p) < tp, 0.5 * ((Roe_p * Roe_p) / tp + tp), Roe_p)
    Roe_m = np.where(np.abs(Roe_m) < tm, 0.5 * ((Roe_m * Roe_m) / tm + tm), Roe_m)
    L_plus = np.maximum(R_m, Roe_m)[:, None]
    L_minus = np.minimum(L_p, Roe_p)[:, None]
    UL, UR = _cons(WL), _cons(WR)
    FL, FR = _phys(WL, UL), _phys(WR, UR)
    with np.errstate(divide="ignore", invalid="ignore"):
        F = (L_plus * FL - L_minus * FR + L_minus * L_plus * (UR - UL)) / (L_plus - L_minus)
    F = np.where(L_minus >= 0, FL, F)
    F = np.where(L_plus <= 0, FR, F)
    return F, L_minus[:, 0], L_plus[:, 0]


def _states(rng, n, mach_lo, mach_hi):
    rho = rng.uniform(0.2, 5.0, n)
    p = rng.uniform(0.1, 10.0, n)
    a = np.sqrt(GAMMA * p / rho)
    u = a * rng.uniform(mach_lo, mach_hi, n)
    v = a * rng.uniform(-1.0, 1.0, n)
    return np.stack([rho, u, v, p], axis=1)


def test_hlle_equals_numpy_transcription_of_reference():
    rng = np.random.default_rng(5)
    WL = _states(rng, 20000, -3.0, 3.0)
    WR = _states(rng, 20000, -3.0, 3.0)
    F = face_flux(E2D_FLUX_HLLE, WL, WR)
    ref, lm, lp = _hlle_numpy(WL, WR)
    # all three branches are exercised
    assert np.any(lm >= 0) and np.any(lp <= 0) and np.any((lm < 0) & (lp > 0))
    assert np.array_equal(F, ref)


def test_hlle_consistency():
    """F(W, W) is the physical flux F(W) (to rounding of the HLL average)."""
    rng = np.random.default_rng(6)
    W = _states(rng, 5000, -2.5, 2.5)
    F = face_flux(E2D_FLUX_HLLE, W, W)
    Fp = _phys(W, _cons(W))
    scale = np.max(np.abs(Fp), axis=1, keepdims=True)
    assert np.all(np.abs(F - Fp) <= 1e-14 * scale)


def test_hlle_supersonic_states_upwind():
    """Both states supersonic to the right: F = F_L exactly.  To the left: F = F_R
    exactly wherever the Harten fix leaves the Roe speeds alone.  Where it fires it
    replaces a small Roe speed by 0.5 (s^2/t + t) > 0 whatever the sign of s
    (flux/base.py:137-146), so a negative fast speed turns positive, L+ > 0 and the
    face takes the HLL average: the reference's rule, kept."""
    rng = np.random.default_rng(7)
    WL = _states(rng, 3000, 3.0, 5.0)
    WR = _states(rng, 3000, 3.0, 5.0)
    assert np.array_equal(face_flux(E2D_FLUX_HLLE, WL, WR), _phys(WL, _cons(WL)))
    WL = _states(rng, 3000, -5.0, -3.0)
    WR = _states(rng, 3000, -5.0, -3.0)
    F = face_flux(E2D_FLUX_HLLE, WL, WR)
    _, _, lp = _hlle_numpy(WL, WR)
    keep = ~_hlle_numpy.fired_fast
    assert keep.sum() > 1000 and np.all(lp[keep] <= 0)
    assert np.array_equal(F[keep], _phys(WR, _cons(WR))[keep])
    assert np.any(~keep) and np.all(lp[~keep] > 0)


def test_hlle_subsonic_is_hll_average():
    """Subsonic pairs: L- < 0 < L+ and the flux is the HLL state-flux average."""
    rng = np.random.default_rng(8)
    WL = _states(rng, 3000, -0.5, 0.5)
    WR = _states(rng, 3000, -0.5, 0.5)
    F = face_flux(E2D_FLUX_HLLE, WL, WR)
    ref, lm, lp = _hlle_numpy(WL, WR)
    assert np.all(lm < 0) and np.all(lp > 0)
    UL, UR = _cons(WL), _cons(WR)
    FL, FR = _phys(WL, UL), _phys(WR, UR)
    hll = (lp[:, None] * FL - lm[:, None] * FR + (lm * lp)[:, None] * (UR - UL)) / (lp - lm)[:, None]
    assert np.array_equal(F, hll)


def test_hlle_mirror_symmetry():
    """Swapping the states and reversing the normal velocity mirrors the flux:
    mass, y-momentum and energy fluxes change sign, the x-momentum flux does not.
    Checked where the Harten fix fires on neither pair (where it fires it keeps the
    corrected speed positive whatever its sign, which is not mirror symmetric)."""
    rng = np.random.default_rng(9)
    WL = _states(rng, 5000, -2.0, 2.0)
    WR = _states(rng, 5000, -2.0, 2.0)
    m = np.array([1.0, -1.0, 1.0, 1.0])
    F = face_flux(E2D_FLUX_HLLE, WL, WR)
    Fm = face_flux(E2D_FLUX_HLLE, WR * m, WL * m)
    _hlle_numpy(WL, WR)
    keep = ~_hlle_numpy.fired
    _hlle_numpy(WR * m, WL * m)
    keep &= ~_hlle_numpy.fired
    assert keep.sum() > 1000
    scale = np.max(np.abs(F), axis=1, keepdims=True)
    # F0(WL, WR) = -F0(mWR, mWL), F1 = F1, F2 = -F2, F3 = -F3
    sign = np.array([-1.0, 1.0, -1.0, -1.0])
    assert np.all((np.abs(F - sign * Fm) <= 1e-13 * scale)[keep])
