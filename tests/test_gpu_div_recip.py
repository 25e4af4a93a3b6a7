"""The FP64 divergence's division by a cell area through the geometry's correctly
rounded 1/A (div_recip: two residual corrections of x * (1/A), Markstein's theorem)
against IEEE division, bit for bit: random operands over many binades, divisors whose
significands are all ones or barely above one, quotients next to rounding midpoints,
exact quotients, zeros of both signs and numerators outside the corrected range."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _doubles(rng, n, emin, emax, sign=True):
    e = rng.integers(emin, emax + 1, n, dtype=np.int64)
    m = rng.integers(0, 1 << 52, n, dtype=np.int64)
    s = (rng.integers(0, 2, n, dtype=np.int64) << 63) if sign else np.zeros(n, dtype=np.int64)
    return (s | ((e + 1023) << 52) | m).view(np.float64)


def _check(x, b):
    import torch

    from pyhype_gb300 import _native

    L = _native.load()
    L.e2d_check_div_recip.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64]
    xd, bd = torch.from_numpy(x).cuda(), torch.from_numpy(b).cuda()
    qd = torch.empty_like(xd)
    assert L.e2d_check_div_recip(xd.data_ptr(), bd.data_ptr(), qd.data_ptr(), x.size) == 0
    q = qd.cpu().numpy()
    ref = x / b
    same = q.view(np.uint64) == ref.view(np.uint64)
    return same, q, ref


def test_div_recip_random_operands():
    rng = np.random.default_rng(21)
    n = 1 << 22
    x = _doubles(rng, n, -200, 200)
    b = _doubles(rng, n, -60, 60, sign=False)
    same, q, ref = _check(x, b)
    assert same.all(), f"{int((~same).sum())} of {n} differ, e.g. {x[~same][:3]} / {b[~same][:3]}"


def test_div_recip_adversarial_divisors_and_midpoints():
    rng = np.random.default_rng(22)
    n = 1 << 21
    e = rng.integers(-40, 41, n, dtype=np.int64)
    kind = rng.integers(0, 4, n)
    low = rng.integers(0, 64, n, dtype=np.int64)
    mant = np.where(kind == 0, (1 << 52) - 1 - low,          # significand all ones (1.111...1)
           np.where(kind == 1, low,                          # just above 1
           np.where(kind == 2, (1 << 51) + low - 32,         # around 1.5
                    rng.integers(0, 1 << 52, n, dtype=np.int64))))
    b = (((e + 1023) << 52) | mant).view(np.float64)
    # numerators whose quotient lies next to a rounding midpoint: x = b * (q + ulp(q)/2)
    # rounded, for random q; and exact quotients b * k for small integers k
    qm = _doubles(rng, n, -30, 30)
    mid = qm + np.spacing(qm) / 2
    x = np.where(rng.random(n) < 0.7, b * mid, b * rng.integers(1, 1 << 20, n).astype(np.float64))
    same, q, ref = _check(x, b)
    assert same.all(), f"{int((~same).sum())} of {n} differ, e.g. {x[~same][:3]} / {b[~same][:3]}"


def test_div_recip_zeros_and_extremes():
    b = np.array([1.0, 3.0, 4e-6, 2.5e-7, 1e300, 1e-300, 7.0, 7.0, 7.0, 7.0, 7.0], dtype=np.float64)
    x = np.array([0.0, -0.0, 1e-305, -1e-310, 1e305, 5e-324, 1e290, -1e280, 2.0 ** -900, 2.0 ** 900, np.inf])
    same, q, ref = _check(x, b)
    assert same.all(), f"{x[~same]} / {b[~same]}: {q[~same]} vs {ref[~same]}"
