"""How far a legitimate re-ordering of the reference's own FP64 arithmetic drifts from
it: the oracle compiled with fused multiply-add contraction, on the 100x100 explosion.
This is the floor below which no implementation that is not bit-exact can agree with
the reference (the limiter switches between 0.75 and ~1 on round-off), and the scale
against which the FP32 form's L1 differences are stated."""
import ctypes
import os
import platform
import subprocess
import tempfile

import numpy as np
import pytest

import _golden as G
from oracle.oracle import Oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _fma_oracle(tmp):
    flags = ["-mfma"] if platform.machine() in ("x86_64", "AMD64") else []
    so = os.path.join(tmp, "liboracle_fma.so")
    subprocess.run(["gcc", "-O2", "-fPIC", "-std=gnu11", "-fopenmp", *flags, "-ffp-contract=fast", "-shared", "-o", so,
                    os.path.join(ROOT, "oracle", "e2d_oracle.c"), "-lm"], check=True)
    return ctypes.CDLL(so)


def test_fma_reordering_floor():
    z = G.load("p100")
    P = G.problem(z)
    a = np.ascontiguousarray(z["tableau"])
    U = P.to_soa(list(z["ic"]))
    O = Oracle(P)
    with tempfile.TemporaryDirectory() as tmp:
        L = _fma_oracle(tmp)
        vp = ctypes.c_void_p
        L.oracle_step.argtypes = [vp, vp, vp, vp, ctypes.c_int, vp, ctypes.c_double, ctypes.c_double]
        args = (ctypes.addressof(P.cfg), ctypes.addressof(P.blocks), ctypes.addressof(P.geometry))
        X = U.copy()
        Y = U.copy()
        t = 0.0
        for _ in range(10):
            dt = float(O.dt(X)[0])
            X = O.step(X, a, dt, t)
            L.oracle_step(*args, Y.ctypes.data, a.shape[0], a.ctypes.data, dt, t)
            t += dt
    l1 = np.sum(np.abs(Y[0] - X[0])) / np.sum(np.abs(X[0]))
    # same formulas, same dt schedule, only contraction differs: already above 1e-5
    assert 1e-5 < l1 < 1e-3, l1
