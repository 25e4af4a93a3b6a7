"""The allocation-free CFL time step (e2d_compute_dt_noalloc) against e2d_compute_dt.

Some callers cannot allocate device memory: an application that gives all of its GPU
memory to its own pool allocator and forbids cudaMalloc/cudaFree once running cannot
create a solver handle, yet needs the CFL step of a state it holds.  The entry point
takes only caller-owned device buffers and keeps its scratch in a static device
array.  This file is collected last so a failure here leaves every other test run.
"""
import ctypes

import numpy as np
import pytest

import _golden as G

pytestmark = pytest.mark.gpu

E2D_NOALLOC_MAX_CELLS = 16777216


def _bind(L):
    f = L.e2d_compute_dt_noalloc
    f.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double,
                  ctypes.c_double, ctypes.c_double, ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)]
    f.restype = ctypes.c_int
    return f


def test_noalloc_dt_equals_compute_dt_on_two_calls():
    import torch

    from pyhype_gb300._native import DeviceSolver, load
    from pyhype_gb300.problem import G_CFL_DX, G_CFL_DY

    z = G.load("m2x4_40")
    P = G.problem(z)
    S = DeviceSolver(P, tableau=z["tableau"])
    S.set_state(P.to_soa(list(z["ic"])))
    f = _bind(load())
    dev = torch.device("cuda")
    dx = torch.from_numpy(np.ctypeslib.as_array(P.geometry.cell[G_CFL_DX], shape=(P.ncell,)).copy()).to(dev)
    dy = torch.from_numpy(np.ctypeslib.as_array(P.geometry.cell[G_CFL_DY], shape=(P.ncell,)).copy()).to(dev)
    state = torch.empty((4, P.ncell), dtype=torch.float64, device=dev)
    t = 0.0
    for call in range(2):
        S.get_state_device(state.data_ptr())
        torch.cuda.synchronize()
        ref = float(S.compute_dt()[0])
        out = ctypes.c_double(0.0)
        code = f(state.data_ptr(), P.ncell, dx.data_ptr(), dy.data_ptr(), P.cfg.gamma, P.cfg.gm1, P.cfg.cfl,
                 None, ctypes.byref(out))
        assert code == 0, f"call {call}: status {code}"
        assert out.value == ref, f"call {call}: {out.value!r} != {ref!r}"
        S.step(ref, t)  # a different state for the second call
        t += ref


def test_noalloc_rejects_oversize():
    import torch

    from pyhype_gb300._native import E2D_ERR_INVALID, load

    f = _bind(load())
    buf = torch.zeros(8, dtype=torch.float64, device="cuda")
    out = ctypes.c_double(0.0)
    code = f(buf.data_ptr(), E2D_NOALLOC_MAX_CELLS + 1, buf.data_ptr(), buf.data_ptr(), 1.4, 0.4, 0.8, None,
             ctypes.byref(out))
    assert code == E2D_ERR_INVALID
    assert b"E2D_NOALLOC_MAX_CELLS" in load().e2d_last_error()
