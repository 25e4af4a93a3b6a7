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


def _cfl_planes(P, dev):
    import torch

    from pyhype_gb300.problem import G_CFL_DX, G_CFL_DY

    dx = np.ctypeslib.as_array(P.geometry.cell[G_CFL_DX], shape=(P.ncell,)).copy()
    dy = np.ctypeslib.as_array(P.geometry.cell[G_CFL_DY], shape=(P.ncell,)).copy()
    return dx, dy, torch.from_numpy(dx).to(dev), torch.from_numpy(dy).to(dev)


def _call(f, state, P, dx, dy):
    out = ctypes.c_double(0.0)
    code = f(state.data_ptr(), P.ncell, dx.data_ptr(), dy.data_ptr(), P.cfg.gamma, P.cfg.gm1, P.cfg.cfl, None,
             ctypes.byref(out))
    return code, out.value


def test_noalloc_dt_equals_compute_dt_on_two_calls():
    import torch

    from pyhype_gb300._native import DeviceSolver, load

    z = G.load("m2x4_40")
    P = G.problem(z)
    S = DeviceSolver(P, tableau=z["tableau"])
    S.set_state(P.to_soa(list(z["ic"])))
    f = _bind(load())
    dev = torch.device("cuda")
    _, _, dx, dy = _cfl_planes(P, dev)
    state = torch.empty((4, P.ncell), dtype=torch.float64, device=dev)
    t = 0.0
    for call in range(2):
        S.get_state_device(state.data_ptr())
        torch.cuda.synchronize()
        ref = float(S.compute_dt()[0])
        code, val = _call(f, state, P, dx, dy)
        assert code == 0, f"call {call}: status {code}"
        assert val == ref, f"call {call}: {val!r} != {ref!r}"
        S.step(ref, t)  # a different state for the second call
        t += ref
    S.close()


def _cfl_min_numpy(U, dx, dy, gamma, gm1):
    """min over cells of min(dx/(|u|+a), dy/(|v|+a)) with the scheme's operations in
    its order (IEEE division and square root, as the device computes them)."""
    rho = U[0]
    u = U[1] / rho
    v = U[2] / rho
    ek = rho * (0.5 * (u * u + v * v))
    p = gm1 * (U[3] - ek)
    a = np.sqrt(gamma * p / rho)
    return float(np.min(np.minimum(dx / (np.abs(u) + a), dy / (np.abs(v) + a))))


def test_noalloc_dt_large_ragged_problem():
    """One 1031 x 1025 block (1,056,775 cells: 4,129 per-tile minima, more than the final
    reduction's 1024 threads, the last tile holding 7 cells) with the smallest CFL time
    in that last tile; two calls with the minimum in different cells."""
    import torch

    from pyhype_gb300._native import DeviceSolver, load
    from pyhype_gb300.mesh import RectagularMeshGenerator
    from pyhype_gb300.problem import build_problem

    nx, ny = 1031, 1025
    mesh = RectagularMeshGenerator.generate(["Reflection"], ["Reflection"], ["Reflection"], ["Reflection"],
                                            10.0, 0.0, 10.0, 0.0, 1, 1)
    P = build_problem(mesh.dict, nx, ny, flux="Roe", limiter="Venkatakrishnan", recon="ConservativeState",
                      gamma=1.4, gm1=1.4 - 1, cfl=0.8)
    assert P.ncell == nx * ny and P.ncell > 4 * 1024 * 256 and P.ncell % 256 == 7
    rng = np.random.default_rng(11)
    W = np.empty((4, P.ncell))
    W[0] = 1.0 + 0.01 * rng.random(P.ncell)
    W[1] = 0.01 * rng.standard_normal(P.ncell)
    W[2] = 0.01 * rng.standard_normal(P.ncell)
    W[3] = 1.0 / 1.4 * (1.0 + 0.01 * rng.random(P.ncell))
    f = _bind(load())
    dev = torch.device("cuda")
    dxh, dyh, dx, dy = _cfl_planes(P, dev)
    S = DeviceSolver(P)
    for call, fast in enumerate((P.ncell - 3, P.ncell - 7)):
        Wc = W.copy()
        Wc[1, fast] = 5.0  # the fastest cell: the smallest CFL time, in the last 256-cell tile
        U = np.empty_like(Wc)
        U[0] = Wc[0]
        U[1] = Wc[0] * Wc[1]
        U[2] = Wc[0] * Wc[2]
        U[3] = Wc[3] / (1.4 - 1) + 0.5 * Wc[0] * (Wc[1] ** 2 + Wc[2] ** 2)
        state = torch.from_numpy(U).to(dev)
        S.set_state(U)
        ref = float(S.compute_dt()[0])
        expect = 0.8 * _cfl_min_numpy(U, dxh, dyh, 1.4, 1.4 - 1)
        code, val = _call(f, state, P, dx, dy)
        assert code == 0, f"call {call}: status {code}"
        assert val == ref == expect, f"call {call}: {val!r}, handle {ref!r}, numpy {expect!r}"
        # the minimum really sits in the ragged last tile
        u = U[1] / U[0]
        a = np.sqrt(1.4 * ((1.4 - 1) * (U[3] - U[0] * 0.5 * (u * u + (U[2] / U[0]) ** 2))) / U[0])
        tx = dxh / (np.abs(u) + a)
        assert int(np.argmin(tx)) == fast
    S.close()


def test_noalloc_allocates_no_device_memory():
    """Warm calls leave the device's free memory unchanged."""
    import torch

    from pyhype_gb300._native import DeviceSolver, load

    z = G.load("m2x4_40")
    P = G.problem(z)
    S = DeviceSolver(P, tableau=z["tableau"])
    S.set_state(P.to_soa(list(z["ic"])))
    f = _bind(load())
    dev = torch.device("cuda")
    _, _, dx, dy = _cfl_planes(P, dev)
    state = torch.empty((4, P.ncell), dtype=torch.float64, device=dev)
    S.get_state_device(state.data_ptr())
    torch.cuda.synchronize()
    code, first = _call(f, state, P, dx, dy)  # warm: the one-time symbol lookup
    assert code == 0
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        code, val = _call(f, state, P, dx, dy)
        assert code == 0 and val == first
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, f"device free memory changed by {free0 - free1} bytes"
    S.close()


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
