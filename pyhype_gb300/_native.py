"""ctypes binding of libeuler2d.so (the C ABI of include/euler2d.h).

There is no CPU fallback: if the library or a CUDA device is missing, the calls
raise.  ``DeviceSolver`` owns one handle and is what the ``Euler2D`` drop-in,
the benchmark and the tests drive.
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional

import numpy as np

from .problem import E2DDebug, E2DPressureObjective, E2DRealizability, Problem, c_double_p

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libeuler2d.so")

E2D_OK = 0
E2D_ERR_INVALID = -1
E2D_ERR_CUDA = -2
E2D_ERR_UNREALIZABLE = -3
E2D_ERR_TIMEOUT = -4
E2D_ERR_UNSUPPORTED = -5
E2D_ERR_NOMEM = -6

# every symbol include/euler2d.h declares
EXPORTS = (
    "e2d_abi_version", "e2d_last_error", "e2d_create", "e2d_destroy", "e2d_set_stream", "e2d_num_cells",
    "e2d_set_state", "e2d_get_state", "e2d_set_state_device", "e2d_get_state_device", "e2d_set_tableau",
    "e2d_compute_dt", "e2d_step", "e2d_run", "e2d_check_realizable", "e2d_residual", "e2d_instance_times",
    "e2d_residual_vjp", "e2d_adjoint_forward", "e2d_adjoint_backward", "e2d_ghost_layer", "e2d_totals",
)


class E2DError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


class RealizabilityError(E2DError):
    def __init__(self, code, msg, info):
        super().__init__(code, msg)
        self.info = info


_lib = None


def load(path: Optional[str] = None):
    """Load the library (building it first if the sources are newer)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        from . import build as _build

        _build.build()
    L = ctypes.CDLL(path)
    vp = ctypes.c_void_p
    L.e2d_abi_version.restype = ctypes.c_int
    L.e2d_last_error.restype = ctypes.c_char_p
    L.e2d_create.argtypes = [vp, vp, vp, ctypes.POINTER(vp)]
    L.e2d_destroy.argtypes = [vp]
    L.e2d_set_stream.argtypes = [vp, vp]
    L.e2d_num_cells.argtypes = [vp]
    L.e2d_num_cells.restype = ctypes.c_int64
    for n in ("e2d_set_state", "e2d_get_state", "e2d_set_state_device", "e2d_get_state_device"):
        getattr(L, n).argtypes = [vp, vp]
    L.e2d_set_tableau.argtypes = [vp, ctypes.c_int32, vp]
    L.e2d_compute_dt.argtypes = [vp, vp]
    L.e2d_step.argtypes = [vp, ctypes.c_double, ctypes.c_double]
    L.e2d_run.argtypes = [vp, ctypes.POINTER(ctypes.c_double), ctypes.c_double, ctypes.c_int32,
                          ctypes.POINTER(ctypes.c_int32), vp]
    L.e2d_check_realizable.argtypes = [vp, vp]
    L.e2d_instance_times.argtypes = [vp, vp, vp]
    L.e2d_set_kernel_choice.argtypes = [vp, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32]
    L.e2d_autotune.argtypes = [vp, ctypes.c_int32, vp]
    L.e2d_residual.argtypes = [vp, ctypes.c_double, vp, vp]
    L.e2d_residual_vjp.argtypes = [vp, ctypes.c_double, vp, vp]
    L.e2d_ghost_layer.argtypes = [vp, ctypes.c_double, vp]
    L.e2d_totals.argtypes = [vp, vp]
    L.e2d_adjoint_forward.argtypes = [vp, ctypes.c_double, ctypes.c_int32, ctypes.c_int32, vp, vp, vp,
                                      ctypes.POINTER(ctypes.c_double)]
    L.e2d_adjoint_backward.argtypes = [vp, vp]
    if L.e2d_abi_version() != 2:
        raise RuntimeError("libeuler2d.so ABI version mismatch")
    _lib = L
    return L


def _check(code: int):
    if code != 0:
        L = load()
        raise E2DError(code, L.e2d_last_error().decode())


class DeviceSolver:
    """One device-resident problem: state, geometry and stage buffers in HBM."""

    def __init__(self, problem: Problem, tableau: Optional[np.ndarray] = None):
        self.L = load()
        self.problem = problem
        h = ctypes.c_void_p()
        _check(self.L.e2d_create(ctypes.addressof(problem.cfg), ctypes.addressof(problem.blocks),
                                 ctypes.addressof(problem.geometry), ctypes.byref(h)))
        self.h = h
        self.ncell = problem.ncell
        if tableau is not None:
            self.set_tableau(tableau)

    def close(self):
        if getattr(self, "h", None):
            self.L.e2d_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- state --------------------------------------------------------------------
    def set_state(self, soa: np.ndarray):
        a = np.ascontiguousarray(soa, dtype=np.float64).reshape(4, self.ncell)
        _check(self.L.e2d_set_state(self.h, a.ctypes.data))

    def get_state(self, out: Optional[np.ndarray] = None) -> np.ndarray:
        if out is None:
            out = np.empty((4, self.ncell), dtype=np.float64)
        _check(self.L.e2d_get_state(self.h, out.ctypes.data))
        return out

    def set_state_device(self, ptr: int):
        _check(self.L.e2d_set_state_device(self.h, ctypes.c_void_p(ptr)))

    def get_state_device(self, ptr: int):
        _check(self.L.e2d_get_state_device(self.h, ctypes.c_void_p(ptr)))

    def set_stream(self, stream_ptr: int):
        _check(self.L.e2d_set_stream(self.h, ctypes.c_void_p(stream_ptr)))

    # ---- time integration ------------------------------------------------------------
    def set_tableau(self, a: np.ndarray):
        a = np.ascontiguousarray(a, dtype=np.float64)
        _check(self.L.e2d_set_tableau(self.h, a.shape[0], a.ctypes.data))

    def compute_dt(self) -> np.ndarray:
        out = np.zeros(max(1, self.problem.cfg.ninstances))
        _check(self.L.e2d_compute_dt(self.h, out.ctypes.data))
        return out

    def step(self, dt: float, t: float = 0.0):
        _check(self.L.e2d_step(self.h, float(dt), float(t)))

    def run(self, t: float, t_final: float, max_steps: int = 2**31 - 1):
        tt = ctypes.c_double(t)
        steps = ctypes.c_int32(0)
        r = E2DRealizability()
        code = self.L.e2d_run(self.h, ctypes.byref(tt), float(t_final), int(max_steps), ctypes.byref(steps),
                              ctypes.addressof(r))
        if code == E2D_ERR_UNREALIZABLE:
            raise RealizabilityError(code, self.L.e2d_last_error().decode(), r)
        _check(code)
        return tt.value, steps.value

    def set_kernel_choice(self, kernel: int, variant: int, persistent: bool = False):
        _check(self.L.e2d_set_kernel_choice(self.h, kernel, variant, int(persistent)))

    def autotune(self, reps: int = 3) -> dict:
        """Pick the fastest kernel variants on the current state (same results)."""
        ch = np.zeros(8, dtype=np.int32)
        _check(self.L.e2d_autotune(self.h, reps, ch.ctypes.data))
        return {"reconstruct": (int(ch[0]), bool(ch[1])), "flux": (int(ch[2]), bool(ch[3])),
                "update": (int(ch[4]), bool(ch[5])), "stage": (int(ch[6]), False)}

    def instance_times(self):
        n = max(1, self.problem.cfg.ninstances)
        t = np.zeros(n)
        steps = np.zeros(n, dtype=np.int32)
        _check(self.L.e2d_instance_times(self.h, t.ctypes.data, steps.ctypes.data))
        return t, steps

    def check_realizable(self) -> E2DRealizability:
        r = E2DRealizability()
        code = self.L.e2d_check_realizable(self.h, ctypes.addressof(r))
        if code not in (0, E2D_ERR_UNREALIZABLE):
            _check(code)
        return r

    def residual(self, debug: bool = False, t: float = 0.0):
        """dUdt of the current state (host copy), optionally with the intermediates."""
        import torch  # device buffers for the per-operator outputs

        P = self.problem
        dev = torch.device("cuda")
        dudt = torch.zeros((4, P.ncell), dtype=torch.float64, device=dev)
        dbg_t = None
        dptr = None
        if debug:
            shapes = {"gx": P.ncell, "gy": P.ncell, "phi": P.ncell, "vL": P.nvface, "vR": P.nvface,
                      "hL": P.nhface, "hR": P.nhface, "vflux_raw": P.nvface, "hflux_raw": P.nhface,
                      "vflux": P.nvface, "hflux": P.nhface}
            dbg_t = {k: torch.zeros((4, n), dtype=torch.float64, device=dev) for k, n in shapes.items()}
            d = E2DDebug()
            for k, buf in dbg_t.items():
                setattr(d, k, ctypes.cast(buf.data_ptr(), c_double_p))
            self._dbg = d
            dptr = ctypes.addressof(d)
        torch.cuda.synchronize()
        _check(self.L.e2d_residual(self.h, float(t), ctypes.c_void_p(dudt.data_ptr()), dptr))
        out = dudt.cpu().numpy()
        if debug:
            return out, {k: v.cpu().numpy() for k, v in dbg_t.items()}
        return out

    def totals(self) -> np.ndarray:
        """Conserved totals (sum of A * U per variable) of every instance, FP64,
        shape (ninstances, 4)."""
        n = max(1, int(self.problem.cfg.ninstances))
        out = np.zeros((n, 4))
        _check(self.L.e2d_totals(self.h, out.ctypes.data))
        return out

    def ghost_layer(self, t: float = 0.0) -> np.ndarray:
        """Ghost layer of every block at solver time t, (4, nghost) host copy in the
        reconstruction variables (``Problem.split_ghosts`` takes it apart)."""
        import torch

        out = torch.zeros((4, self.problem.nghost), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        _check(self.L.e2d_ghost_layer(self.h, float(t), ctypes.c_void_p(out.data_ptr())))
        return out.cpu().numpy()

    # ---- adjoint ------------------------------------------------------------------------
    def residual_vjp(self, lam, t: float = 0.0):
        """(dR/dU)^T lam at the current state; lam and the result are device tensors of
        shape (4, ncell) (FP64)."""
        import torch

        lam = lam.contiguous()
        out = torch.empty_like(lam)
        torch.cuda.synchronize()
        _check(self.L.e2d_residual_vjp(self.h, float(t), ctypes.c_void_p(lam.data_ptr()),
                                       ctypes.c_void_p(out.data_ptr())))
        return out

    def adjoint_forward(self, nsteps: int, ckpt_every: int, block: int, side: int, t0: float = 0.0,
                        dts: Optional[np.ndarray] = None):
        """Recorded forward pass of J = sum_n dt_n * P(U^{n+1}) (pressure integral along
        one block side); returns (J, dt schedule).  ``dts`` replays a frozen schedule."""
        obj = E2DPressureObjective(int(block), int(side))
        out = np.zeros(nsteps)
        J = ctypes.c_double(0.0)
        din = None
        if dts is not None:
            dts = np.ascontiguousarray(dts, dtype=np.float64)
            assert dts.shape == (nsteps,)
            din = dts.ctypes.data
        code = self.L.e2d_adjoint_forward(self.h, float(t0), int(nsteps), int(ckpt_every), ctypes.addressof(obj),
                                          din, out.ctypes.data, ctypes.byref(J))
        _check(code)
        return J.value, (dts.copy() if dts is not None else out)

    def adjoint_backward(self, out=None):
        """dJ/dU^0 of the last recorded forward pass as a (4, ncell) FP64 device tensor."""
        import torch

        if out is None:
            out = torch.empty((4, self.ncell), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        _check(self.L.e2d_adjoint_backward(self.h, ctypes.c_void_p(out.data_ptr())))
        return out
