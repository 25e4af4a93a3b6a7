"""ctypes front end of the CPU oracle (liboracle.so).  Test infrastructure: used by
tests/, by the smoke check and by the benchmark's CPU-baseline / reference arm, only
as the checker or the CPU baseline, never by the product path."""
from __future__ import annotations

import ctypes
import os
import subprocess
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
_lib = None


def build(force: bool = False) -> str:
    src = os.path.join(HERE, "e2d_oracle.c")
    hdr = os.path.join(HERE, "..", "include", "euler2d.h")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < max(
            os.path.getmtime(src), os.path.getmtime(hdr)):
        subprocess.run(["make", "-s", "-C", HERE, "-B", "liboracle.so"], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        vp = ctypes.c_void_p
        L.oracle_residual.argtypes = [vp, vp, vp, vp, ctypes.c_double, vp, vp]
        L.oracle_step.argtypes = [vp, vp, vp, vp, ctypes.c_int, vp, ctypes.c_double, ctypes.c_double]
        L.oracle_dt.argtypes = [vp, vp, vp, vp, vp]
        L.oracle_realizable.argtypes = [vp, vp, vp, vp, vp]
        L.oracle_ghost_layer.argtypes = [vp, vp, vp, vp, ctypes.c_double, vp]
        L.oracle_flux.argtypes = [ctypes.c_int, ctypes.c_int64, vp, vp, ctypes.c_double, ctypes.c_double, vp]
        L.oracle_set_threads.argtypes = [ctypes.c_int]
        L.oracle_max_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def _p(x):
    return ctypes.cast(ctypes.byref(x), ctypes.c_void_p) if not isinstance(x, np.ndarray) else x.ctypes.data


def face_flux(flux: int, WL: np.ndarray, WR: np.ndarray, gamma: float = 1.4, gm1: float = 1.4 - 1) -> np.ndarray:
    """The oracle's Riemann flux (code as in E2DConfig.flux) of face-frame primitive
    states WL, WR, each (n, 4) (rho, u, v, p); returns (n, 4)."""
    WL = np.ascontiguousarray(WL, dtype=np.float64).reshape(-1, 4)
    WR = np.ascontiguousarray(WR, dtype=np.float64).reshape(-1, 4)
    out = np.zeros_like(WL)
    lib().oracle_flux(int(flux), WL.shape[0], WL.ctypes.data, WR.ctypes.data, float(gamma), float(gm1),
                      out.ctypes.data)
    return out


class Oracle:
    """CPU oracle bound to one ``pyhype_gb300.problem.Problem``."""

    def __init__(self, problem, threads: Optional[int] = None):
        self.P = problem
        self.L = lib()
        if threads:
            self.L.oracle_set_threads(int(threads))

    def _args(self):
        P = self.P
        return (ctypes.addressof(P.cfg), ctypes.addressof(P.blocks), ctypes.addressof(P.geometry))

    def residual(self, U: np.ndarray, t: float = 0.0, debug: bool = False):
        U = np.ascontiguousarray(U, dtype=np.float64).reshape(4, self.P.ncell)
        out = np.zeros_like(U)
        dbg_arrays = None
        dbg_ptr = None
        if debug:
            from pyhype_gb300.problem import E2DDebug, c_double_p
            P = self.P
            dbg_arrays = {
                "gx": np.zeros((4, P.ncell)), "gy": np.zeros((4, P.ncell)), "phi": np.zeros((4, P.ncell)),
                "vL": np.zeros((4, P.nvface)), "vR": np.zeros((4, P.nvface)),
                "hL": np.zeros((4, P.nhface)), "hR": np.zeros((4, P.nhface)),
                "vflux_raw": np.zeros((4, P.nvface)), "hflux_raw": np.zeros((4, P.nhface)),
                "vflux": np.zeros((4, P.nvface)), "hflux": np.zeros((4, P.nhface)),
            }
            d = E2DDebug()
            for k, a in dbg_arrays.items():
                setattr(d, k, a.ctypes.data_as(c_double_p))
            dbg_ptr = ctypes.addressof(d)
            self._dbg = d
        self.L.oracle_residual(*self._args(), U.ctypes.data, float(t), out.ctypes.data, dbg_ptr)
        return (out, dbg_arrays) if debug else out

    def ghost_layer(self, U: np.ndarray, t: float = 0.0) -> np.ndarray:
        """Ghost layer of every block, (4, nghost) in the reconstruction variables
        (``Problem.split_ghosts`` takes it apart per block and side)."""
        U = np.ascontiguousarray(U, dtype=np.float64).reshape(4, self.P.ncell)
        out = np.zeros((4, self.P.nghost))
        self.L.oracle_ghost_layer(*self._args(), U.ctypes.data, float(t), out.ctypes.data)
        return out

    def step(self, U: np.ndarray, tableau: np.ndarray, dt: float, t: float = 0.0, inplace: bool = False) -> np.ndarray:
        """One RK step; returns a new array, or advances U itself with ``inplace`` (U
        must then be a C-contiguous float64 array of 4 x ncell values)."""
        if inplace:
            if U.dtype != np.float64 or not U.flags.c_contiguous or U.size != 4 * self.P.ncell:
                raise ValueError("inplace step needs a C-contiguous float64 state of 4 x ncell values")
        else:
            U = np.array(U, dtype=np.float64, copy=True).reshape(4, self.P.ncell)
        a = np.ascontiguousarray(tableau, dtype=np.float64)
        self.L.oracle_step(*self._args(), U.ctypes.data, a.shape[0], a.ctypes.data, float(dt), float(t))
        return U

    def dt(self, U: np.ndarray) -> np.ndarray:
        U = np.ascontiguousarray(U, dtype=np.float64).reshape(4, self.P.ncell)
        out = np.zeros(max(1, self.P.cfg.ninstances))
        self.L.oracle_dt(*self._args(), U.ctypes.data, out.ctypes.data)
        return out

    def realizable(self, U: np.ndarray):
        from pyhype_gb300.problem import E2DRealizability
        U = np.ascontiguousarray(U, dtype=np.float64).reshape(4, self.P.ncell)
        r = E2DRealizability()
        self.L.oracle_realizable(*self._args(), U.ctypes.data, ctypes.addressof(r))
        return r

    def run(self, U: np.ndarray, tableau: np.ndarray, t: float, t_final: float, max_steps: int):
        """The reference's solve loop: dt -> clamp -> step -> t += dt."""
        U = np.array(U, dtype=np.float64, copy=True).reshape(4, self.P.ncell)
        dts = []
        steps = 0
        while t < t_final and steps < max_steps:
            dt = float(self.dt(U)[0])
            if t_final - t < dt:
                dt = t_final - t
            U = self.step(U, tableau, dt, t)
            t += dt
            dts.append(dt)
            steps += 1
        return U, t, dts
