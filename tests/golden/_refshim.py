"""Import shim that lets the unmodified pyHype reference run in a container without
numba, mpi4py or matplotlib.  Used only by ``make_golden.py`` (fixture generation);
nothing on the GPU path or in the package imports it.

What it installs in ``sys.modules`` before ``pyhype`` is imported:

* ``numba`` whose ``njit``/``jit`` are identity decorators: the ``@nb.njit`` loop bodies
  then run as plain Python on numpy float64 scalars, with IEEE semantics and no
  contraction (numba's own default is no fastmath either).
* ``mpi4py`` / ``mpi4py.MPI`` as a one-rank world (``Get_rank`` 0, ``Get_size`` 1,
  ``gather`` -> ``[x]``, ``bcast`` -> ``x``, ``Abort`` raises, ``Request.Waitall`` no-op).
* stub ``matplotlib`` modules (plotting is not on the numeric path).
* ``np.int = int``: ``pyhype/flux/eigen_system.py:251`` uses ``dtype=np.int``, removed in
  numpy >= 1.24.
"""
from __future__ import annotations

import os
import sys
import types

REFERENCE_ROOT = os.environ.get("PYHYPE_REFERENCE", "/root/reference")


def _identity_decorator(*args, **kwargs):
    if len(args) == 1 and callable(args[0]) and not kwargs:
        return args[0]

    def wrap(fn):
        return fn

    return wrap


def install() -> None:
    import numpy as np

    if not hasattr(np, "int"):
        np.int = int  # type: ignore[attr-defined]

    nb = types.ModuleType("numba")
    nb.njit = _identity_decorator
    nb.jit = _identity_decorator
    nb.prange = range
    sys.modules.setdefault("numba", nb)

    class _Comm:
        def Get_rank(self):
            return 0

        def Get_size(self):
            return 1

        def Barrier(self):
            return None

        def gather(self, x, root=0):
            return [x]

        def bcast(self, x, root=0):
            return x

        def Abort(self, *a):
            raise RuntimeError("MPI.Abort called by the reference")

        def Isend(self, *a, **k):
            raise RuntimeError("no inter-rank sends in a one-rank world")

        def Irecv(self, *a, **k):
            raise RuntimeError("no inter-rank receives in a one-rank world")

    class _Request:
        @staticmethod
        def Waitall(reqs):
            return None

    class _MPIException(Exception):
        pass

    class _Status:
        def Get_error(self):
            return 0

    mpi_mod = types.ModuleType("mpi4py.MPI")
    mpi_mod.COMM_WORLD = _Comm()
    mpi_mod.Request = _Request
    mpi_mod.Exception = _MPIException
    mpi_mod.Status = _Status
    mpi_mod.Finalize = lambda: None
    mpi_pkg = types.ModuleType("mpi4py")
    mpi_pkg.MPI = mpi_mod
    sys.modules.setdefault("mpi4py", mpi_pkg)
    sys.modules.setdefault("mpi4py.MPI", mpi_mod)

    class _Anything:
        def __getattr__(self, name):
            return _Anything()

        def __call__(self, *a, **k):
            return _Anything()

        def __iter__(self):
            return iter((_Anything(), _Anything()))

    mpl = types.ModuleType("matplotlib")
    plt = types.ModuleType("matplotlib.pyplot")
    plt.__getattr__ = lambda name: _Anything()  # type: ignore[assignment]
    colors = types.ModuleType("matplotlib.colors")

    class _LSC:
        @staticmethod
        def from_list(*a, **k):
            return _Anything()

    colors.LinearSegmentedColormap = _LSC
    collections = types.ModuleType("matplotlib.collections")
    collections.LineCollection = _Anything
    mpl.pyplot = plt
    mpl.colors = colors
    mpl.collections = collections
    for name, mod in (
        ("matplotlib", mpl),
        ("matplotlib.pyplot", plt),
        ("matplotlib.colors", colors),
        ("matplotlib.collections", collections),
    ):
        sys.modules.setdefault(name, mod)

    sys.dont_write_bytecode = True
    if REFERENCE_ROOT not in sys.path:
        sys.path.insert(0, REFERENCE_ROOT)

    import logging

    logging.disable(logging.CRITICAL)
