"""The C-ABI library loads (no GPU needed) and exports every symbol its headers declare."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    names = []
    for h in ("euler2d.h", "euler2d_bench.h"):
        src = open(os.path.join(ROOT, "include", h)).read()
        names += re.findall(r"^E2D_API\s+[\w\s\*]+?\b(e2d_\w+)\s*\(", src, flags=re.M)
    return names


def test_headers_declare_entry_points():
    names = declared()
    assert "e2d_create" in names and "e2d_run" in names and "e2d_bench_fp64_peak" in names
    assert len(names) == len(set(names))


def test_library_exports_all_declared_symbols():
    from pyhype_gb300 import _native

    L = _native.load()
    for name in declared():
        assert hasattr(L, name), name
    assert L.e2d_abi_version() == 2
    assert set(_native.EXPORTS) <= set(declared())


def test_struct_layouts_match_header():
    """ctypes mirrors of the ABI structs have the C sizes (checked by compiling a
    probe with the system C compiler)."""
    import subprocess
    import tempfile

    from pyhype_gb300.problem import E2DBlock, E2DConfig, E2DDebug, E2DGeometry, E2DMixedSide, E2DRealizability

    src = """#include <stdio.h>
#include <stddef.h>
#include "euler2d.h"
int main(void){printf("%zu %zu %zu %zu %zu %zu %zu %zu\\n", sizeof(E2DBlock), sizeof(E2DConfig), sizeof(E2DGeometry),
 sizeof(E2DMixedSide), sizeof(E2DRealizability), sizeof(E2DDebug), offsetof(E2DBlock, cell_offset), offsetof(E2DBlock, mixed));return 0;}"""
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "p.c")
        open(c, "w").write(src)
        exe = os.path.join(d, "p")
        subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), c, "-o", exe], check=True)
        got = list(map(int, subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()))
    want = [ctypes.sizeof(E2DBlock), ctypes.sizeof(E2DConfig), ctypes.sizeof(E2DGeometry), ctypes.sizeof(E2DMixedSide),
            ctypes.sizeof(E2DRealizability), ctypes.sizeof(E2DDebug), E2DBlock.cell_offset.offset, E2DBlock.mixed.offset]
    assert got == want


def test_no_device_fails_loudly():
    """Without a GPU, creating a solver raises instead of falling back to the CPU."""
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import _golden as G
    from pyhype_gb300._native import DeviceSolver, E2DError

    z = G.load("ops_explosion_cons")
    with pytest.raises(E2DError):
        DeviceSolver(G.problem(z))


def _copy(obj):
    dup = type(obj)()
    ctypes.memmove(ctypes.addressof(dup), ctypes.addressof(obj), ctypes.sizeof(obj))
    return dup


def _mutations():
    def cfg(field, value):
        return lambda c, b, g: setattr(c, field, value)

    def blk(i, field, value, idx=None):
        def f(c, b, g):
            if idx is None:
                setattr(b[i], field, value)
            else:
                getattr(b[i], field)[idx] = value
        return f

    def no_plane(c, b, g):
        g.cell[0] = None

    return [
        ("nblocks", cfg("nblocks", 0), "nblocks must be >= 1"),
        ("precision", cfg("precision", 7), "unknown precision"),
        ("flux code", cfg("flux", 9), "unknown flux/limiter/reconstruction code"),
        ("quadrature points", cfg("nqp", 4), "nqp must be 1, 2 or 3"),
        ("block size", blk(0, "nx", 0), "block 0: nx, ny must be >= 1"),
        ("instance id", blk(0, "instance", 5), "block 0: bad instance id"),
        ("offset", blk(1, "cell_offset", -1), "block 1: negative offset"),
        ("side kind", blk(0, "side_kind", 99, 0), "block 0 side 0: bad kind"),
        ("neighbour index", blk(0, "neighbor", 42, 0), "neighbour 42 out of range"),
        ("neighbour size", blk(1, "ny", 39), "neighbour size mismatch"),
        ("geometry", no_plane, "geometry cell plane 0 missing"),
    ]


@pytest.mark.parametrize("name,mutate,message", _mutations(), ids=[m[0] for m in _mutations()])
def test_create_validates_the_problem_before_touching_a_device(name, mutate, message):
    """e2d_create checks the configuration, block table and geometry on the host and
    returns E2D_ERR_INVALID with a message, before any device call (so this runs
    without a GPU)."""
    import _golden as G
    from pyhype_gb300 import _native

    z = G.load("m2x4_40")
    P = G.problem(z)
    assert P.cfg.nblocks == 8
    c = _copy(P.cfg)
    b = (type(P.blocks[0]) * P.cfg.nblocks)()
    ctypes.memmove(b, P.blocks, ctypes.sizeof(b))
    g = _copy(P.geometry)
    mutate(c, b, g)
    L = _native.load()
    h = ctypes.c_void_p()
    code = L.e2d_create(ctypes.addressof(c), ctypes.addressof(b), ctypes.addressof(g), ctypes.byref(h))
    assert code == -1 and not h.value
    assert message in L.e2d_last_error().decode()


def test_bench_and_check_entry_points_validate_arguments():
    """The measurement and check entry points reject bad arguments before touching a
    device: a null handle, a missing output, a wait bound below one poll."""
    from pyhype_gb300._native import E2D_ERR_INVALID, load

    L = load()
    L.e2d_bench_halo.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p]
    L.e2d_bench_set_tma.argtypes = [ctypes.c_void_p, ctypes.c_int32]
    L.e2d_check_wait_bound.argtypes = [ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(ctypes.c_int32)]
    L.e2d_set_kernel_choice.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32]
    ms = (ctypes.c_double * 3)()
    assert L.e2d_bench_halo(None, 10, ctypes.addressof(ms), None) == E2D_ERR_INVALID
    assert L.e2d_bench_set_tma(None, 1) == E2D_ERR_INVALID
    arrived = ctypes.c_int32(0)
    assert L.e2d_check_wait_bound(0, 0, ctypes.byref(arrived)) == E2D_ERR_INVALID
    assert L.e2d_check_wait_bound(0, 10, None) == E2D_ERR_INVALID
    assert L.e2d_set_kernel_choice(None, 0, 0, 0) == E2D_ERR_INVALID
