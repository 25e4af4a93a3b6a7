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
