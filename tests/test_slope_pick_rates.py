"""How often the FP64 reconstruction kernel's face pick gives up on the benchmark's
data.  The pick is exact either way; this is about speed: a warp whose lane gives
up evaluates psi at all four faces for that variable.  The cell data are the seeded
explosion state of the benchmark (2x4 blocks, here 256 x 256 cells per block), with
the stencil, Green-Gauss gradient, high-order terms and davg formed in numpy float64
by the kernel's expressions on the problem's own geometry planes (interior cells of
block 0), and the pick compiled for the host."""
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def _records(n=256):
    from bench import make_solver
    from pyhype_gb300.problem import (F_LC, F_LS, G_HX_E, G_HY_E, G_INV_A)

    (P, U), _ = make_solver(n, device_solver=False)
    g = P.geometry
    cell = lambda k: np.ctypeslib.as_array(g.cell[k], shape=(P.ncell,))
    vf = lambda k: np.ctypeslib.as_array(g.vface[k], shape=(P.nvface,))
    hf = lambda k: np.ctypeslib.as_array(g.hface[k], shape=(P.nhface,))
    B = P.blocks[0]
    nx, ny = B.nx, B.ny
    i, j = np.meshgrid(np.arange(1, ny - 1), np.arange(1, nx - 1), indexing="ij")
    c = B.cell_offset + i * nx + j
    fE, fW = B.vface_offset + i * (nx + 1) + j + 1, B.vface_offset + i * (nx + 1) + j
    fN, fS = B.hface_offset + (i + 1) * nx + j, B.hface_offset + i * nx + j
    LcE, LcW, LsE, LsW = vf(F_LC)[fE], vf(F_LC)[fW], vf(F_LS)[fE], vf(F_LS)[fW]
    LcN, LcS, LsN, LsS = hf(F_LC)[fN], hf(F_LC)[fS], hf(F_LS)[fN], hf(F_LS)[fS]
    ia = cell(G_INV_A)[c]
    hx = [cell(G_HX_E + s)[c] for s in range(4)]
    hy = [cell(G_HY_E + s)[c] for s in range(4)]
    recs = []
    for v in range(4):
        Uv = U[v]
        w0, we, ea, so, no = Uv[c], Uv[c - 1], Uv[c + 1], Uv[c - nx], Uv[c + nx]
        ie, iw, in_, is_ = 0.5 * (w0 + ea), 0.5 * (we + w0), 0.5 * (w0 + no), 0.5 * (so + w0)
        gx = (ie * LcE + iw * (-LcW) + in_ * LcN + is_ * (-LcS)) * ia
        gy = (ie * LsE + iw * (-LsW) + in_ * LsN + is_ * (-LsS)) * ia
        st = np.stack([w0, we, ea, so, no])
        dmax, dmin = st.max(0) - w0, st.min(0) - w0
        davg = [(w0 + (gx * hx[s] + gy * hy[s])) - w0 for s in range(4)]
        recs.append(np.stack([dmax, dmin] + davg, axis=-1).reshape(-1, 6))
    return np.concatenate(recs)


def test_pick_rarely_gives_up_on_the_benchmark_state(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    exe = str(tmp_path / "rates")
    subprocess.run([gxx, "-O2", "-std=c++17", "-ffp-contract=off", "-Wno-unknown-pragmas",
                    os.path.join(HERE, "slope_pick_rates.cpp"), "-o", exe], check=True)
    data = tmp_path / "records.bin"
    _records().astype(np.float64).tofile(data)
    out = subprocess.run([exe, str(data)], capture_output=True, text=True, check=True).stdout
    r = {k: int(v) for k, v in re.findall(r"(\w+)=(\d+)", out)}
    print(out)
    assert r["lanes"] > 200_000
    assert r["fallback"] < 1e-3 * r["lanes"]           # all-faces path per lane-variable
    assert r["warp_fallback"] < 1e-2 * r["warps"]      # and per warp-variable
    assert r["warp_second"] < 2e-2 * r["warps"]        # both ends evaluated
