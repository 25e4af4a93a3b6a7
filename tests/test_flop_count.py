"""Instrumented algorithmic work for the roofline (pyhype_gb300/roofline.py).

The FP64 PyTorch restatement of the scheme (oracle/torch_scheme.py: value-exact
against the reference's fixtures and vectorised over whole arrays as the reference's
numpy code is) runs one residual under an operation counter: every add, sub, mul,
div, reciprocal and sqrt element is one flop (selects, compares, abs, negation: none).
The blocks take the rotation path, as the benchmark's 2x4 rectangular blocks do (they
are skewed by a few ulps).  Per interior cell and per face the counts must equal the
constants the benchmark divides by: 388 flops (40 divisions) per cell in the
reconstruction and 154 flops (8 divisions or reciprocals, 6 square roots) per face
in the Roe flux; the outside states of block-edge cells add 156/n per cell on an
n x n block, which the n = 32 and 64 counts separate."""
import collections

import pytest

torch = pytest.importorskip("torch")
from torch.utils._python_dispatch import TorchDispatchMode  # noqa: E402

import oracle.torch_scheme as TS  # noqa: E402
from pyhype_gb300 import roofline  # noqa: E402

FLOP = {"add", "sub", "mul", "div", "rsub", "reciprocal", "sqrt"}
DIV = {"div", "reciprocal"}


def _count(n):
    from pyhype_gb300.adjoint import adjoint_problem, smoothed_explosion

    c = {"reconstruct": collections.Counter(), "flux": collections.Counter()}
    part = {"p": "reconstruct"}

    class Counter(TorchDispatchMode):
        def __torch_dispatch__(self, func, types, args=(), kwargs=None):
            out = func(*args, **(kwargs or {}))
            name = func.overloadpacket.__name__
            if name in FLOP and isinstance(out, torch.Tensor):
                c[part["p"]]["flop"] += out.numel()
                if name in DIV:
                    c[part["p"]]["div"] += out.numel()
            return out

    roe, sq = TS.roe_flux, TS._Sqrt.forward

    def roe_counted(*a, **k):  # everything from the first flux on is the flux kernel's
        part["p"] = "flux"
        return roe(*a, **k)

    def sqrt_counted(ctx, x):  # the restatement's square roots go through numpy
        c[part["p"]]["flop"] += x.numel()
        c[part["p"]]["sqrt"] += x.numel()
        return sq(ctx, x)

    TS.roe_flux, TS._Sqrt.forward = roe_counted, staticmethod(sqrt_counted)
    try:
        P = adjoint_problem(n=n)
        g = P.block_geometry[0]
        G = TS.Geometry(g)
        G.cart = False
        U = smoothed_explosion(P, 4.0, 2.0, 5.3, device="cpu").reshape(4, g.ny, g.nx).double()
        with Counter():
            TS.Scheme(G, 1.4, 1.4 - 1, limiter="Venkatakrishnan").residual(U)
    finally:
        TS.roe_flux, TS._Sqrt.forward = roe, sq
    ncell, nface = g.nx * g.ny, (g.nx + 1) * g.ny + (g.ny + 1) * g.nx
    # the divergence 0.5 * (((I_W - I_E) + I_S) - I_N) / A of the last line belongs to k_update
    div_flops, div_divs = 20 * ncell, 4 * ncell
    return {"rec": c["reconstruct"]["flop"] / ncell, "rec_div": c["reconstruct"]["div"] / ncell,
            "flux": (c["flux"]["flop"] - div_flops) / nface, "flux_div": (c["flux"]["div"] - div_divs) / nface,
            "flux_sqrt": c["flux"]["sqrt"] / nface}


def test_roofline_work_is_the_instrumented_count():
    a, b = _count(32), _count(64)
    # reconstruct per cell = interior + edge / n
    edge = (a["rec"] - b["rec"]) * 64.0
    interior = b["rec"] - edge / 64.0
    assert interior == roofline.FLOPS_PER_CELL_RECONSTRUCT, (interior, edge)
    assert edge == 156.0
    edge_div = (a["rec_div"] - b["rec_div"]) * 64.0  # the outside states' conversions: 8/n
    assert b["rec_div"] - edge_div / 64.0 == roofline.DIV_PER_CELL_RECONSTRUCT
    assert edge_div == 8.0
    for c in (a, b):
        assert c["flux"] == roofline.FLOPS_PER_FACE_ROE
        assert c["flux_div"] == roofline.DIV_PER_FACE_ROE
        assert c["flux_sqrt"] == roofline.SQRT_PER_FACE_ROE
