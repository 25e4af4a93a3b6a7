"""Helpers that turn a golden fixture (tests/golden/*.npz) back into a problem."""
from __future__ import annotations

import hashlib
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name: str):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def fingerprint(arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(np.asarray(a, dtype=np.float64) + 0.0).tobytes())
    return h.hexdigest()[:32]


def mesh_dict(z) -> dict:
    out = {}
    for k, b in enumerate(z["blk_ids"]):
        b = int(b)
        c = z["corners"][k]
        d = {"nBLK": b, "SW": list(c[0]), "SE": list(c[1]), "NW": list(c[2]), "NE": list(c[3])}
        for s, side in enumerate("EWNS"):
            nb = int(z["neighbors"][k, s])
            d["Neighbor" + side] = None if nb < 0 else nb
            bc = str(z["bc"][k, s])
            d["BCType" + side] = None if bc == "None" else bc
        for corner in ("NE", "NW", "SE", "SW"):
            d["Neighbor" + corner] = None
            d["BCType" + corner] = None
        out[b] = d
    return out


def problem(z, precision: int = 0):
    from pyhype_gb300.fluids import Air
    from pyhype_gb300.problem import build_problem

    air = Air(a_inf=343.0, rho_inf=1.0)
    return build_problem(
        mesh_dict(z), int(z["nx"]), int(z["ny"]),
        flux=str(z["flux"]), limiter=str(z["limiter"]), recon=str(z["recon"]),
        gamma=air.gamma(), gm1=air.gamma() - 1, cfl=float(z["cfl"]), fluid=air, precision=precision,
    )


def t_final(z) -> float:
    return float(z["t_final"]) * 343.0


def cases():
    return sorted(f[:-4] for f in os.listdir(GOLDEN) if f.endswith(".npz"))
