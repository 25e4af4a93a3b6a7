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


def _device_bc(name: str, side: str, W=None):
    """Device boundary condition for the fixtures' custom reference BC objects (the
    double-Mach setup and the supersonic-wedge inlet of make_golden.py).  ``W`` is a
    Dirichlet side's recorded non-dimensional primitive state."""
    from pyhype_gb300.configs import double_mach_bcs

    west, south, north = double_mach_bcs()
    if name == "Dirichlet":
        if W is None:
            return west()
        from pyhype_gb300.boundary_conditions.base import PrimitiveDirichletBC
        from pyhype_gb300.fluids import Air
        from pyhype_gb300.states import PrimitiveState

        # already non-dimensional: the unit far field makes the class's scaling exact
        return PrimitiveDirichletBC(PrimitiveState(Air(1.0, 1.0), array=np.asarray(W, dtype=float).reshape(1, 1, 4)))
    if name == "Switch":
        return {"S": south, "N": north}[side]()
    return None if name == "None" else name


def mesh_dict(z) -> dict:
    out = {}
    for k, b in enumerate(z["blk_ids"]):
        b = int(b)
        c = z["corners"][k]
        d = {"nBLK": b, "SW": list(c[0]), "SE": list(c[1]), "NW": list(c[2]), "NE": list(c[3])}
        for s, side in enumerate("EWNS"):
            nb = int(z["neighbors"][k, s])
            d["Neighbor" + side] = None if nb < 0 else nb
            W = z["dirichlet_W"][k, s] if "dirichlet_W" in z.files else None
            d["BCType" + side] = _device_bc(str(z["bc"][k, s]), side, W)
        for corner in ("NE", "NW", "SE", "SW"):
            d["Neighbor" + corner] = None
            d["BCType" + corner] = None
        out[b] = d
    return out


def geometry(z, b: int):
    """BlockGeometry assembled from the reference's recorded mesh arrays of block b.

    The transcendental functions behind the face angles and areas (numpy arctan,
    arccos, cos, sin) may round differently on another platform; parity with the
    reference's run is compared on the reference's own geometry."""
    from pyhype_gb300.mesh.quad_mesh import BlockGeometry

    p = f"geo{b}_"
    g = {k[len(p):]: z[k] for k in z.files if k.startswith(p)}
    v = lambda w, e: np.ascontiguousarray(np.concatenate([w[:, :1], e], axis=1))  # noqa: E731
    h = lambda s, n: np.ascontiguousarray(np.concatenate([s[:1, :], n], axis=0))  # noqa: E731
    ny, nx = g["A"].shape
    return BlockGeometry(
        nx=nx, ny=ny, nodes_x=g["nodes_x"], nodes_y=g["nodes_y"], xc=g["xc"], yc=g["yc"], A=g["A"],
        dx=g["dx"], dy=g["dy"],
        v_L=v(g["LW"], g["LE"]), v_theta=v(g["thW"], g["thE"]),
        v_cos=v(g["cos_scalarW"], g["cos_scalarE"]), v_sin=v(g["sin_scalarW"], g["sin_scalarE"]),
        v_mid_x=None, v_mid_y=None,
        h_L=h(g["LS"], g["LN"]), h_theta=h(g["thS"], g["thN"]),
        h_cos=h(g["cos_scalarS"], g["cos_scalarN"]), h_sin=h(g["sin_scalarS"], g["sin_scalarN"]),
        h_mid_x=None, h_mid_y=None,
        qE_x=g["qxE"], qE_y=g["qyE"], qW_x=g["qxW"], qW_y=g["qyW"],
        qN_x=g["qxN"], qN_y=g["qyN"], qS_x=g["qxS"], qS_y=g["qyS"],
        is_cartesian=bool(g["is_cartesian"]),
    )


def problem(z, precision: int = 0, reference_geometry: bool = True, flux=None, recon=None):
    """The fixture's problem; ``flux`` / ``recon`` replace the recorded scheme choice
    (cases the reference cannot run, compared with the oracle only)."""
    from pyhype_gb300.fluids import Air
    from pyhype_gb300.problem import build_problem

    a_inf = float(z["a_inf"]) if "a_inf" in z.files else 343.0
    air = Air(a_inf=a_inf, rho_inf=1.0)
    geos = {int(b): geometry(z, int(b)) for b in z["blk_ids"]} if reference_geometry else None
    return build_problem(
        mesh_dict(z), int(z["nx"]), int(z["ny"]),
        flux=flux or str(z["flux"]), limiter=str(z["limiter"]), recon=recon or str(z["recon"]),
        gamma=air.gamma(), gm1=air.gamma() - 1, cfl=float(z["cfl"]), fluid=air, precision=precision,
        geometries=geos, nqp=int(z["nqp"]) if "nqp" in z.files else 1,
    )


def t_final(z) -> float:
    a_inf = float(z["a_inf"]) if "a_inf" in z.files else 343.0
    return float(z["t_final"]) * a_inf


def cases():
    return sorted(f[:-4] for f in os.listdir(GOLDEN) if f.endswith(".npz"))
