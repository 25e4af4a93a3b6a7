"""Per-block structured quad geometry, built once on the host with numpy.

The geometry a block carries into the kernels (cell areas, face lengths, face angles,
normals, quadrature points, centroid offsets, CFL lengths) must be bit-identical to
the reference's, because the limiter reacts to exact zeros and ULP-level differences
in the 2x4 rectangular layout (its block corners are perturbed by ULPs by the
transfinite generator, so those blocks are not Cartesian).  Every array below is
therefore formed with the same numpy operations, in the same order, as the reference:

* nodes: row-wise ``np.linspace`` between the west and east edges, themselves
  ``np.linspace`` between the corners (``pyhype/mesh/quad_mesh.py:71-98``);
* centroid ``0.25*(((ne+nw)+se)+sw)`` (``quad_mesh.py:186-199``);
* face length ``sqrt(dx**2+dy**2)``, midpoint ``0.5*(hi+lo)``, angle ``arctan`` /
  ``pi/2-arctan`` and normal ``dir*(cos, sin)`` (``pyhype/mesh/base.py:29-78``);
* area by Bretschneider's formula with ``arccos``/``cos`` (``quad_mesh.py:137-184``);
* CFL lengths from face-midpoint differences (``quad_mesh.py:134-135``);
* one-point Gauss rule ``0.5*((p2-p1)*0+(p2+p1))`` (``pyhype/mesh/quadratures.py:45-95``).

Unlike the reference, faces are stored once per face (``vertical`` faces between
columns, ``horizontal`` faces between rows) rather than once per cell side: the
east side of cell ``j`` and the west side of cell ``j+1`` are the same node pair, so
the reference's two copies are equal bit for bit.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class BlockGeometry:
    nx: int
    ny: int
    nodes_x: np.ndarray  # (ny+1, nx+1)
    nodes_y: np.ndarray
    xc: np.ndarray  # (ny, nx) centroids
    yc: np.ndarray
    A: np.ndarray  # (ny, nx)
    dx: np.ndarray  # (ny, nx) CFL lengths
    dy: np.ndarray
    # vertical faces (ny, nx+1): face j is the west side of cell j / east side of j-1
    v_L: np.ndarray
    v_theta: np.ndarray
    v_cos: np.ndarray
    v_sin: np.ndarray
    v_mid_x: np.ndarray
    v_mid_y: np.ndarray
    # horizontal faces (ny+1, nx): face i is the south side of row i / north side of i-1
    h_L: np.ndarray
    h_theta: np.ndarray
    h_cos: np.ndarray
    h_sin: np.ndarray
    h_mid_x: np.ndarray
    h_mid_y: np.ndarray
    # one-point quadrature locations per cell side, (ny, nx)
    qE_x: np.ndarray
    qE_y: np.ndarray
    qW_x: np.ndarray
    qW_y: np.ndarray
    qN_x: np.ndarray
    qN_y: np.ndarray
    qS_x: np.ndarray
    qS_y: np.ndarray
    is_cartesian: bool

    # ---- views in the reference's per-side convention (used by tests and the host) ----
    def side(self, s: str):
        """(L, theta, norm_x, norm_y) of side ``s`` of every cell, shape (ny, nx)."""
        if s == "E":
            return self.v_L[:, 1:], self.v_theta[:, 1:], 1 * self.v_cos[:, 1:], 1 * self.v_sin[:, 1:]
        if s == "W":
            return self.v_L[:, :-1], self.v_theta[:, :-1], -1 * self.v_cos[:, :-1], -1 * self.v_sin[:, :-1]
        if s == "N":
            return self.h_L[1:, :], self.h_theta[1:, :], 1 * self.h_cos[1:, :], 1 * self.h_sin[1:, :]
        if s == "S":
            return self.h_L[:-1, :], self.h_theta[:-1, :], -1 * self.h_cos[:-1, :], -1 * self.h_sin[:-1, :]
        raise ValueError(s)

    def boundary_angle(self, s: str) -> np.ndarray:
        """Face angles along block side ``s`` (``quad_mesh.py:362-369``)."""
        return {"E": self.v_theta[:, -1], "W": self.v_theta[:, 0],
                "N": self.h_theta[-1, :], "S": self.h_theta[0, :]}[s]


def _one_point(p1: np.ndarray, p2: np.ndarray) -> np.ndarray:
    p = 0  # the single Gauss point, weight 2
    return 0.5 * ((p2 - p1) * p + (p2 + p1))


# Gauss-Legendre rules on [-1, 1] as (point, weight) in the reference's order
# (pyhype/mesh/quadratures.py:33-37)
QUADRATURE = {
    1: ((0, 2),),
    2: ((-1 / np.sqrt(3), 1), (1 / np.sqrt(3), 1)),
    3: ((-np.sqrt(3 / 5), 5 / 9), (0, 8 / 9), (np.sqrt(3 / 5), 5 / 9)),
}


def quadrature_points(g: "BlockGeometry", nqp: int):
    """Face quadrature points of every cell of a block (pyhype/mesh/quadratures.py:
    40-90): a list over the rule's points of (weight, {side: (x, y)}), each point
    0.5*((p2 - p1)*p + (p2 + p1)) between the side's end nodes (E: NE->SE, W: NW->SW,
    N: NE->NW, S: SE->SW), arrays of shape (ny, nx)."""
    x, y = g.nodes_x, g.nodes_y
    ends = {
        "E": ((x[1:, 1:], y[1:, 1:]), (x[:-1, 1:], y[:-1, 1:])),
        "W": ((x[1:, :-1], y[1:, :-1]), (x[:-1, :-1], y[:-1, :-1])),
        "N": ((x[1:, 1:], y[1:, 1:]), (x[1:, :-1], y[1:, :-1])),
        "S": ((x[:-1, 1:], y[:-1, 1:]), (x[:-1, :-1], y[:-1, :-1])),
    }
    out = []
    for p, w in QUADRATURE[nqp]:
        pts = {}
        for side, ((x1, y1), (x2, y2)) in ends.items():
            pts[side] = (0.5 * ((x2 - x1) * p + (x2 + x1)), 0.5 * ((y2 - y1) * p + (y2 + y1)))
        out.append((w, pts))
    return out


def _length(x1, x2, y1, y2):
    dx = x1 - x2
    dy = y1 - y2
    return np.sqrt(dx * dx + dy * dy)


def build_block_geometry(vertices: dict, nx: int, ny: int) -> BlockGeometry:
    """Geometry of one block from its corner dictionary ``{"NE":..,"NW":..,"SE":..,"SW":..}``."""
    NE, NW, SE, SW = (vertices[k] for k in ("NE", "NW", "SE", "SW"))
    Ex = np.linspace(SE[0], NE[0], ny + 1)
    Ey = np.linspace(SE[1], NE[1], ny + 1)
    Wx = np.linspace(SW[0], NW[0], ny + 1)
    Wy = np.linspace(SW[1], NW[1], ny + 1)
    x = np.zeros((ny + 1, nx + 1), dtype=float)
    y = np.zeros((ny + 1, nx + 1), dtype=float)
    for i in range(ny + 1):
        x[i, :] = np.linspace(Wx[i], Ex[i], nx + 1)
        y[i, :] = np.linspace(Wy[i], Ey[i], nx + 1)

    x_ne, y_ne = x[1:, 1:], y[1:, 1:]
    x_nw, y_nw = x[1:, :-1], y[1:, :-1]
    x_se, y_se = x[:-1, 1:], y[:-1, 1:]
    x_sw, y_sw = x[:-1, :-1], y[:-1, :-1]
    xc = 0.25 * (x_ne + x_nw + x_se + x_sw)
    yc = 0.25 * (y_ne + y_nw + y_se + y_sw)

    # vertical faces: high = upper node, low = lower node of each column line
    vhx, vhy, vlx, vly = x[1:, :], y[1:, :], x[:-1, :], y[:-1, :]
    v_L = np.sqrt((vhx - vlx) ** 2 + (vhy - vly) ** 2)
    v_mid_x = 0.5 * (vhx + vlx)
    v_mid_y = 0.5 * (vhy + vly)
    v_theta = np.arctan((vlx - vhx) / (vhy - vly))
    # horizontal faces: high = west node, low = east node of each row line
    hhx, hhy, hlx, hly = x[:, :-1], y[:, :-1], x[:, 1:], y[:, 1:]
    h_L = np.sqrt((hhx - hlx) ** 2 + (hhy - hly) ** 2)
    h_mid_x = 0.5 * (hhx + hlx)
    h_mid_y = 0.5 * (hhy + hly)
    h_theta = np.pi / 2 - np.arctan((hhy - hly) / (hlx - hhx))

    # Bretschneider area from the per-side lengths of quad_mesh.py:211-268
    s1 = _length(x_sw, x_nw, y_nw, y_sw)  # west
    s3 = _length(x_se, x_ne, y_ne, y_se)  # east
    s2 = _length(x_nw, x_ne, y_ne, y_nw)  # north
    s4 = _length(x_sw, x_se, y_se, y_sw)  # south
    d2 = (x[1:, :-1] - x[:-1, 1:]) ** 2 + (y[1:, :-1] - y[:-1, 1:]) ** 2
    a1 = np.arccos((s1 ** 2 + s4 ** 2 - d2) / (2 * s1 * s4))
    a2 = np.arccos((s2 ** 2 + s3 ** 2 - d2) / (2 * s2 * s3))
    s = 0.5 * (s1 + s2 + s3 + s4)
    p1 = (s - s1) * (s - s2) * (s - s3) * (s - s4)
    p2 = s1 * s2 * s3 * s4
    A = np.sqrt(p1 - 0.5 * p2 * (1 + np.cos(a1 + a2)))

    dx = v_mid_x[:, 1:] - v_mid_x[:, :-1]
    dy = h_mid_y[1:, :] - h_mid_y[:-1, :]

    is_cartesian = bool(
        (NE[1] == NW[1]) and (SE[1] == SW[1]) and (SE[0] == NE[0]) and (SW[0] == NW[0])
    )
    return BlockGeometry(
        nx=nx, ny=ny, nodes_x=x, nodes_y=y, xc=xc, yc=yc, A=A, dx=dx, dy=dy,
        v_L=v_L, v_theta=v_theta, v_cos=np.cos(v_theta), v_sin=np.sin(v_theta),
        v_mid_x=v_mid_x, v_mid_y=v_mid_y,
        h_L=h_L, h_theta=h_theta, h_cos=np.cos(h_theta), h_sin=np.sin(h_theta),
        h_mid_x=h_mid_x, h_mid_y=h_mid_y,
        qE_x=_one_point(x_ne, x_se), qE_y=_one_point(y_ne, y_se),
        qW_x=_one_point(x_nw, x_sw), qW_y=_one_point(y_nw, y_sw),
        qN_x=_one_point(x_ne, x_nw), qN_y=_one_point(y_ne, y_nw),
        qS_x=_one_point(x_se, x_sw), qS_y=_one_point(y_se, y_sw),
        is_cartesian=is_cartesian,
    )


class QuadMesh:
    """Reference-shaped view of a block's geometry (``mesh.x``/``mesh.y`` as
    ``(ny, nx, 1)`` centroid arrays, the shape initial conditions index)."""

    def __init__(self, geometry: BlockGeometry, vertices: dict):
        self.geometry = geometry
        self.vertices = vertices
        self.nx, self.ny = geometry.nx, geometry.ny
        self.x = geometry.xc[:, :, None]
        self.y = geometry.yc[:, :, None]
        self.A = geometry.A[:, :, None]
        self.dx = geometry.dx[:, :, None]
        self.dy = geometry.dy[:, :, None]
        self.shape = (self.ny, self.nx)
