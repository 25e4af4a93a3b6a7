"""Multiblock layout generators that produce the reference's mesh dictionaries.

``QuadMeshGenerator`` builds a grid of block corners by transfinite (Coons-patch)
interpolation of the four edge curves and numbers the blocks row by row, with the
neighbour and BC keys of ``pyhype/mesh/base.py:133-226``.  The interpolation is the
same weighted sum in the same operation order, so the block corners (and thus every
derived geometry array) come out bit-identical; the reference's 2x4 rectangular
layout has ULP-perturbed interior corners for exactly this reason.
"""
from __future__ import annotations

import numpy as np


class MeshGenerator:
    def __init__(self):
        self.dict = {}


def _coons_interior(x: np.ndarray, nx: int, ny: int) -> np.ndarray:
    jm, im = np.meshgrid(
        np.linspace(1 / nx, (nx - 1) / nx, nx - 2),
        np.linspace(1 / ny, (ny - 1) / ny, ny - 2),
    )
    mj, mi = np.meshgrid(
        np.linspace((nx - 1) / nx, 1 / nx, nx - 2),
        np.linspace((ny - 1) / ny, 1 / ny, ny - 2),
    )
    x[1:-1, 1:-1] = (
        mi * x[0, 1:-1]
        + im * x[-1, 1:-1]
        + mj * x[1:-1, 0, None]
        + jm * x[1:-1, -1, None]
        - mi * mj * x[0, 0]
        - mi * jm * x[0, -1]
        - im * mj * x[-1, 0]
        - im * jm * x[-1, -1]
    )
    return x


class QuadMeshGenerator(MeshGenerator):
    def __init__(self, nx_blk: int, ny_blk: int, BCE, BCW, BCN, BCS,
                 BCNE=None, BCNW=None, BCSE=None, BCSW=None,
                 NE=None, NW=None, SE=None, SW=None,
                 left_x=None, left_y=None, right_x=None, right_y=None,
                 top_x=None, top_y=None, bot_x=None, bot_y=None,
                 blk_num_offset: int = 0):
        super().__init__()
        self.nx, self.ny = nx_blk + 1, ny_blk + 1
        self._blk_num_offset = blk_num_offset
        self.BCE = [BCE[0]] * ny_blk if len(BCE) == 1 else list(BCE)
        self.BCW = [BCW[0]] * ny_blk if len(BCW) == 1 else list(BCW)
        self.BCN = [BCN[0]] * nx_blk if len(BCN) == 1 else list(BCN)
        self.BCS = [BCS[0]] * nx_blk if len(BCS) == 1 else list(BCS)
        _x, _y = np.meshgrid(np.linspace(0, 1, self.nx), np.linspace(0, 1, self.ny))
        _x[0, :] = np.linspace(SW[0], SE[0], self.nx) if bot_x is None else bot_x
        _y[0, :] = np.linspace(SW[1], SE[1], self.nx) if bot_y is None else bot_y
        _x[-1, :] = np.linspace(NW[0], NE[0], self.nx) if top_x is None else top_x
        _y[-1, :] = np.linspace(NW[1], NE[1], self.nx) if top_y is None else top_y
        _x[:, 0] = np.linspace(SW[0], NW[0], self.ny) if left_x is None else left_x
        _y[:, 0] = np.linspace(SW[1], NW[1], self.ny) if left_y is None else left_y
        _x[:, -1] = np.linspace(SE[0], NE[0], self.ny) if right_x is None else right_x
        _y[:, -1] = np.linspace(SE[1], NE[1], self.ny) if right_y is None else right_y
        self.x = _coons_interior(_x, self.nx, self.ny)
        self.y = _coons_interior(_y, self.nx, self.ny)
        self.dict = self._create_block_descriptions()

    def _create_block_descriptions(self) -> dict:
        ny, nx = self.ny - 1, self.nx - 1
        out = {}
        for i in range(ny):
            for j in range(nx):
                n = nx * i + j + self._blk_num_offset
                out[n] = {
                    "nBLK": n,
                    "NW": [self.x[i + 1, j], self.y[i + 1, j]],
                    "NE": [self.x[i + 1, j + 1], self.y[i + 1, j + 1]],
                    "SW": [self.x[i, j], self.y[i, j]],
                    "SE": [self.x[i, j + 1], self.y[i, j + 1]],
                    "NeighborE": n + 1 if j < nx - 1 else None,
                    "NeighborW": n - 1 if j > 0 else None,
                    "NeighborN": n + nx if n + nx < ny * nx else None,
                    "NeighborS": n - nx if n - nx >= 0 else None,
                    "NeighborNE": None,
                    "NeighborNW": None,
                    "NeighborSE": None,
                    "NeighborSW": None,
                    "BCTypeE": self.BCE[i] if j == nx - 1 else None,
                    "BCTypeW": self.BCW[i] if j == 0 else None,
                    "BCTypeN": self.BCN[j] if i == ny - 1 else None,
                    "BCTypeS": self.BCS[j] if i == 0 else None,
                    # the reference's corner keys (mesh/base.py:219-222), kept for the
                    # dictionary format; the corners carry no boundary condition on the
                    # path (the ghost layers are the four sides)
                    "BCTypeNE": self.BCE[i] if j == nx - 1 else None,
                    "BCTypeNW": self.BCW[i] if j == 0 else None,
                    "BCTypeSE": self.BCN[j] if i == ny - 1 else None,
                    "BCTypeSW": self.BCS[j] if i == 0 else None,
                }
        return out
