"""Axis-aligned multiblock rectangle, as ``pyhype/mesh/rectangular.py:23-62``."""
from __future__ import annotations

import numpy as np

from .base import QuadMeshGenerator


class RectagularMeshGenerator:
    @staticmethod
    def generate(BCE, BCW, BCN, BCS, east: float, west: float, north: float, south: float,
                 n_blocks_horizontal: int, n_blocks_vertical: int) -> QuadMeshGenerator:
        if east <= west:
            raise ValueError(f"East value {east} must be larger than west {west}")
        if north <= south:
            raise ValueError(f"North value {north} must be larger than south {south}")
        tb_y = np.ones(n_blocks_horizontal + 1)
        tb_x = np.linspace(west, east, n_blocks_horizontal + 1)
        ew_x = np.ones(n_blocks_vertical + 1)
        ew_y = np.linspace(south, north, n_blocks_vertical + 1)
        return QuadMeshGenerator(
            nx_blk=n_blocks_horizontal, ny_blk=n_blocks_vertical,
            BCE=BCE, BCW=BCW, BCN=BCN, BCS=BCS,
            top_x=tb_x, bot_x=tb_x, top_y=north * tb_y, bot_y=south * tb_y,
            left_x=west * ew_x, right_x=east * ew_x, left_y=ew_y, right_y=ew_y,
        )


# the spelling most users expect; the reference's name above is kept for drop-in use
RectangularMeshGenerator = RectagularMeshGenerator
