"""Algorithmic HBM bytes per cell-stage (pyhype_gb300/roofline.py), the denominators of
the bench's HBM roofline, against hand counts of the stage program that the C ABI
builds for the reference's RK4 (time_marching/explicit_runge_kutta.py:212-224) and
for the Butcher form of SSP-RK2, a = [[1], [0.5, 0.5]]."""
import pytest

from pyhype_gb300.roofline import (BYTES_PER_CELL_STAGE_FP32, BYTES_PER_CELL_STAGE_FP64, bytes_per_cell_stage,
                                   stage_state_values)

RK4 = [[0.5, 0, 0, 0], [0, 0.5, 0, 0], [0, 0, 1, 0], [1 / 6, 1 / 3, 1 / 3, 1 / 6]]
SSPRK2 = [[1.0, 0.0], [0.5, 0.5]]


def test_rk4_state_values_per_stage():
    # stage 0: its input U^n (the source of both updates, read once), row 0's and row
    # 3's partial sums written; stages 1 and 2: input, U^n read, own row written, row
    # 3's partial sum read and written; stage 3: input, row 3's sum read and written
    assert stage_state_values(RK4, kahan=False) == [12, 20, 20, 12]
    # with Kahan compensation the last update reads and writes U^n and its
    # compensation in place of a destination; the first update of row 3 starts from 0
    assert stage_state_values(RK4, kahan=True) == [12, 20, 20, 24]


def test_ssprk2_state_values_per_stage():
    assert stage_state_values(SSPRK2, kahan=False) == [12, 12]
    assert stage_state_values(SSPRK2, kahan=True) == [12, 24]


def test_benchmark_bytes_per_cell_stage():
    # FP64, rotation path: 16 state values, 20 geometry planes, the CFL dt's 6 values
    # once per step: 8 * (16 + 20 + 1.5) = 300
    assert BYTES_PER_CELL_STAGE_FP64 == pytest.approx(300.0)
    # FP32 form on blocks it takes as Cartesian: 19 state values, 10 geometry planes
    # (A, 1/A, the four own-axis offsets, L and the own-axis normal component of the
    # west and south faces): 4 * (19 + 10 + 1.5) = 122
    assert BYTES_PER_CELL_STAGE_FP32 == pytest.approx(122.0)
    # the planes the FP32 form leaves out: the face frames (4), then the cross-axis
    # offsets and normal components (6)
    assert bytes_per_cell_stage(RK4, 4, True) == pytest.approx(162.0)
    assert bytes_per_cell_stage(RK4, 4, True, frames=False) == pytest.approx(146.0)
