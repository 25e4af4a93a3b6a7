"""Algorithmic work per launch of each FP64 stage kernel, for the roofline.

Counts are +, -, *, /, sqrt = 1 flop each (min/max/compare/abs/negation/select = 0) of
the reference's own operation sequence on the benchmark's path (Roe flux,
Venkatakrishnan limiter, conservative reconstruction, blocks that take the rotation
path, as the 2x4 rectangular layout's ULP-skewed blocks do).  They are instrumented,
not read off by hand: tests/test_flop_count.py runs an FP64 PyTorch restatement of the
scheme (value-exact against the reference's fixtures, vectorised over whole arrays as
the reference's numpy code is) under an operation counter and checks these constants.

k_reconstruct, per interior cell: 388 (block-edge cells add the outside states: 156/n
per cell on an n x n block).  By hand: interface averages 4 x (add + mul) = 8,
  Green-Gauss gx, gy 2 x (4 mul + 3 add + 1 mul) = 16, dmax/dmin 2, per side (4): high-
  order term 3, davg 2, slope 1 div, Venkatakrishnan 5 + 1 div = 48, limited face states
  8 -> 82 per variable x 4 = 328; 4 face states rotated (6) and converted to primitive
  (2 div + 7) = 60.  40 of them divisions (the kernel evaluates the slope and psi only
  at the faces that decide phi, about 4 of the 16 per cell, and gets the same phi).
k_flux, per face: 154.  Roe average 18 (1 div, 3 sqrt), 3 sound speeds 9 (3 div,
  3 sqrt), speeds 6, Harten 4 + 8 for both corrected speeds (the reference forms them
  over whole arrays and selects), H/ua/1/a/r2a/h 13 (2 div), dW 4, Lp dW 8, |L| 4,
  Rc 22, F(WL)+F(WR) 26, flux combine 16, rotation back 6, 2 L F 8; a cell owns 2 faces.
k_update, per cell-stage: divergence 5 / var = 20, RK4 stage program on average
  1.75 updates x (1 + 4 x 2) = 35.75.
k_dt, per cell (once per step): conversion 9 (2 div), sound 3 (1 div, 1 sqrt),
  2 x (add + div) = 16.
"""
from __future__ import annotations

FLOPS_PER_CELL_RECONSTRUCT = 388
FLOPS_PER_FACE_ROE = 154
FLOPS_PER_CELL_UPDATE_RK4 = 35.75
FLOPS_PER_CELL_DT = 16
DIV_PER_CELL_RECONSTRUCT = 40
DIV_PER_FACE_ROE = 8  # 6, and the 2 of both corrected speeds
SQRT_PER_FACE_ROE = 6

# FP64 arithmetic instructions (DADD + DMUL + DFMA, per thread) per cell of each FP64
# stage kernel, counted by ncu on the seeded benchmark state
# (smsp__sass_thread_inst_executed_op_{dadd,dmul,dfma}_pred_on.sum over one launch of
# 2 097 152 cells).  With multiply-add contraction off, the DFMAs are those of the
# division and square-root sequences.  The flux kernel's count is per cell (2 faces).
FP64_INST_PER_CELL = {"reconstruct": 432, "flux": 407, "update": 63}
# The FP64 pipe issues at most 2 thread-instructions per SM per clock on GB300 (the
# peak that ncu's FP64 pipe utilisation is relative to).
FP64_INST_PER_SM_CLOCK = 2

# Geometry planes a stage reads once per cell: A, 1/A, the 8 face-point offsets, and
# of the two faces the cell owns (its west and south faces) L, L cos, L sin, cos, sin.
# The face frames (cos, sin) are read only for blocks that take the rotation path.  The
# FP32 form takes the benchmark's blocks, whose frames are axis-aligned to FP32's
# resolution, as Cartesian: it reads no frames (4 planes) and no cross-axis components
# (6 planes: the y offsets of the east and west face points, the x offsets of the
# north and south ones, L sin of the west face and L cos of the south face).
GEOMETRY_PLANES_PER_CELL = 2 + 8 + 2 * 5
FRAME_PLANES_PER_CELL = 2 * 2
CROSS_AXIS_PLANES_PER_CELL = 4 + 2


def stage_state_values(tableau, kahan: bool) -> list:
    """State values (of 4 variables) one RK stage must read and write per cell, per
    stage, as the stage program of the C ABI forms them (e2d_api.cu build_program):
    the stage input, then per Butcher update its source (U^n, or the row's partial
    sum once started; the input is counted once when the source is the input) and
    destination; with Kahan compensation (the FP32 form) the last row's update reads
    and writes U^n and its compensation.  Values of every buffer are 4 per cell."""
    import numpy as np

    a = np.asarray(tableau, dtype=float)
    S = a.shape[0]
    row_buf = lambda r: S if r == S - 1 else r + 1  # noqa: E731
    started = [False] * S
    out = []
    inp = 0
    for s in range(S):
        if s > 0:
            inp = row_buf(s - 1) if any(a[s - 1, j] != 0.0 for j in range(s)) else 0
        n = 1  # the stage input
        for r in range(s, S):
            c = a[r, s]
            if c == 0.0:
                continue
            src = row_buf(r) if started[r] else 0
            zero = kahan and r == S - 1 and not started[r]
            if not zero and src != inp:
                n += 1  # read the source
            if kahan and r == S - 1 and s == S - 1:
                n += 4  # U^n and compensation, read and written
            else:
                n += 1  # write the destination
            started[r] = True
        out.append(4 * n)
    return out


def bytes_per_cell_stage(tableau, elem: int, kahan: bool, frames: bool = True, cross_axis: bool = True) -> float:
    """Algorithmic HBM bytes per cell-stage of a whole step: the stage program's state
    values, the geometry planes once per cell and stage (without the face frames when
    the blocks are taken as Cartesian, and without the cross-axis components when the
    FP32 form takes them so), and the CFL dt's state and two geometry planes once per
    step, averaged over the stages.  Face states, fluxes and halo re-reads are
    implementation traffic, not counted."""
    vals = stage_state_values(tableau, kahan)
    S = len(vals)
    geo = (GEOMETRY_PLANES_PER_CELL - (0 if frames else FRAME_PLANES_PER_CELL)
           - (0 if cross_axis else CROSS_AXIS_PLANES_PER_CELL))
    per_stage = sum(vals) / S + geo
    return elem * (per_stage + 6.0 / S)


# the benchmark's RK4: FP64 128 + 160 + 12 = 300 B (rotation path); FP32 form (Kahan,
# blocks taken as Cartesian) 76 + 40 + 6 = 122 B
_RK4 = [[0.5, 0, 0, 0], [0, 0.5, 0, 0], [0, 0, 1, 0], [1 / 6, 1 / 3, 1 / 3, 1 / 6]]
BYTES_PER_CELL_STAGE_FP64 = bytes_per_cell_stage(_RK4, 8, False)
BYTES_PER_CELL_STAGE_FP32 = bytes_per_cell_stage(_RK4, 4, True, frames=False, cross_axis=False)


def kernel_flops(kind: str, ncell: int, nvface: int, nhface: int) -> float:
    """Algorithmic flops of one launch of a kernel class over the whole problem."""
    if kind == "reconstruct":
        return FLOPS_PER_CELL_RECONSTRUCT * ncell
    if kind == "flux":
        return FLOPS_PER_FACE_ROE * (nvface + nhface)
    if kind == "update":
        return FLOPS_PER_CELL_UPDATE_RK4 * ncell
    if kind == "dt":
        return FLOPS_PER_CELL_DT * ncell
    return 0.0
