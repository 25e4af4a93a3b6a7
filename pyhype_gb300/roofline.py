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

# Algorithmic HBM bytes per cell-stage of the whole stage (state reads/writes and
# geometry of the cell and its two owned faces), FP64, RK4 low-storage average:
# U_s 32 + U^n 32 + accumulator read+write 64 + U_{s+1} 32 + geometry 64 (A, 1/A and
# 8 quadrature offsets ... counted once per cell).  Face-array traffic between the
# three kernels and halo re-reads are implementation overhead, not counted.
BYTES_PER_CELL_STAGE_FP64 = 224


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
