"""Host-side problem description: the block table and geometry planes the C ABI takes.

``build_problem`` turns a reference-style configuration (``SolverConfig`` + mesh
dictionary) into the structures declared in ``include/euler2d.h``: one ``E2DBlock``
per block (sizes, offsets into the concatenated planes, side kinds, neighbour
indices, boundary-state constants) and the geometry planes (cell and face
quantities, concatenated over blocks).  It runs once per solver construction.

Side kinds follow the reference's ghost logic (``pyhype/blocks/ghost.py:128-216``):
a side with a BC uses the BC even if a neighbour is named; a side with no BC and a
neighbour is an inter-block side; a side with neither copies its own boundary cells.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field
from typing import Dict, List, Optional

import numpy as np

from .mesh.quad_mesh import BlockGeometry, build_block_geometry

# ---- enums of include/euler2d.h --------------------------------------------------
FLUX = {"Roe": 0, "HLLL": 1, "HLLE": 2}
LIMITER = {"Venkatakrishnan": 0, "BarthJespersen": 1, "VanAlbada": 2, "VanLeer": 3}
RECON = {"ConservativeState": 0, "PrimitiveState": 1}
SIDE_NEIGHBOR, SIDE_COPY, SIDE_REFLECT, SIDE_OUTLET, SIDE_DIRICHLET, SIDE_MIXED = range(6)
SIDES = ("E", "W", "N", "S")
G_A, G_INV_A, G_HX_E, G_HX_W, G_HX_N, G_HX_S, G_HY_E, G_HY_W, G_HY_N, G_HY_S, G_CFL_DX, G_CFL_DY = range(12)
N_CELL_PLANES = 12
F_L, F_LC, F_LS, F_COS, F_SIN = range(5)
N_FACE_PLANES = 5

c_double_p = ctypes.POINTER(ctypes.c_double)


class E2DMixedSide(ctypes.Structure):
    _fields_ = [
        ("x0", ctypes.c_double),
        ("speed", ctypes.c_double),
        ("kind_below", ctypes.c_int32),
        ("kind_above", ctypes.c_int32),
        ("ghost_below", ctypes.c_double * 4),
        ("face_below", ctypes.c_double * 4),
        ("ghost_above", ctypes.c_double * 4),
        ("face_above", ctypes.c_double * 4),
    ]


class E2DBlock(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int32),
        ("ny", ctypes.c_int32),
        ("is_cartesian", ctypes.c_int32),
        ("side_kind", ctypes.c_int32 * 4),
        ("neighbor", ctypes.c_int32 * 4),
        ("instance", ctypes.c_int32),
        ("cell_offset", ctypes.c_int64),
        ("vface_offset", ctypes.c_int64),
        ("hface_offset", ctypes.c_int64),
        ("dirichlet_ghost", (ctypes.c_double * 4) * 4),
        ("dirichlet_face", (ctypes.c_double * 4) * 4),
        ("mixed", E2DMixedSide * 4),
        ("side_coord", c_double_p * 4),
    ]


class E2DConfig(ctypes.Structure):
    _fields_ = [
        ("nblocks", ctypes.c_int32),
        ("flux", ctypes.c_int32),
        ("limiter", ctypes.c_int32),
        ("recon", ctypes.c_int32),
        ("precision", ctypes.c_int32),
        ("ninstances", ctypes.c_int32),
        ("gamma", ctypes.c_double),
        ("gm1", ctypes.c_double),
        ("cfl", ctypes.c_double),
        ("nqp", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
    ]


MAX_QP = 3


class E2DGeometry(ctypes.Structure):
    _fields_ = [
        ("cell", c_double_p * N_CELL_PLANES),
        ("vface", c_double_p * N_FACE_PLANES),
        ("hface", c_double_p * N_FACE_PLANES),
        ("qp", (c_double_p * 8) * MAX_QP),
    ]


class E2DRealizability(ctypes.Structure):
    _fields_ = [
        ("ok", ctypes.c_int32),
        ("block", ctypes.c_int32),
        ("cell", ctypes.c_int64),
        ("nbad", ctypes.c_int64),
    ]


class E2DPressureObjective(ctypes.Structure):
    _fields_ = [("block", ctypes.c_int32), ("side", ctypes.c_int32)]


class E2DDebug(ctypes.Structure):
    _fields_ = [(name, c_double_p) for name in
                ("gx", "gy", "phi", "vL", "vR", "hL", "hR", "vflux_raw", "hflux_raw", "vflux", "hflux")]


def _ptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(c_double_p)


@dataclass
class SideSpec:
    """Resolved description of one block side."""

    kind: int
    neighbor: int = -1
    ghost: Optional[np.ndarray] = None      # conservative ghost state (DIRICHLET)
    face: Optional[np.ndarray] = None       # outside state in reconstruction variables
    mixed: Optional[dict] = None            # MIXED parameters


@dataclass
class Problem:
    """Block table + geometry planes for one solver (or one batched ensemble)."""

    cfg: E2DConfig
    blocks: "ctypes.Array"
    geometry: E2DGeometry
    block_geometry: List[BlockGeometry]
    block_ids: List[int]
    cell_offsets: np.ndarray
    ncell: int
    nvface: int
    nhface: int
    _keep: list = field(default_factory=list)

    @property
    def nblocks(self) -> int:
        return len(self.block_ids)

    def with_precision(self, precision: int) -> "Problem":
        """The same block table and geometry with another arithmetic precision
        (0 = FP64, 1 = FP32); arrays are shared, not copied."""
        cfg = E2DConfig()
        ctypes.pointer(cfg)[0] = self.cfg
        cfg.precision = precision
        return Problem(cfg=cfg, blocks=self.blocks, geometry=self.geometry, block_geometry=self.block_geometry,
                       block_ids=self.block_ids, cell_offsets=self.cell_offsets, ncell=self.ncell,
                       nvface=self.nvface, nhface=self.nhface, _keep=self._keep)

    # ---- layout helpers: (nblocks, ny, nx, 4) <-> SoA planes ----------------------
    def to_soa(self, per_block: List[np.ndarray]) -> np.ndarray:
        out = np.empty((4, self.ncell), dtype=np.float64)
        for b, arr in enumerate(per_block):
            B = self.blocks[b]
            n = B.nx * B.ny
            out[:, B.cell_offset:B.cell_offset + n] = np.asarray(arr, dtype=np.float64).reshape(n, 4).T
        return np.ascontiguousarray(out)

    def from_soa(self, soa: np.ndarray) -> List[np.ndarray]:
        soa = np.asarray(soa).reshape(4, self.ncell)
        res = []
        for b in range(self.nblocks):
            B = self.blocks[b]
            n = B.nx * B.ny
            res.append(np.ascontiguousarray(soa[:, B.cell_offset:B.cell_offset + n].T.reshape(B.ny, B.nx, 4)))
        return res

    @property
    def nghost(self) -> int:
        """Cells in the ghost layers of all blocks, 2 (nx + ny) per block."""
        return sum(2 * (self.blocks[b].nx + self.blocks[b].ny) for b in range(self.nblocks))

    def split_ghosts(self, planes: np.ndarray) -> List[dict]:
        """Per block {"E": (ny, 4), "W": (ny, 4), "N": (nx, 4), "S": (nx, 4)} from a
        4-plane ghost-layer array (blocks in table order, sides E, W, N, S)."""
        planes = np.asarray(planes).reshape(4, self.nghost)
        res, o = [], 0
        for b in range(self.nblocks):
            B = self.blocks[b]
            d = {}
            for side, n in (("E", B.ny), ("W", B.ny), ("N", B.nx), ("S", B.nx)):
                d[side] = np.ascontiguousarray(planes[:, o:o + n].T)
                o += n
            res.append(d)
        return res

    def vface_block(self, planes: np.ndarray, b: int) -> np.ndarray:
        """(ny, nx+1, 4) view of a 4-plane vertical-face array for block b."""
        B = self.blocks[b]
        m = B.ny * (B.nx + 1)
        return planes.reshape(4, self.nvface)[:, B.vface_offset:B.vface_offset + m].T.reshape(B.ny, B.nx + 1, 4)

    def hface_block(self, planes: np.ndarray, b: int) -> np.ndarray:
        B = self.blocks[b]
        m = (B.ny + 1) * B.nx
        return planes.reshape(4, self.nhface)[:, B.hface_offset:B.hface_offset + m].T.reshape(B.ny + 1, B.nx, 4)


def _bc_name(bc) -> Optional[str]:
    return None if bc is None else bc


def resolve_side(bc, neighbor_index: Optional[int], recon: int, fluid, geo: BlockGeometry, side: str) -> SideSpec:
    """Map a reference BC value (None, a string, or a BoundaryCondition object) to a
    device side kind."""
    from .boundary_conditions.base import DeviceBoundaryCondition

    if bc is None:
        if neighbor_index is None:
            return SideSpec(SIDE_COPY)
        return SideSpec(SIDE_NEIGHBOR, neighbor=neighbor_index)
    if isinstance(bc, str):
        if bc in ("Reflection", "Slipwall"):
            return SideSpec(SIDE_REFLECT)
        if bc == "OutletDirichlet":
            return SideSpec(SIDE_OUTLET)
        raise ValueError(f"Boundary Condition type {bc} has not been specialized.")
    if isinstance(bc, DeviceBoundaryCondition):
        return bc.side_spec(recon=recon, fluid=fluid, geometry=geo, side=side)
    raise NotImplementedError(
        f"Boundary condition {type(bc).__name__} is a host-side Python callable; only the "
        "built-in kinds and DeviceBoundaryCondition subclasses run on the GPU.")


def build_problem(
    mesh_dict: Dict[int, dict],
    nx: int,
    ny: int,
    flux: str,
    limiter: str,
    recon: str,
    gamma: float,
    gm1: float,
    cfl: float,
    fluid=None,
    precision: int = 0,
    instance_of: Optional[Dict[int, int]] = None,
    sizes: Optional[Dict[int, tuple]] = None,
    geometries: Optional[Dict[int, BlockGeometry]] = None,
    nqp: int = 1,
) -> Problem:
    """Assemble the block table and the geometry planes.

    ``nqp`` is the number of face quadrature points (1, 2 or 3,
    ``SolverConfig.fvm_num_quadrature_points``); with more than one the offsets of
    every point from the centroid are added as extra cell planes.

    ``sizes`` optionally gives per-block ``(nx, ny)`` (independent batched instances);
    otherwise every block uses ``nx, ny`` as the reference does
    (``pyhype/solvers/base.py:90-101``).  ``geometries`` optionally supplies
    precomputed block geometry (e.g. arrays recorded from another platform, whose
    libm may round arctan/cos differently in the last bit).
    """
    if flux not in FLUX:
        raise ValueError(f"Flux function type {flux} is not available.")
    if limiter not in LIMITER:
        raise ValueError("MUSCL: Slope limiter type not specified.")
    if recon not in RECON:
        raise ValueError(f"reconstruction type {recon} is not supported")
    ids = sorted(mesh_dict.keys())
    index = {blk: k for k, blk in enumerate(ids)}
    recon_code = RECON[recon]
    geos, specs, dims = [], [], []
    for blk in ids:
        d = mesh_dict[blk]
        bnx, bny = (sizes[blk] if sizes is not None else (nx, ny))
        if geometries is not None and blk in geometries:
            g = geometries[blk]
        else:
            g = build_block_geometry({k: d[k] for k in ("NE", "NW", "SE", "SW")}, bnx, bny)
        geos.append(g)
        dims.append((bnx, bny))
        sides = []
        for s in SIDES:
            nb = d.get("Neighbor" + s)
            nbi = None if nb is None else index[nb]
            if nbi is not None:
                nnx, nny = sizes[nb] if sizes is not None else (nx, ny)
                if (s in "EW" and nny != bny) or (s in "NS" and nnx != bnx):
                    raise ValueError(f"block {blk} side {s}: neighbour {nb} has a different size")
            sides.append(resolve_side(_bc_name(d.get("BCType" + s)), nbi, recon_code, fluid, g, s))
        specs.append(sides)

    nb = len(ids)
    blocks = (E2DBlock * nb)()
    keep = []
    cell_off = vface_off = hface_off = 0
    cell_offsets = np.zeros(nb, dtype=np.int64)
    for k, (g, sides, (bnx, bny)) in enumerate(zip(geos, specs, dims)):
        B = blocks[k]
        B.nx, B.ny = bnx, bny
        B.is_cartesian = int(g.is_cartesian)
        B.instance = 0 if instance_of is None else int(instance_of[ids[k]])
        B.cell_offset, B.vface_offset, B.hface_offset = cell_off, vface_off, hface_off
        cell_offsets[k] = cell_off
        for si, sp in enumerate(sides):
            B.side_kind[si] = sp.kind
            B.neighbor[si] = sp.neighbor
            if sp.ghost is not None:
                for v in range(4):
                    B.dirichlet_ghost[si][v] = float(sp.ghost[v])
                    B.dirichlet_face[si][v] = float(sp.face[v])
            if sp.mixed is not None:
                m = sp.mixed
                M = B.mixed[si]
                M.x0, M.speed = m["x0"], m["speed"]
                M.kind_below, M.kind_above = m["kind_below"], m["kind_above"]
                for v in range(4):
                    M.ghost_below[v] = m["ghost_below"][v]
                    M.face_below[v] = m["face_below"][v]
                    M.ghost_above[v] = m["ghost_above"][v]
                    M.face_above[v] = m["face_above"][v]
                coord = np.ascontiguousarray(m["coord"], dtype=np.float64)
                keep.append(coord)
                B.side_coord[si] = _ptr(coord)
        cell_off += bnx * bny
        vface_off += bny * (bnx + 1)
        hface_off += (bny + 1) * bnx

    cell = np.empty((N_CELL_PLANES, cell_off))
    vface = np.empty((N_FACE_PLANES, vface_off))
    hface = np.empty((N_FACE_PLANES, hface_off))
    for k, g in enumerate(geos):
        B = blocks[k]
        c0, n = B.cell_offset, B.nx * B.ny
        cell[G_A, c0:c0 + n] = g.A.ravel()
        cell[G_INV_A, c0:c0 + n] = (1.0 / g.A).ravel()
        for si, s in enumerate(SIDES):
            cell[G_HX_E + si, c0:c0 + n] = (getattr(g, f"q{s}_x") - g.xc).ravel()
            cell[G_HY_E + si, c0:c0 + n] = (getattr(g, f"q{s}_y") - g.yc).ravel()
        cell[G_CFL_DX, c0:c0 + n] = g.dx.ravel()
        cell[G_CFL_DY, c0:c0 + n] = g.dy.ravel()
        v0, m = B.vface_offset, B.ny * (B.nx + 1)
        vface[F_L, v0:v0 + m] = g.v_L.ravel()
        vface[F_LC, v0:v0 + m] = (g.v_L * (1 * g.v_cos)).ravel()
        vface[F_LS, v0:v0 + m] = (g.v_L * (1 * g.v_sin)).ravel()
        vface[F_COS, v0:v0 + m] = g.v_cos.ravel()
        vface[F_SIN, v0:v0 + m] = g.v_sin.ravel()
        h0, m = B.hface_offset, (B.ny + 1) * B.nx
        hface[F_L, h0:h0 + m] = g.h_L.ravel()
        hface[F_LC, h0:h0 + m] = (g.h_L * (1 * g.h_cos)).ravel()
        hface[F_LS, h0:h0 + m] = (g.h_L * (1 * g.h_sin)).ravel()
        hface[F_COS, h0:h0 + m] = g.h_cos.ravel()
        hface[F_SIN, h0:h0 + m] = g.h_sin.ravel()

    geometry = E2DGeometry()
    for p in range(N_CELL_PLANES):
        geometry.cell[p] = _ptr(cell[p])
    for p in range(N_FACE_PLANES):
        geometry.vface[p] = _ptr(vface[p])
        geometry.hface[p] = _ptr(hface[p])
    keep += [cell, vface, hface]
    if nqp not in (1, 2, 3):
        raise ValueError(f"fvm_num_quadrature_points must be 1, 2 or 3, not {nqp}")
    if nqp > 1:
        from .mesh.quad_mesh import quadrature_points

        qoff = np.empty((nqp, 8, cell_off))
        for k, g in enumerate(geos):
            B = blocks[k]
            c0, n = B.cell_offset, B.nx * B.ny
            for q, (_, pts) in enumerate(quadrature_points(g, nqp)):
                for si, sd in enumerate(SIDES):
                    qoff[q, si, c0:c0 + n] = (pts[sd][0] - g.xc).ravel()
                    qoff[q, 4 + si, c0:c0 + n] = (pts[sd][1] - g.yc).ravel()
        for q in range(nqp):
            for k in range(8):
                geometry.qp[q][k] = _ptr(qoff[q, k])
        keep.append(qoff)

    cfg = E2DConfig()
    cfg.nblocks = nb
    cfg.flux = FLUX[flux]
    cfg.limiter = LIMITER[limiter]
    cfg.recon = recon_code
    cfg.precision = precision
    cfg.ninstances = 1 if instance_of is None else int(max(instance_of.values()) + 1)
    cfg.gamma = gamma
    cfg.gm1 = gm1
    cfg.cfl = cfl
    cfg.nqp = nqp
    return Problem(cfg=cfg, blocks=blocks, geometry=geometry, block_geometry=geos, block_ids=ids,
                   cell_offsets=cell_offsets, ncell=cell_off, nvface=vface_off, nhface=hface_off, _keep=keep)


def problem_from_config(config, mesh_dict: Dict[int, dict], precision: int = 0) -> Problem:
    """``build_problem`` for a ``SolverConfig`` (reference keyword names)."""
    if config.fvm_type != "MUSCL":
        raise ValueError(f"Specified finite volume method type {config.fvm_type} has not been specialized.")
    if config.fvm_spatial_order != 2:
        raise ValueError(f"No MUSCL finite volume method has been specialized with order {config.fvm_spatial_order}")
    if config.nghost != 1:
        raise ValueError("Number of ghost cells must be equal to 1 for this method.")
    if config.fvm_num_quadrature_points not in (1, 2, 3):
        raise ValueError("fvm_num_quadrature_points must be 1, 2 or 3 (pyhype/mesh/quadratures.py:33-37)")
    if config.fvm_gradient_type != "GreenGauss":
        raise ValueError(f"Gradient type {config.fvm_gradient_type} is not available.")
    if config.interface_interpolation != "arithmetic_average":
        raise ValueError("Interface Interpolation method is not defined.")
    fluid = config.fluid
    return build_problem(
        mesh_dict, config.nx, config.ny,
        flux=config.fvm_flux_function_type,
        limiter=config.fvm_slope_limiter_type,
        recon=config.reconstruction_type.__name__,
        gamma=fluid.gamma(), gm1=fluid.gamma() - 1, cfl=config.CFL, fluid=fluid,
        precision=precision, nqp=int(config.fvm_num_quadrature_points),
    )
