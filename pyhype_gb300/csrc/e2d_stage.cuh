// e2d_stage.cuh - the stage kernels of the 2D Euler MUSCL scheme, templated on the
// arithmetic type.  Included by e2d_fp64.cu (T = double, -fmad=false: the
// bit-exact path) and e2d_fp32.cu (T = float, contraction allowed, Kahan-compensated
// step accumulation).
//
// One RK stage is three launches over every block of the problem at once (a tile
// table maps CTAs to (block, tile) pairs):
//
//   k_reconstruct  per cell: reconstruction-type state of the cell and its four
//                  neighbours (an interior tile arrives by one TMA box load, edge tiles
//                  by plain loads with ghost cells formed on the fly), interface
//                  averages, Green-Gauss gradient, limiter (in FP64 psi only at the
//                  faces that decide phi, e2d_slope_pick.cuh), limited face states;
//                  each face state is rotated into its face frame, converted to
//                  primitive and written to the face-indexed L/R arrays, block-boundary
//                  cells also write the outside state of their boundary face.
//   k_flux         per face, exactly once: Riemann flux of (L, R), rotated back,
//                  times 2*L (one-point rule, weight 2).
//   k_update       per cell: dUdt = 0.5*(((I_W - I_E) + I_S) - I_N)/A and the RK stage
//                  program (every partial Butcher sum this stage contributes to);
//                  on the last stage also the positivity check.
//
// GB300's FP64 pipe is the binding resource of this scheme in FP64 (about 900 FP64
// instructions per cell-stage against ~250 bytes of HBM traffic), so the split
// avoids every recomputation a fused halo-tile kernel would do (gradients and
// limiter of the halo ring, fluxes of tile-edge faces); the extra face-array traffic
// costs HBM bandwidth that is otherwise idle.
#pragma once
#include <cstdio>

#include "e2d_device.cuh"
#include "e2d_kernels.cuh"
#include "e2d_slope_pick.cuh"
#include "e2d_tma.cuh"

namespace e2d {


__device__ __forceinline__ int64_t cell_at(const E2DBlock* B, int i, int j) {
  return B->cell_offset + (int64_t)i * B->nx + j;
}
__device__ __forceinline__ int64_t vf_at(const E2DBlock* B, int i, int j) {
  return B->vface_offset + (int64_t)i * (B->nx + 1) + j;
}
__device__ __forceinline__ int64_t hf_at(const E2DBlock* B, int i, int j) {
  return B->hface_offset + (int64_t)i * B->nx + j;
}

// Side kind at position k along a side, resolving MIXED sides; gd/fd point at the
// Dirichlet ghost (conservative) and face (reconstruction variables) vectors.
__device__ __forceinline__ int side_kind_at(const E2DBlock* B, int side, int k, double t,
                                            const double*& gd, const double*& fd) {
  int kind = B->side_kind[side];
  gd = B->dirichlet_ghost[side];
  fd = B->dirichlet_face[side];
  if (kind == E2D_SIDE_MIXED) {
    const E2DMixedSide* m = &B->mixed[side];
    double coord = B->side_coord[side][k];
    if (coord < m->x0 + m->speed * t) {
      kind = m->kind_below; gd = m->ghost_below; fd = m->face_below;
    } else {
      kind = m->kind_above; gd = m->ghost_above; fd = m->face_above;
    }
  }
  return kind;
}

template <typename T>
__device__ __forceinline__ void boundary_cs(const ParamsT<T>& P, const E2DBlock* B, int side, int k, T& c, T& s) {
  int64_t f;
  if (side == E2D_E) { f = vf_at(B, k, B->nx); c = P.geo.vface[E2D_F_COS][f]; s = P.geo.vface[E2D_F_SIN][f]; }
  else if (side == E2D_W) { f = vf_at(B, k, 0); c = P.geo.vface[E2D_F_COS][f]; s = P.geo.vface[E2D_F_SIN][f]; }
  else if (side == E2D_N) { f = hf_at(B, B->ny, k); c = P.geo.hface[E2D_F_COS][f]; s = P.geo.hface[E2D_F_SIN][f]; }
  else { f = hf_at(B, 0, k); c = P.geo.hface[E2D_F_COS][f]; s = P.geo.hface[E2D_F_SIN][f]; }
}

template <typename T>
__device__ __forceinline__ void load_cell(const T* __restrict__ U, int64_t ncell, int64_t c, T* q) {
  q[0] = U[c];
  q[1] = U[ncell + c];
  q[2] = U[2 * ncell + c];
  q[3] = U[3 * ncell + c];
}

// Ghost cell (conservative variables) at position k along a side: neighbour cell,
// own boundary cell (copy / outlet), its reflection, or a Dirichlet state
// (pyhype/blocks/ghost.py:149-158,187-216).
template <typename T>
__device__ void ghost_cons(const ParamsT<T>& P, const E2DBlock* B, int side, int k, const T* __restrict__ U,
                           double t, T* g) {
  const double *gd, *fd;
  int kind = side_kind_at(B, side, k, t, gd, fd);
  if (kind == E2D_SIDE_NEIGHBOR) {
    const E2DBlock* N = P.blocks + B->neighbor[side];
    int64_t c;
    if (side == E2D_E) c = cell_at(N, k, 0);
    else if (side == E2D_W) c = cell_at(N, k, N->nx - 1);
    else if (side == E2D_N) c = cell_at(N, 0, k);
    else c = cell_at(N, N->ny - 1, k);
    load_cell(U, P.ncell, c, g);
    return;
  }
  if (kind == E2D_SIDE_DIRICHLET) {
    g[0] = T(gd[0]); g[1] = T(gd[1]); g[2] = T(gd[2]); g[3] = T(gd[3]);
    return;
  }
  int64_t c;
  if (side == E2D_E) c = cell_at(B, k, B->nx - 1);
  else if (side == E2D_W) c = cell_at(B, k, 0);
  else if (side == E2D_N) c = cell_at(B, B->ny - 1, k);
  else c = cell_at(B, 0, k);
  load_cell(U, P.ncell, c, g);
  if (kind == E2D_SIDE_REFLECT) {
    T cs, sn;
    boundary_cs(P, B, side, k, cs, sn);
    reflect(g, cs, sn);
  }
}

template <typename T>
__device__ __forceinline__ void store4(T* __restrict__ base, int64_t stride, int64_t f, const T* q) {
  base[f] = q[0];
  base[stride + f] = q[1];
  base[2 * stride + f] = q[2];
  base[3 * stride + f] = q[3];
}

// Outside state (reconstruction variables) of the boundary face at position k of
// side `side`: ghost average for inter-block/copy sides, else the block's own
// limited face state with the side's BC applied (pyhype/fvm/base.py:305-325 and the
// apply_boundary_condition_to_state calls of fvm/base.py:353-363,419-429).
template <typename T>
__device__ __forceinline__ void outside_state(const ParamsT<T>& P, const E2DBlock* B, int side, int k, double t,
                                              const T* ghost_recon, const T* own_face, T* o) {
  const double *gd, *fd;
  int kind = side_kind_at(B, side, k, t, gd, fd);
  if (kind == E2D_SIDE_NEIGHBOR || kind == E2D_SIDE_COPY) {
    o[0] = ghost_recon[0]; o[1] = ghost_recon[1]; o[2] = ghost_recon[2]; o[3] = ghost_recon[3];
  } else if (kind == E2D_SIDE_DIRICHLET) {
    o[0] = T(fd[0]); o[1] = T(fd[1]); o[2] = T(fd[2]); o[3] = T(fd[3]);
  } else {
    o[0] = own_face[0]; o[1] = own_face[1]; o[2] = own_face[2]; o[3] = own_face[3];
    if (kind == E2D_SIDE_REFLECT) {
      T c, s;
      boundary_cs(P, B, side, k, c, s);
      reflect(o, c, s);
    }
  }
}

// --------------------------------------------------------------------------------------
// Per-cell and per-face pieces shared by the split stage kernels (k_reconstruct, k_flux,
// k_update) and the fused stage kernel (e2d_fused.cuh), so both forms evaluate the same
// expressions.
// --------------------------------------------------------------------------------------

// Geometry one cell's reconstruction reads: L cos and L sin of its four faces, 1/A and
// the face points' offsets from the centroid (E, W, N, S).
template <typename T>
struct CellGeo {
  T LcE, LsE, LcW, LsW, LcN, LsN, LcS, LsS, ia;
  T hx[4], hy[4];
};

// by the cell's index c, its west face fW and south face fS in a block nx cells wide.
// AXG (the FP32 form on a block it takes as Cartesian): the cross-axis components are
// not read, of the normals (L sin of vertical faces, L cos of horizontal ones, below
// 2^-24 of L) and of the face points' offsets from the centroid (y of the east and
// west points, x of the north and south ones: on such a cell below 2^-24 of its
// width); the gradient and the face differences leave their terms out (limit_cell4).
// Kernels that choose that form per block at run time load every component.
template <typename T, bool AXG = false>
__device__ __forceinline__ void load_cell_geo_at(const ParamsT<T>& P, int64_t c, int64_t fW, int64_t fS, int nx,
                                                 CellGeo<T>& g) {
  const int64_t fE = fW + 1, fN = fS + nx;
  g.LcE = P.geo.vface[E2D_F_LC][fE];
  g.LcW = P.geo.vface[E2D_F_LC][fW];
  g.LsN = P.geo.hface[E2D_F_LS][fN];
  g.LsS = P.geo.hface[E2D_F_LS][fS];
  if constexpr (AXG) {
    g.LsE = g.LsW = g.LcN = g.LcS = T(0);
  } else {
    g.LsE = P.geo.vface[E2D_F_LS][fE];
    g.LsW = P.geo.vface[E2D_F_LS][fW];
    g.LcN = P.geo.hface[E2D_F_LC][fN];
    g.LcS = P.geo.hface[E2D_F_LC][fS];
  }
  g.ia = P.geo.cell[E2D_G_INV_A][c];
  g.hx[E2D_E] = P.geo.cell[E2D_G_HX_E][c];
  g.hx[E2D_W] = P.geo.cell[E2D_G_HX_W][c];
  g.hy[E2D_N] = P.geo.cell[E2D_G_HY_N][c];
  g.hy[E2D_S] = P.geo.cell[E2D_G_HY_S][c];
  if constexpr (AXG) {
    g.hy[E2D_E] = g.hy[E2D_W] = g.hx[E2D_N] = g.hx[E2D_S] = T(0);
  } else {
    g.hy[E2D_E] = P.geo.cell[E2D_G_HY_E][c];
    g.hy[E2D_W] = P.geo.cell[E2D_G_HY_W][c];
    g.hx[E2D_N] = P.geo.cell[E2D_G_HX_N][c];
    g.hx[E2D_S] = P.geo.cell[E2D_G_HX_S][c];
  }
}
template <typename T>
__device__ __forceinline__ void load_cell_geo(const ParamsT<T>& P, const E2DBlock* B, int i, int j, CellGeo<T>& g) {
  load_cell_geo_at<T>(P, cell_at(B, i, j), vf_at(B, i, j), hf_at(B, i, j), B->nx, g);
}

// FP32 form: the limiter value of one variable at one cell from its five-point
// stencil and its four unlimited face differences hot (E, W, N, S): every face's
// slope from the reciprocal approximation (slope32), psi only at the smallest and, for
// the limiters with a maximum, the largest of them (the functions are unimodal:
// psi_has_peak), a negative value clipped to 0.
template <int LIM>
__device__ __forceinline__ float phi32(float w0, float we, float ea, float so, float no, const float (&hot)[4]) {
  const float dmax = vmax(vmax(vmax(vmax(w0, we), ea), so), no) - w0;
  const float dmin = vmin(vmin(vmin(vmin(w0, we), ea), so), no) - w0;
  // FP64's round trip (w0 + hot) - w0 is hot itself unless |hot| is below half an FP64
  // ulp of w0, where it is zero and the slope takes its davg == 0 branch (psi(1)).  In
  // FP32 the same round trip would zero every |hot| below 2^-25 |w0| and switch
  // branches where the FP64 path does not, so the FP32 form applies the FP64
  // threshold, 2^-53 times the power of two of w0.
  const float half_ulp64 = __int_as_float(__float_as_int(w0) & 0x7f800000) * 1.1102230246251565e-16f;
  const float floor = fmaxf(half_ulp64, FLOAT_TRUE_MIN);
  float smin = 0.f, smax = 0.f;
#pragma unroll
  for (int s = 0; s < 4; ++s) {
    const float sl = slope32(dmax, dmin, hot[s], floor);
    smin = (s == 0) ? sl : vmin(smin, sl);
    smax = (s == 0) ? sl : vmax(smax, sl);
  }
  float ph;
  if constexpr (psi_has_peak<LIM>()) ph = psi_min_pair<LIM>(smin, smax);
  else ph = psi_s<LIM>(smin);
  return is_neg(ph) ? 0.f : ph;
}

// Green-Gauss gradient, limiter value and the limited face states fv (E, W, N, S) of
// one variable at one cell from its five-point stencil (reconstruction variables).
template <typename T, int LIM>
__device__ __forceinline__ void limit_cell_var(T w0, T we, T ea, T so, T no, const CellGeo<T>& g, T (&fv)[4],
                                               T& gx_out, T& gy_out, T& ph_out) {
  // interface averages (quad_block.py:181-218) and Green-Gauss (greengauss.py:137-155)
  const T ie = half(w0 + ea), iw = half(we + w0);
  const T in = half(w0 + no), is = half(so + w0);
  // ((ie LcE + iw (-LcW)) + in LcN) + is (-LcS), times 1/A
  const T gx = fmaT(is, -g.LcS, fmaT(in, g.LcN, fmaT(ie, g.LcE, iw * (-g.LcW)))) * g.ia;
  const T gy = fmaT(is, -g.LsS, fmaT(in, g.LsN, fmaT(ie, g.LsE, iw * (-g.LsW)))) * g.ia;
  // limiter (limiters/base.py:47-221)
  T hot[4];
  T ph = T(0);
  if constexpr (sizeof(T) == 8) {
    const T dmax = vmax(vmax(vmax(vmax(w0, we), ea), so), no) - w0;
    const T dmin = vmin(vmin(vmin(vmin(w0, we), ea), so), no) - w0;
    // FP64: psi only at the faces that decide the minimum (e2d_slope_pick.cuh); all
    // four when the pick cannot rule a face out.  Same expressions, same phi.
    double davg[4];
#pragma unroll
    for (int s = 0; s < 4; ++s) {
      hot[s] = fmaT(gx, g.hx[s], gy * g.hy[s]);
      davg[s] = (w0 + hot[s]) - w0;
    }
    const SlopePick k = pick_slopes<LIM>(dmax, dmin, davg);
    if (k.ok) {
      ph = psi_s<LIM>(k.ga ? qdiv(k.na, k.da) : T(1));
      if (k.second) ph = vmin(ph, psi_s<LIM>(k.gb ? qdiv(k.nb, k.db) : T(1)));
    } else {
#pragma unroll
      for (int s = 0; s < 4; ++s) {
        const bool pos = is_pos(davg[s]), neg = is_neg(davg[s]);
        const T p = psi_s<LIM>((pos || neg) ? qdiv(pos ? dmax : dmin, davg[s]) : T(1));
        ph = (s == 0) ? p : vmin(ph, p);
      }
    }
  } else {
#pragma unroll
    for (int s = 0; s < 4; ++s) hot[s] = fmaT(gx, g.hx[s], gy * g.hy[s]);
    ph = phi32<LIM>(w0, we, ea, so, no, hot);
  }
  ph = is_neg(ph) ? T(0) : ph;
#pragma unroll
  for (int s = 0; s < 4; ++s) fv[s] = fmaT(ph, hot[s], w0);
  gx_out = gx;
  gy_out = gy;
  ph_out = ph;
}

// The four variables of one cell: face[s][v] the limited state of side s (E, W, N, S),
// gx/gy/ph the gradient and limiter value of variable v.  st(v, p) is variable v's
// stencil value at point p (0 the cell, 1 its west, 2 east, 3 south, 4 north
// neighbour).  FP32 evaluates the interface averages, gradients, face differences and
// face states of two variables at a time in paired instructions (same values).  AXG
// (FP32 only): on a block the FP32 form takes as Cartesian, the gradient without the
// normals' cross-axis terms, (ie LcE - iw LcW) / A and (in LsN - is LsS) / A, and the
// face differences without the offsets' cross-axis terms, gx hx at the east and west
// points and gy hy at the north and south ones; axg chooses that form at run time
// (one limiter body, the shorter sums selected).
template <typename T, int LIM, bool AXG = false, typename Stencil>
__device__ __forceinline__ void limit_cell4(const Stencil& st, const CellGeo<T>& g, T (&face)[4][4], T (&gx)[4],
                                            T (&gy)[4], T (&ph)[4], bool axg = false) {
  static_assert(!AXG || sizeof(T) == 4, "the FP64 path keeps every term");
  if constexpr (sizeof(T) == 8) {
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      T fv[4];
      limit_cell_var<T, LIM>(st(v, 0), st(v, 1), st(v, 2), st(v, 3), st(v, 4), g, fv, gx[v], gy[v], ph[v]);
#pragma unroll
      for (int s = 0; s < 4; ++s) face[s][v] = fv[s];
    }
  } else {
    const float2 H = pair(0.5f, 0.5f);
    const float2 LcE = pair(g.LcE, g.LcE), nLcW = pair(-g.LcW, -g.LcW), LcN = pair(g.LcN, g.LcN),
                 nLcS = pair(-g.LcS, -g.LcS), LsE = pair(g.LsE, g.LsE), nLsW = pair(-g.LsW, -g.LsW),
                 LsN = pair(g.LsN, g.LsN), nLsS = pair(-g.LsS, -g.LsS), IA = pair(g.ia, g.ia);
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int a = 2 * q, b = 2 * q + 1;
      const float2 w0 = pair(st(a, 0), st(b, 0)), we = pair(st(a, 1), st(b, 1)), ea = pair(st(a, 2), st(b, 2)),
                   so = pair(st(a, 3), st(b, 3)), no = pair(st(a, 4), st(b, 4));
      // the scalar form's expressions (limit_cell_var), lane by lane
      const float2 ie = mul2(H, add2(w0, ea)), iw = mul2(H, add2(we, w0));
      const float2 in = mul2(H, add2(w0, no)), is = mul2(H, add2(so, w0));
      const bool ax = AXG || axg;
      const float2 sx = fma2(ie, LcE, mul2(iw, nLcW));
      const float2 gxp = mul2(ax ? sx : fma2(is, nLcS, fma2(in, LcN, sx)), IA);
      const float2 sy = ax ? mul2(in, LsN) : fma2(in, LsN, fma2(ie, LsE, mul2(iw, nLsW)));
      const float2 gyp = mul2(fma2(is, nLsS, sy), IA);
      float2 hot[4];
      float ha[4], hb[4];
#pragma unroll
      for (int s = 0; s < 4; ++s) {
        const float2 hx = pair(g.hx[s], g.hx[s]), hy = pair(g.hy[s], g.hy[s]);
        hot[s] = ax ? (s == E2D_E || s == E2D_W ? mul2(gxp, hx) : mul2(gyp, hy)) : fma2(gxp, hx, mul2(gyp, hy));
        ha[s] = hot[s].x;
        hb[s] = hot[s].y;
      }
      const float pa = phi32<LIM>(w0.x, we.x, ea.x, so.x, no.x, ha);
      const float pb = phi32<LIM>(w0.y, we.y, ea.y, so.y, no.y, hb);
      const float2 php = pair(pa, pb);
#pragma unroll
      for (int s = 0; s < 4; ++s) {
        const float2 f = fma2(php, hot[s], w0);
        face[s][a] = f.x;
        face[s][b] = f.y;
      }
      gx[a] = gxp.x; gx[b] = gxp.y;
      gy[a] = gyp.x; gy[b] = gyp.y;
      ph[a] = pa; ph[b] = pb;
    }
  }
}

// A face state (reconstruction variables) rotated into the frame of vertical face f
// and converted to primitive variables (fvm/base.py:327-390).
template <typename T, int RECON>
__device__ __forceinline__ void vface_prim_cs(const Gas<T>& G, bool cart, T c, T s, const T* in, T* w) {
  T q[4] = {in[0], in[1], in[2], in[3]};
  if (!cart) rotate(q, c, s);
  recon_to_prim<RECON>(q, G, w);
}
template <typename T, int RECON>
__device__ __forceinline__ void vface_prim(const ParamsT<T>& P, const Gas<T>& G, bool cart, int64_t f, const T* in,
                                           T* w) {
  vface_prim_cs<T, RECON>(G, cart, cart ? T(1) : P.geo.vface[E2D_F_COS][f], cart ? T(0) : P.geo.vface[E2D_F_SIN][f],
                          in, w);
}
// the same for horizontal face f (the y sweep in the x frame, fvm/base.py:392-486)
template <typename T, int RECON>
__device__ __forceinline__ void hface_prim_cs(const Gas<T>& G, bool cart, T c, T s, const T* in, T* w) {
  T q[4] = {in[0], in[1], in[2], in[3]};
  if (cart) rotate90(q);
  else rotate(q, c, s);
  recon_to_prim<RECON>(q, G, w);
}
template <typename T, int RECON>
__device__ __forceinline__ void hface_prim(const ParamsT<T>& P, const Gas<T>& G, bool cart, int64_t f, const T* in,
                                           T* w) {
  hface_prim_cs<T, RECON>(G, cart, cart ? T(0) : P.geo.hface[E2D_F_COS][f], cart ? T(1) : P.geo.hface[E2D_F_SIN][f],
                          in, w);
}

// Riemann flux of vertical face f in its frame, rotated back and integrated with the
// one-point rule (I = L * 2 F); DBG records the raw and rotated-back fluxes.
template <typename T, int FLUX, bool DBG>
__device__ __forceinline__ void vface_flux(const ParamsT<T>& P, const Gas<T>& G, bool cart, int64_t f, const T* L,
                                           const T* R, T* I, const DebugOutT<T>& dbg) {
  T Fx[4];
  riemann<FLUX>(L, R, G, Fx);
  if (DBG && dbg.vflux_raw) store4(dbg.vflux_raw, P.nvface, f, Fx);
  if (!cart) unrotate(Fx, P.geo.vface[E2D_F_COS][f], P.geo.vface[E2D_F_SIN][f]);
  if (DBG && dbg.vflux) store4(dbg.vflux, P.nvface, f, Fx);
  const T len = P.geo.vface[E2D_F_L][f];
  I[0] = len * twice(Fx[0]); I[1] = len * twice(Fx[1]); I[2] = len * twice(Fx[2]); I[3] = len * twice(Fx[3]);
}
template <typename T, int FLUX, bool DBG>
__device__ __forceinline__ void hface_flux(const ParamsT<T>& P, const Gas<T>& G, bool cart, int64_t f, const T* L,
                                           const T* R, T* I, const DebugOutT<T>& dbg) {
  T Fy[4];
  riemann<FLUX>(L, R, G, Fy);
  if (DBG && dbg.hflux_raw) store4(dbg.hflux_raw, P.nhface, f, Fy);
  if (cart) unrotate90(Fy);
  else unrotate(Fy, P.geo.hface[E2D_F_COS][f], P.geo.hface[E2D_F_SIN][f]);
  if (DBG && dbg.hflux) store4(dbg.hflux, P.nhface, f, Fy);
  const T len = P.geo.hface[E2D_F_L][f];
  I[0] = len * twice(Fy[0]); I[1] = len * twice(Fy[1]); I[2] = len * twice(Fy[2]); I[3] = len * twice(Fy[3]);
}

// dUdt of one variable of a cell from its integrated face fluxes, area A and 1/A
// (fvm/base.py:171-190): 0.5 * (((I_W - I_E) + I_S) - I_N) / A.  FP64 divides with the
// geometry's correctly rounded 1/A (div_recip: the IEEE quotient); the FP32 form by
// the (positive, normal) area with rdiv.
template <typename T>
__device__ __forceinline__ T cell_dudt(T IW, T IE, T IS, T IN, T A, T iA) {
  if constexpr (sizeof(T) == 4) return rdiv(half(IW - IE + IS - IN), A);
  else return div_recip(half(IW - IE + IS - IN), A, iA);
}

// The RK stage program at cell c: every partial Butcher sum this stage contributes
// to, dst = src + (dt a) k, or on the FP32 path the last row's increment added to U^n
// with Kahan compensation carried across steps.  Each update's loads wait behind the
// previous update's stores (the buffers are plain pointers); loading every source
// first was measured slower in both the split and the fused kernel: the values held
// across the stores cost registers, and so occupancy or spills.
// NU bounds the updates a stage has (the loop is unrolled NU times; programs of the
// explicit tableaux up to RK4 have at most two per stage).
template <typename T, int NU = MAX_STAGES>
__device__ __forceinline__ void stage_program(const ParamsT<T>& P, const StateBuffersT<T>& S, const StageProgram& prog,
                                              double dt, int64_t c, const T* k) {
#pragma unroll
  for (int u = 0; u < NU; ++u) {  // unrolled: the program is read from kernel parameters
    if (u >= prog.nupd) break;
    const StageUpdate& up = prog.upd[u];
    const T* src = static_cast<const T*>(up.srcp);
    const T dta = T(dt * up.a);
    T base[4];
#pragma unroll
    for (int v = 0; v < 4; ++v) base[v] = up.src_zero ? T(0) : src[v * P.ncell + c];
    if (!up.kahan) {
      T* dst = static_cast<T*>(up.dstp);
#pragma unroll
      for (int v = 0; v < 4; ++v) dst[v * P.ncell + c] = fmaT(dta, k[v], base[v]);
    } else {
      // U^{n+1} = U^n + increment with Kahan compensation carried across steps
      T* U0 = S.buf[0];
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        const T inc = fmaT(dta, k[v], base[v]);
        const T cmp = S.comp[v * P.ncell + c], u0 = U0[v * P.ncell + c];
        const T y = inc - cmp;
        const T tt = u0 + y;
        S.comp[v * P.ncell + c] = (tt - u0) - y;
        U0[v * P.ncell + c] = tt;
      }
    }
  }
}

// --------------------------------------------------------------------------------------
// K1: reconstruction
// --------------------------------------------------------------------------------------

// One tile of cells: the body of k_reconstruct.  Returns early (uniformly per CTA)
// for an inactive instance; the caller synchronises before sW is refilled.
//
// A TMA wait that runs out is counted in tma.timeouts (the host then reports the
// step as failed, and the state it produced is not to be used).  The CTA waits once
// more, as long again, for the copy in flight: if it lands, sW is the CTA's again and
// later tiles take plain loads (tma_live = false); if it does not, the CTA sets
// `abandon` and the caller stops, so nothing writes sW while the copy may still be
// writing it.
template <typename T, int LIM, int RECON, bool DBG, int RTY>
__device__ __forceinline__ void reconstruct_tile(const ParamsT<T>& P, const int4 tl, const T* __restrict__ U,
                                                 const InstanceState* __restrict__ inst, const FaceArraysT<T>& F,
                                                 const DebugOutT<T>& dbg,
                                                 T (&sW)[4][RTY + 2][TileCols<T>::TXW], const TmaTiles& tma,
                                                 unsigned long long* bar, unsigned& phase, bool& tma_live,
                                                 bool& abandon) {
  constexpr int C0 = TileCols<T>::C0;
  const Gas<T> G{P.gas[0], P.gas[1], P.gas[2], P.gas[3]};
  const E2DBlock* B = P.blocks + tl.x;
  const InstanceState* I = inst + B->instance;
  if (!I->active) return;
  const double t = I->t;
  const int nx = B->nx, ny = B->ny;
  const int i0 = tl.y, j0 = tl.z;
  // A tile whose halo lies inside the block needs no ghost cell and owns no block-
  // boundary face.  The test is uniform over the CTA, so interior tiles branch past
  // the ghost and boundary code instead of issuing it under predicates.
  const bool edge = i0 == 0 || j0 == 0 || i0 + RTY >= ny || j0 + TX >= nx;
  // Interior tiles of blocks with a tensor map arrive by one TMA box load (the tile, its
  // halo and the alignment columns, 4 planes); the test is uniform over the CTA.
  if (!edge && tma_live && tma.maps != nullptr && tma.ok[tl.x]) {
    if (threadIdx.x == 0)
      tma_load_box(&sW[0][0][0], &tma.maps[tl.x], j0 - TileCols<T>::XO, i0 - 1, 0, bar, (unsigned)sizeof(sW));
    const bool arrived = __syncthreads_and(mbar_wait(bar, phase));
    if (!arrived) {  // a wait ran out: report it, wait once more for the copy in flight, drop the tile
      if (threadIdx.x == 0) atomicAdd(tma.timeouts, 1ULL);
      const bool landed = __syncthreads_and(mbar_wait(bar, phase));
      phase ^= 1u;
      tma_live = false;
      abandon = !landed;  // uniform over the CTA
      return;
    }
    phase ^= 1u;
    if (RECON == E2D_RECON_PRIMITIVE) {  // conversion in place, one thread per staged cell
      for (int p = threadIdx.x; p < (RTY + 2) * (TX + 2); p += TX * RTY) {
        const int ly = p / (TX + 2), lx = p - ly * (TX + 2);
        T q[4] = {sW[0][ly][C0 + lx], sW[1][ly][C0 + lx], sW[2][ly][C0 + lx], sW[3][ly][C0 + lx]}, r[4];
        to_recon<RECON>(q, G, r);
        sW[0][ly][C0 + lx] = r[0];
        sW[1][ly][C0 + lx] = r[1];
        sW[2][ly][C0 + lx] = r[2];
        sW[3][ly][C0 + lx] = r[3];
      }
    }
  } else
  for (int p = threadIdx.x; p < (RTY + 2) * (TX + 2); p += TX * RTY) {

    const int ly = p / (TX + 2), lx = p - ly * (TX + 2);
    const int gi = i0 + ly - 1, gj = j0 + lx - 1;
    T q[4], r[4] = {T(0), T(0), T(0), T(0)};
    if (!edge) {
      load_cell(U, P.ncell, cell_at(B, gi, gj), q);
      to_recon<RECON>(q, G, r);
    } else {
      const bool in_i = gi >= 0 && gi < ny, in_j = gj >= 0 && gj < nx;
      bool ok = true;
      if (in_i && in_j) load_cell(U, P.ncell, cell_at(B, gi, gj), q);
      else if (in_i && gj == -1) ghost_cons(P, B, E2D_W, gi, U, t, q);
      else if (in_i && gj == nx) ghost_cons(P, B, E2D_E, gi, U, t, q);
      else if (in_j && gi == -1) ghost_cons(P, B, E2D_S, gj, U, t, q);
      else if (in_j && gi == ny) ghost_cons(P, B, E2D_N, gj, U, t, q);
      else ok = false;
      if (ok) to_recon<RECON>(q, G, r);
    }
    sW[0][ly][C0 + lx] = r[0];
    sW[1][ly][C0 + lx] = r[1];
    sW[2][ly][C0 + lx] = r[2];
    sW[3][ly][C0 + lx] = r[3];
  }
  __syncthreads();

  const int ty = threadIdx.x / TX, tx = threadIdx.x - (threadIdx.x / TX) * TX;
  const int i = i0 + ty, j = j0 + tx;
  if (i >= ny || j >= nx) return;
  const int64_t c = cell_at(B, i, j);
  const int64_t fE = vf_at(B, i, j + 1), fW = vf_at(B, i, j);
  const int64_t fN = hf_at(B, i + 1, j), fS = hf_at(B, i, j);
  // the FP32 form on a block it takes as Cartesian: the gradient and the face
  // differences without cross-axis terms (as the fused kernel computes them)
  const bool axg = sizeof(T) == 4 && block_cart(P, B, tl.x);
  CellGeo<T> g;
  load_cell_geo(P, B, i, j, g);

  T face[4][4];  // [side][var] limited face states, reconstruction variables
  {
    // stencil points: the cell, W, E, S, N
    auto st = [&](int v, int p) -> T {
      return sW[v][ty + 1 + (p == 3 ? -1 : p == 4 ? 1 : 0)][C0 + tx + 1 + (p == 1 ? -1 : p == 2 ? 1 : 0)];
    };
    T gx[4], gy[4], ph[4];
    limit_cell4<T, LIM, false>(st, g, face, gx, gy, ph, axg);
    if (DBG) {
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        if (dbg.gx) dbg.gx[v * P.ncell + c] = gx[v];
        if (dbg.gy) dbg.gy[v * P.ncell + c] = gy[v];
        if (dbg.phi) dbg.phi[v * P.ncell + c] = ph[v];
      }
    }
  }

  const bool cart = block_cart(P, B, tl.x);
  // the four face frames, read before the first store of a face state (a load after a
  // store through these plain pointers would wait for it)
  T fc[4] = {T(1), T(1), T(0), T(0)}, fs[4] = {T(0), T(0), T(1), T(1)};
  if (!cart) {
    fc[0] = P.geo.vface[E2D_F_COS][fE]; fs[0] = P.geo.vface[E2D_F_SIN][fE];
    fc[1] = P.geo.vface[E2D_F_COS][fW]; fs[1] = P.geo.vface[E2D_F_SIN][fW];
    fc[2] = P.geo.hface[E2D_F_COS][fN]; fs[2] = P.geo.hface[E2D_F_SIN][fN];
    fc[3] = P.geo.hface[E2D_F_COS][fS]; fs[3] = P.geo.hface[E2D_F_SIN][fS];
  }
  T w[4];
  vface_prim_cs<T, RECON>(G, cart, fc[0], fs[0], face[E2D_E], w);  // east face = left state of vertical face j+1
  store4(F.vL, P.nvface, fE, w);
  vface_prim_cs<T, RECON>(G, cart, fc[1], fs[1], face[E2D_W], w);  // west face = right state of vertical face j
  store4(F.vR, P.nvface, fW, w);
  hface_prim_cs<T, RECON>(G, cart, fc[2], fs[2], face[E2D_N], w);  // north face = left state of horizontal face i+1
  store4(F.hL, P.nhface, fN, w);
  hface_prim_cs<T, RECON>(G, cart, fc[3], fs[3], face[E2D_S], w);  // south face = right state of horizontal face i
  store4(F.hR, P.nhface, fS, w);
  // outside states of block-boundary faces
  if (!edge) return;
  if (j == 0) {
    const T gr[4] = {sW[0][ty + 1][C0 + tx], sW[1][ty + 1][C0 + tx], sW[2][ty + 1][C0 + tx], sW[3][ty + 1][C0 + tx]};
    T o[4];
    outside_state(P, B, E2D_W, i, t, gr, face[E2D_W], o);
    vface_prim<T, RECON>(P, G, cart, fW, o, w);
    store4(F.vL, P.nvface, fW, w);
  }
  if (j == nx - 1) {
    const T gr[4] = {sW[0][ty + 1][C0 + tx + 2], sW[1][ty + 1][C0 + tx + 2], sW[2][ty + 1][C0 + tx + 2],
                     sW[3][ty + 1][C0 + tx + 2]};
    T o[4];
    outside_state(P, B, E2D_E, i, t, gr, face[E2D_E], o);
    vface_prim<T, RECON>(P, G, cart, fE, o, w);
    store4(F.vR, P.nvface, fE, w);
  }
  if (i == 0) {
    const T gr[4] = {sW[0][ty][C0 + tx + 1], sW[1][ty][C0 + tx + 1], sW[2][ty][C0 + tx + 1], sW[3][ty][C0 + tx + 1]};
    T o[4];
    outside_state(P, B, E2D_S, j, t, gr, face[E2D_S], o);
    hface_prim<T, RECON>(P, G, cart, fS, o, w);
    store4(F.hL, P.nhface, fS, w);
  }
  if (i == ny - 1) {
    const T gr[4] = {sW[0][ty + 2][C0 + tx + 1], sW[1][ty + 2][C0 + tx + 1], sW[2][ty + 2][C0 + tx + 1],
                     sW[3][ty + 2][C0 + tx + 1]};
    T o[4];
    outside_state(P, B, E2D_N, j, t, gr, face[E2D_N], o);
    hface_prim<T, RECON>(P, G, cart, fN, o, w);
    store4(F.hR, P.nhface, fN, w);
  }
}

// A grid of ntiles CTAs does one tile each (PERSIST false); a persistent grid of
// resident CTAs strides over the tile table.  The two forms are separate
// instantiations so the one-tile form carries no loop state in registers.
template <typename T, int LIM, int RECON, bool DBG, int RTY, int MINB, bool PERSIST>
__global__ void __launch_bounds__(TX * RTY, MINB) k_reconstruct(ParamsT<T> P, const int4* __restrict__ tiles,
                                                                int ntiles, const T* __restrict__ U,
                                                                const InstanceState* __restrict__ inst,
                                                                FaceArraysT<T> F, DebugOutT<T> dbg, TmaTiles tma) {
  __shared__ __align__(128) T sW[4][RTY + 2][TileCols<T>::TXW];
  __shared__ __align__(8) unsigned long long bar;
  unsigned phase = 0;
  bool tma_live = tma.maps != nullptr;
  bool abandon = false;
  if (tma_live) {
    if (threadIdx.x == 0) mbar_init(&bar);
    __syncthreads();
  }
  if constexpr (!PERSIST) {
    reconstruct_tile<T, LIM, RECON, DBG, RTY>(P, tiles[blockIdx.x], U, inst, F, dbg, sW, tma, &bar, phase, tma_live,
                                              abandon);
  } else {
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
      reconstruct_tile<T, LIM, RECON, DBG, RTY>(P, tiles[tile], U, inst, F, dbg, sW, tma, &bar, phase, tma_live,
                                                abandon);
      if (abandon) break;  // a copy may still be writing sW: no further tile touches it
      __syncthreads();  // the next tile refills sW
    }
  }
}

// --------------------------------------------------------------------------------------
// K1 with 2 or 3 face quadrature points (SolverConfig.fvm_num_quadrature_points,
// pyhype/mesh/quadratures.py:33-90, fvm/SecondOrderMUSCL.py:128-158): the high-order
// term is evaluated at every point of every face, the limiter takes the minimum over
// the E, W, N, S points in that order (limiters/base.py:147-187), and a limited state
// is written per point (face-array plane offset 4q).  The high-order term is formed
// once for the limiter and once more for the face state, by the same expression.
// --------------------------------------------------------------------------------------
template <typename T, int LIM, int RECON, int NQP>
__global__ void __launch_bounds__(TX * TY) k_reconstruct_qp(ParamsT<T> P, const int4* __restrict__ tiles,
                                                            const T* __restrict__ U,
                                                            const InstanceState* __restrict__ inst,
                                                            FaceArraysT<T> F) {
  __shared__ T sW[4][TY + 2][TX + 2];
  const Gas<T> G{P.gas[0], P.gas[1], P.gas[2], P.gas[3]};
  const int4 tl = tiles[blockIdx.x];
  const E2DBlock* B = P.blocks + tl.x;
  const InstanceState* I = inst + B->instance;
  if (!I->active) return;
  const double t = I->t;
  const int nx = B->nx, ny = B->ny;
  const int i0 = tl.y, j0 = tl.z;
  const bool edge = i0 == 0 || j0 == 0 || i0 + TY >= ny || j0 + TX >= nx;  // as in reconstruct_tile
  for (int p = threadIdx.x; p < (TY + 2) * (TX + 2); p += TX * TY) {
    const int ly = p / (TX + 2), lx = p - ly * (TX + 2);
    const int gi = i0 + ly - 1, gj = j0 + lx - 1;
    T q[4], r[4] = {T(0), T(0), T(0), T(0)};
    if (!edge) {
      load_cell(U, P.ncell, cell_at(B, gi, gj), q);
      to_recon<RECON>(q, G, r);
    } else {
      const bool in_i = gi >= 0 && gi < ny, in_j = gj >= 0 && gj < nx;
      bool ok = true;
      if (in_i && in_j) load_cell(U, P.ncell, cell_at(B, gi, gj), q);
      else if (in_i && gj == -1) ghost_cons(P, B, E2D_W, gi, U, t, q);
      else if (in_i && gj == nx) ghost_cons(P, B, E2D_E, gi, U, t, q);
      else if (in_j && gi == -1) ghost_cons(P, B, E2D_S, gj, U, t, q);
      else if (in_j && gi == ny) ghost_cons(P, B, E2D_N, gj, U, t, q);
      else ok = false;
      if (ok) to_recon<RECON>(q, G, r);
    }
    sW[0][ly][lx] = r[0];
    sW[1][ly][lx] = r[1];
    sW[2][ly][lx] = r[2];
    sW[3][ly][lx] = r[3];
  }
  __syncthreads();

  const int ty = threadIdx.x / TX, tx = threadIdx.x - (threadIdx.x / TX) * TX;
  const int i = i0 + ty, j = j0 + tx;
  if (i >= ny || j >= nx) return;
  const int64_t c = cell_at(B, i, j);
  const int64_t fE = vf_at(B, i, j + 1), fW = vf_at(B, i, j);
  const int64_t fN = hf_at(B, i + 1, j), fS = hf_at(B, i, j);
  const T LcE = P.geo.vface[E2D_F_LC][fE], LsE = P.geo.vface[E2D_F_LS][fE];
  const T LcW = P.geo.vface[E2D_F_LC][fW], LsW = P.geo.vface[E2D_F_LS][fW];
  const T LcN = P.geo.hface[E2D_F_LC][fN], LsN = P.geo.hface[E2D_F_LS][fN];
  const T LcS = P.geo.hface[E2D_F_LC][fS], LsS = P.geo.hface[E2D_F_LS][fS];
  const T ia = P.geo.cell[E2D_G_INV_A][c];

  T gxs[4], gys[4], phs[4];
#pragma unroll
  for (int v = 0; v < 4; ++v) {
    const T w0 = sW[v][ty + 1][tx + 1];
    const T we = sW[v][ty + 1][tx];
    const T ea = sW[v][ty + 1][tx + 2];
    const T so = sW[v][ty][tx + 1];
    const T no = sW[v][ty + 2][tx + 1];
    const T ie = half(w0 + ea), iw = half(we + w0);
    const T in = half(w0 + no), is = half(so + w0);
    const T gx = fmaT(is, -LcS, fmaT(in, LcN, fmaT(ie, LcE, iw * (-LcW)))) * ia;
    const T gy = fmaT(is, -LsS, fmaT(in, LsN, fmaT(ie, LsE, iw * (-LsW)))) * ia;
    const T dmax = vmax(vmax(vmax(vmax(w0, we), ea), so), no) - w0;
    const T dmin = vmin(vmin(vmin(vmin(w0, we), ea), so), no) - w0;
    T ph = T(0);
    T dv[4 * NQP];  // davg of every point, E points first, then W, N, S
#pragma unroll
    for (int s = 0; s < 4; ++s)
#pragma unroll
      for (int q = 0; q < NQP; ++q) {
        const T hot = fmaT(gx, P.geo.qp[q][s][c], gy * P.geo.qp[q][4 + s][c]);
        if constexpr (sizeof(T) == 4) {
          const T half_ulp64 = __int_as_float(__float_as_int(w0) & 0x7f800000) * T(1.1102230246251565e-16);
          dv[s * NQP + q] = (fabs(hot) < half_ulp64) ? T(0) : hot;
        } else {
          dv[s * NQP + q] = (w0 + hot) - w0;
        }
      }
    bool done = false;
    if constexpr (sizeof(T) == 8) {  // psi only at the points that decide phi, as k_reconstruct does
      const SlopePick k = pick_slopes<LIM, 4 * NQP>(dmax, dmin, dv);
      if (k.ok) {
        ph = psi_s<LIM>(k.ga ? qdiv(k.na, k.da) : T(1));
        if (k.second) ph = vmin(ph, psi_s<LIM>(k.gb ? qdiv(k.nb, k.db) : T(1)));
        done = true;
      }
    }
    if (!done) {
#pragma unroll
      for (int m = 0; m < 4 * NQP; ++m) {
        const T davg = dv[m];
        const bool pos = is_pos(davg), neg = is_neg(davg);
        const T sl = (pos || neg) ? qdiv(pos ? dmax : dmin, davg) : T(1);
        const T p = psi_s<LIM>(sl);
        ph = (m == 0) ? p : vmin(ph, p);
      }
    }
    phs[v] = is_neg(ph) ? T(0) : ph;
    gxs[v] = gx;
    gys[v] = gy;
  }

  const bool cart = block_cart(P, B, tl.x);
#pragma unroll
  for (int s = 0; s < 4; ++s)
#pragma unroll
    for (int q = 0; q < NQP; ++q) {
      T fq[4];
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        const T hot = fmaT(gxs[v], P.geo.qp[q][s][c], gys[v] * P.geo.qp[q][4 + s][c]);
        fq[v] = fmaT(phs[v], hot, sW[v][ty + 1][tx + 1]);
      }
      const bool vert = s == E2D_E || s == E2D_W;
      const int64_t f = s == E2D_E ? fE : s == E2D_W ? fW : s == E2D_N ? fN : fS;
      const T fc = vert ? P.geo.vface[E2D_F_COS][f] : P.geo.hface[E2D_F_COS][f];
      const T fs = vert ? P.geo.vface[E2D_F_SIN][f] : P.geo.hface[E2D_F_SIN][f];
      const int64_t stride = vert ? P.nvface : P.nhface;
      // this cell's own face state: left state of its E/N face, right state of W/S
      {
        T qv[4] = {fq[0], fq[1], fq[2], fq[3]}, w[4];
        if (vert) {
          if (!cart) rotate(qv, fc, fs);
        } else {
          if (cart) rotate90(qv);
          else rotate(qv, fc, fs);
        }
        recon_to_prim<RECON>(qv, G, w);
        T* dst = s == E2D_E ? F.vL : s == E2D_W ? F.vR : s == E2D_N ? F.hL : F.hR;
        store4(dst + (int64_t)q * 4 * stride, stride, f, w);
      }
      // the outside state of a block-boundary face, for this point
      const bool at = s == E2D_E ? j == nx - 1 : s == E2D_W ? j == 0 : s == E2D_N ? i == ny - 1 : i == 0;
      if (edge && at) {
        T gr[4];
#pragma unroll
        for (int v = 0; v < 4; ++v)
          gr[v] = s == E2D_E ? sW[v][ty + 1][tx + 2] : s == E2D_W ? sW[v][ty + 1][tx]
                : s == E2D_N ? sW[v][ty + 2][tx + 1] : sW[v][ty][tx + 1];
        T o[4], w[4];
        outside_state(P, B, s, vert ? i : j, t, gr, fq, o);
        if (vert) {
          if (!cart) rotate(o, fc, fs);
        } else {
          if (cart) rotate90(o);
          else rotate(o, fc, fs);
        }
        recon_to_prim<RECON>(o, G, w);
        T* dst = s == E2D_E ? F.vR : s == E2D_W ? F.vL : s == E2D_N ? F.hR : F.hL;
        store4(dst + (int64_t)q * 4 * stride, stride, f, w);
      }
    }
}

// K2 with 2 or 3 quadrature points: one Riemann flux per face and point, un-rotated,
// integrated as L * sum_q w_q F_q summed from zero in point order
// (pyhype/fvm/base.py:171-190).
template <typename T, int FLUX, int NQP>
__global__ void __launch_bounds__(TX * TY) k_flux_qp(ParamsT<T> P, const int4* __restrict__ tiles,
                                                     const InstanceState* __restrict__ inst, FaceArraysT<T> F) {
  const int4 tl = tiles[blockIdx.x];
  const E2DBlock* B = P.blocks + tl.x;
  if (!inst[B->instance].active) return;
  const int nx = B->nx, ny = B->ny;
  const int ty = threadIdx.x / TX, tx = threadIdx.x - (threadIdx.x / TX) * TX;
  const int i = tl.y + ty, j = tl.z + tx;
  if (i > ny || j > nx) return;
  const Gas<T> G{P.gas[0], P.gas[1], P.gas[2], P.gas[3]};
  const bool cart = block_cart(P, B, tl.x);
#pragma unroll
  for (int dir = 0; dir < 2; ++dir) {
    const bool vert = dir == 0;
    if (vert ? i >= ny : j >= nx) continue;
    const int64_t f = vert ? vf_at(B, i, j) : hf_at(B, i, j);
    const int64_t stride = vert ? P.nvface : P.nhface;
    const T* Ls = vert ? F.vL : F.hL;
    const T* Rs = vert ? F.vR : F.hR;
    const T fc = vert ? P.geo.vface[E2D_F_COS][f] : P.geo.hface[E2D_F_COS][f];
    const T fs = vert ? P.geo.vface[E2D_F_SIN][f] : P.geo.hface[E2D_F_SIN][f];
    T acc[4] = {T(0), T(0), T(0), T(0)};
#pragma unroll
    for (int q = 0; q < NQP; ++q) {
      const int64_t o = (int64_t)q * 4 * stride + f;
      T L[4] = {Ls[o], Ls[o + stride], Ls[o + 2 * stride], Ls[o + 3 * stride]};
      T R[4] = {Rs[o], Rs[o + stride], Rs[o + 2 * stride], Rs[o + 3 * stride]};
      T Fq[4];
      riemann<FLUX>(L, R, G, Fq);
      if (vert) {
        if (!cart) unrotate(Fq, fc, fs);
      } else {
        if (cart) unrotate90(Fq);
        else unrotate(Fq, fc, fs);
      }
#pragma unroll
      for (int v = 0; v < 4; ++v) acc[v] = fmaT(P.qw[q], Fq[v], acc[v]);
    }
    const T len = vert ? P.geo.vface[E2D_F_L][f] : P.geo.hface[E2D_F_L][f];
    T Iv[4] = {len * acc[0], len * acc[1], len * acc[2], len * acc[3]};
    store4(vert ? F.vI : F.hI, stride, f, Iv);
  }
}

// --------------------------------------------------------------------------------------
// K2: one Riemann flux per face
// --------------------------------------------------------------------------------------
template <typename T, int FLUX, bool DBG>
__device__ __forceinline__ void flux_tile(const ParamsT<T>& P, const int4 tl, const InstanceState* __restrict__ inst,
                                          const FaceArraysT<T>& F, const DebugOutT<T>& dbg) {
  const E2DBlock* B = P.blocks + tl.x;
  if (!inst[B->instance].active) return;
  const int nx = B->nx, ny = B->ny;
  const int ty = threadIdx.x / TX, tx = threadIdx.x - (threadIdx.x / TX) * TX;
  const int i = tl.y + ty, j = tl.z + tx;
  if (i > ny || j > nx) return;
  const Gas<T> G{P.gas[0], P.gas[1], P.gas[2], P.gas[3]};
  const bool cart = block_cart(P, B, tl.x);
  const bool hv = i < ny, hh = j < nx;
  const int64_t fv = hv ? vf_at(B, i, j) : 0, fh = hh ? hf_at(B, i, j) : 0;
  T vLs[4], vRs[4], hLs[4], hRs[4];
  if constexpr (sizeof(T) == 4) {
    // FP32 (issue- and latency-bound): both faces' states are loaded before the first
    // store (the face arrays are plain pointers: a load after a store would wait for
    // it).  FP64 is bound by its FP64 pipe, and the extra live values would spill.
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      if (hv) { vLs[v] = F.vL[v * P.nvface + fv]; vRs[v] = F.vR[v * P.nvface + fv]; }
      if (hh) { hLs[v] = F.hL[v * P.nhface + fh]; hRs[v] = F.hR[v * P.nhface + fh]; }
    }
    T Iv[4], Ih[4];
    if (hv) vface_flux<T, FLUX, DBG>(P, G, cart, fv, vLs, vRs, Iv, dbg);
    if (hh) hface_flux<T, FLUX, DBG>(P, G, cart, fh, hLs, hRs, Ih, dbg);
    if (hv) store4(F.vI, P.nvface, fv, Iv);
    if (hh) store4(F.hI, P.nhface, fh, Ih);
  } else {
    T I[4];
    if (hv) {
#pragma unroll
      for (int v = 0; v < 4; ++v) { vLs[v] = F.vL[v * P.nvface + fv]; vRs[v] = F.vR[v * P.nvface + fv]; }
      vface_flux<T, FLUX, DBG>(P, G, cart, fv, vLs, vRs, I, dbg);
      store4(F.vI, P.nvface, fv, I);
    }
    if (hh) {
#pragma unroll
      for (int v = 0; v < 4; ++v) { hLs[v] = F.hL[v * P.nhface + fh]; hRs[v] = F.hR[v * P.nhface + fh]; }
      hface_flux<T, FLUX, DBG>(P, G, cart, fh, hLs, hRs, I, dbg);
      store4(F.hI, P.nhface, fh, I);
    }
  }
}

template <typename T, int FLUX, bool DBG, int MINB, bool PERSIST>
__global__ void __launch_bounds__(TX * TY, MINB) k_flux(ParamsT<T> P, const int4* __restrict__ tiles, int ntiles,
                                                        const InstanceState* __restrict__ inst, FaceArraysT<T> F,
                                                        DebugOutT<T> dbg) {
  if constexpr (!PERSIST) {
    flux_tile<T, FLUX, DBG>(P, tiles[blockIdx.x], inst, F, dbg);
  } else {
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) flux_tile<T, FLUX, DBG>(P, tiles[tile], inst, F, dbg);
  }
}

// --------------------------------------------------------------------------------------
// K3: divergence + RK stage program (+ positivity on the last stage)
// --------------------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ void update_tile(const ParamsT<T>& P, const int4 tl, const FaceArraysT<T>& F,
                                            const StateBuffersT<T>& S, const StageProgram& prog,
                                            InstanceState* __restrict__ inst, RealizState* __restrict__ real,
                                            T* __restrict__ dudt_out) {
  const E2DBlock* B = P.blocks + tl.x;
  const InstanceState* I = inst + B->instance;
  if (!I->active) return;
  const int ty = threadIdx.x / TX, tx = threadIdx.x - (threadIdx.x / TX) * TX;
  const int i = tl.y + ty, j = tl.z + tx;
  const bool live = i < B->ny && j < B->nx;
  bool bad = false;
  int64_t c = 0;
  if (live) {
    c = cell_at(B, i, j);
    const int64_t fW = vf_at(B, i, j), fE = fW + 1;
    const int64_t fS = hf_at(B, i, j), fN = fS + B->nx;
    const T A = P.geo.cell[E2D_G_A][c];
    const T iA = sizeof(T) == 8 ? P.geo.cell[E2D_G_INV_A][c] : T(0);
    T k[4];
#pragma unroll
    for (int v = 0; v < 4; ++v)
      k[v] = cell_dudt(F.vI[v * P.nvface + fW], F.vI[v * P.nvface + fE], F.hI[v * P.nhface + fS],
                       F.hI[v * P.nhface + fN], A, iA);
    if (dudt_out) {
#pragma unroll
      for (int v = 0; v < 4; ++v) dudt_out[v * P.ncell + c] = k[v];
    }
    stage_program(P, S, prog, I->dt, c, k);
    if (prog.final_stage) {
      const T rho = S.buf[0][c], E = S.buf[0][3 * P.ncell + c];
      bad = !(rho > T(0)) || !(E > T(0));
      if (bad) atomicMin(&real->first, ((unsigned long long)tl.x << 40) | (unsigned long long)(c - B->cell_offset));
    }
  }
  if (prog.final_stage) {
    const int nb = __syncthreads_count(bad);
    if (threadIdx.x == 0 && nb) {
      atomicAdd(&real->nbad, (unsigned long long)nb);
      atomicAdd(&inst[B->instance].nbad, nb);  // halts this instance only
    }
  }
}

template <typename T, bool PERSIST>
__global__ void __launch_bounds__(TX * TY) k_update(ParamsT<T> P, const int4* __restrict__ tiles, int ntiles,
                                                    FaceArraysT<T> F, StateBuffersT<T> S, StageProgram prog,
                                                    InstanceState* __restrict__ inst,
                                                    RealizState* __restrict__ real, T* __restrict__ dudt_out) {
  if constexpr (!PERSIST) {
    update_tile<T>(P, tiles[blockIdx.x], F, S, prog, inst, real, dudt_out);
  } else {
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x)
      update_tile<T>(P, tiles[tile], F, S, prog, inst, real, dudt_out);
  }
}

// --------------------------------------------------------------------------------------
// CFL time step: min over cells of min(dx/(|u|+a), dy/(|v|+a)) per instance
// (quad_block.py:423-436)
// --------------------------------------------------------------------------------------
// One CTA of DT_THREADS threads per cell tile (TY rows x 32 cells, one instance), each
// thread TY / (DT_THREADS / 32) cells of its column: the cells' loads are independent
// and in flight together, the reduction is one atomic per tile.  The minimum is exact,
// so its order changes nothing.
constexpr int DT_THREADS = 64;
template <typename T>
__global__ void __launch_bounds__(DT_THREADS) k_dt(ParamsT<T> P, const int4* __restrict__ tiles,
                                                   const T* __restrict__ U, InstanceState* __restrict__ inst) {
  constexpr int ROWS = DT_THREADS / 32, PER = TY / ROWS;
  const int4 tl = tiles[blockIdx.x];
  const E2DBlock* B = P.blocks + tl.x;
  InstanceState* I = inst + B->instance;
  const int tx = threadIdx.x & 31, r0 = threadIdx.x >> 5;
  const int j = tl.z + tx;
  const Gas<T> G{P.gas[0], P.gas[1], P.gas[2], P.gas[3]};
  unsigned long long bits = 0x7ff0000000000000ULL;  // +inf
#pragma unroll
  for (int k = 0; k < PER; ++k) {
    const int i = tl.y + r0 + k * ROWS;
    if (i < B->ny && j < B->nx) {
      const int64_t c = cell_at(B, i, j);
      T q[4], w[4];
      load_cell(U, P.ncell, c, q);
      cons_to_prim(q, G, w);
      const T a = sqrt(pdiv(P.gas[0] * w[3], w[0]));
      const T tx_ = pdiv(P.geo.cell[E2D_G_CFL_DX][c], fabs(w[1]) + a);
      const T ty_ = pdiv(P.geo.cell[E2D_G_CFL_DY][c], fabs(w[2]) + a);
      // the reduction itself is FP64 on every path
      const unsigned long long b = (unsigned long long)__double_as_longlong(double(vmin(tx_, ty_)));
      bits = b < bits ? b : bits;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long other = __shfl_xor_sync(0xffffffffu, bits, o);
    bits = other < bits ? other : bits;
  }
  __shared__ unsigned long long wmin[ROWS];
  if (tx == 0) wmin[r0] = bits;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long b = wmin[0];
    for (int w = 1; w < ROWS; ++w) b = wmin[w] < b ? wmin[w] : b;
    atomicMin(&I->min_bits, b);
  }
}

template <typename T>
__global__ void k_realizable(ParamsT<T> P, const int4* __restrict__ tiles, const T* __restrict__ U,
                             RealizState* __restrict__ real) {
  const int4 tl = tiles[blockIdx.x];
  const E2DBlock* B = P.blocks + tl.x;
  const int ty = threadIdx.x / TX, tx = threadIdx.x - (threadIdx.x / TX) * TX;
  const int i = tl.y + ty, j = tl.z + tx;
  bool bad = false;
  if (i < B->ny && j < B->nx) {
    const int64_t c = cell_at(B, i, j);
    bad = !(U[c] > T(0)) || !(U[3 * P.ncell + c] > T(0));
    if (bad) atomicMin(&real->first, ((unsigned long long)tl.x << 40) | (unsigned long long)(c - B->cell_offset));
  }
  const int nb = __syncthreads_count(bad);
  if (threadIdx.x == 0 && nb) atomicAdd(&real->nbad, (unsigned long long)nb);
}


}  // namespace e2d

namespace e2d {
// ---- launchers ------------------------------------------------------------------------
// Kernel variants the autotuner chooses from (e2d_autotune): tile height and the
// occupancy target of __launch_bounds__ for k_reconstruct, the occupancy target for
// k_flux, and for every kernel an optional persistent grid (one wave of resident CTAs
// striding over the tile table).
// one wave of resident CTAs (resident CTAs per SM x SMs), at most n
template <typename K>
static int persistent_grid(K kern, int threads, int n) {
  int dev = 0, sms = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, threads, 0);
  const int g = sms * (per > 0 ? per : 1);
  return g < n ? g : n;
}

template <typename T, int LIM, int RECON, bool DBG, int RTY, int MINB>
static cudaError_t recon_launch(const ParamsT<T>& P, const int4* tiles, int n, bool persistent, const T* U,
                                const InstanceState* inst, FaceArraysT<T> F, const DebugOutT<T>& dbg, cudaStream_t st,
                                const TmaSet* tset) {
  const TmaTiles tma = tset ? tset->by_rty[RTY == 4 ? 0 : (RTY == 8 ? 1 : 2)] : TmaTiles{nullptr, nullptr, nullptr};
  if (persistent) {
    auto kern = k_reconstruct<T, LIM, RECON, DBG, RTY, MINB, true>;
    kern<<<persistent_grid(kern, TX * RTY, n), TX * RTY, 0, st>>>(P, tiles, n, U, inst, F, dbg, tma);
  } else {
    k_reconstruct<T, LIM, RECON, DBG, RTY, MINB, false><<<n, TX * RTY, 0, st>>>(P, tiles, n, U, inst, F, dbg, tma);
  }
  return cudaGetLastError();
}

template <typename T, int LIM, int RECON>
static cudaError_t recon_variant(const ParamsT<T>& P, const int4* const* tiles_by_rty, const int* n_by_rty,
                                 int variant, bool persistent, const T* U, const InstanceState* inst, FaceArraysT<T> F,
                                 const DebugOutT<T>* dbg, cudaStream_t st, const TmaSet* tma) {
  if (dbg)  // the per-operator outputs are built for the default variant only
    return recon_launch<T, LIM, RECON, true, 8, 1>(P, tiles_by_rty[1], n_by_rty[1], false, U, inst, F, *dbg, st, tma);
  const DebugOutT<T> none{};
  switch (variant) {
    case 1: return recon_launch<T, LIM, RECON, false, 8, 1>(P, tiles_by_rty[1], n_by_rty[1], persistent, U, inst, F, none, st, tma);
    case 2: return recon_launch<T, LIM, RECON, false, 4, 2>(P, tiles_by_rty[0], n_by_rty[0], persistent, U, inst, F, none, st, tma);
    case 3: return recon_launch<T, LIM, RECON, false, 4, 4>(P, tiles_by_rty[0], n_by_rty[0], persistent, U, inst, F, none, st, tma);
    case 4: return recon_launch<T, LIM, RECON, false, 16, 1>(P, tiles_by_rty[2], n_by_rty[2], persistent, U, inst, F, none, st, tma);
    case 5:  // FP32 only (64 registers, 8 CTAs of 128 threads per SM); FP64 would spill
      if constexpr (sizeof(T) == 4)
        return recon_launch<T, LIM, RECON, false, 4, 8>(P, tiles_by_rty[0], n_by_rty[0], persistent, U, inst, F, none, st, tma);
      else
        return recon_launch<T, LIM, RECON, false, 8, 2>(P, tiles_by_rty[1], n_by_rty[1], persistent, U, inst, F, none, st, tma);
    default: return recon_launch<T, LIM, RECON, false, 8, 2>(P, tiles_by_rty[1], n_by_rty[1], persistent, U, inst, F, none, st, tma);
  }
}

// One limiter's reconstruction launchers (every variant, and the multi-point form).
// Each (type, limiter) pair is instantiated in a translation unit of its own
// (e2d_recon_unit.cu), so the kernels compile in parallel.
template <typename T, int LIM>
cudaError_t recon_lim(const ParamsT<T>& P, const int4* const* tiles, const int* n, int variant, bool persistent,
                             const T* U, const InstanceState* inst, FaceArraysT<T> F, const DebugOutT<T>* dbg,
                             cudaStream_t st, const TmaSet* tma) {
  if (P.recon == E2D_RECON_PRIMITIVE)
    return recon_variant<T, LIM, E2D_RECON_PRIMITIVE>(P, tiles, n, variant, persistent, U, inst, F, dbg, st, tma);
  return recon_variant<T, LIM, E2D_RECON_CONSERVATIVE>(P, tiles, n, variant, persistent, U, inst, F, dbg, st, tma);
}

template <typename T, int LIM, int RECON>
static cudaError_t recon_qp(const ParamsT<T>& P, const TileSet& ts, const T* U, const InstanceState* inst,
                            FaceArraysT<T> F, cudaStream_t st) {
  if (P.nqp == 3)
    k_reconstruct_qp<T, LIM, RECON, 3><<<ts.ncell[1], TX * TY, 0, st>>>(P, ts.cell[1], U, inst, F);
  else
    k_reconstruct_qp<T, LIM, RECON, 2><<<ts.ncell[1], TX * TY, 0, st>>>(P, ts.cell[1], U, inst, F);
  return cudaGetLastError();
}

template <typename T, int LIM>
cudaError_t recon_qp_lim(const ParamsT<T>& P, const TileSet& ts, const T* U, const InstanceState* inst,
                                FaceArraysT<T> F, cudaStream_t st) {
  if (P.recon == E2D_RECON_PRIMITIVE) return recon_qp<T, LIM, E2D_RECON_PRIMITIVE>(P, ts, U, inst, F, st);
  return recon_qp<T, LIM, E2D_RECON_CONSERVATIVE>(P, ts, U, inst, F, st);
}

template <typename T>
cudaError_t launch_reconstruct(const ParamsT<T>& P, const TileSet& ts, KernelChoice kc, const T* U,
                               const InstanceState* inst, FaceArraysT<T> F, const DebugOutT<T>* dbg, cudaStream_t st,
                               const TmaSet* tma) {
  const int4* tiles[3] = {ts.cell[0], ts.cell[1], ts.cell[2]};
  if (ts.ncell[1] <= 0) return cudaSuccess;
  if (P.nqp > 1) {  // several face quadrature points: one kernel form, no per-operator outputs
    switch (P.limiter) {
      case E2D_LIM_BARTH_JESPERSEN: return recon_qp_lim<T, E2D_LIM_BARTH_JESPERSEN>(P, ts, U, inst, F, st);
      case E2D_LIM_VAN_ALBADA: return recon_qp_lim<T, E2D_LIM_VAN_ALBADA>(P, ts, U, inst, F, st);
      case E2D_LIM_VAN_LEER: return recon_qp_lim<T, E2D_LIM_VAN_LEER>(P, ts, U, inst, F, st);
      default: return recon_qp_lim<T, E2D_LIM_VENKATAKRISHNAN>(P, ts, U, inst, F, st);
    }
  }
  switch (P.limiter) {
    case E2D_LIM_BARTH_JESPERSEN:
      return recon_lim<T, E2D_LIM_BARTH_JESPERSEN>(P, tiles, ts.ncell, kc.variant, kc.persistent, U, inst, F, dbg, st, tma);
    case E2D_LIM_VAN_ALBADA:
      return recon_lim<T, E2D_LIM_VAN_ALBADA>(P, tiles, ts.ncell, kc.variant, kc.persistent, U, inst, F, dbg, st, tma);
    case E2D_LIM_VAN_LEER:
      return recon_lim<T, E2D_LIM_VAN_LEER>(P, tiles, ts.ncell, kc.variant, kc.persistent, U, inst, F, dbg, st, tma);
    default:
      return recon_lim<T, E2D_LIM_VENKATAKRISHNAN>(P, tiles, ts.ncell, kc.variant, kc.persistent, U, inst, F, dbg, st, tma);
  }
}

template <typename T, int FLUX, bool DBG, int MINB>
static cudaError_t flux_launch(const ParamsT<T>& P, const int4* tiles, int n, bool persistent,
                               const InstanceState* inst, FaceArraysT<T> F, const DebugOutT<T>& dbg, cudaStream_t st) {
  if (persistent) {
    auto kern = k_flux<T, FLUX, DBG, MINB, true>;
    kern<<<persistent_grid(kern, TX * TY, n), TX * TY, 0, st>>>(P, tiles, n, inst, F, dbg);
  } else {
    k_flux<T, FLUX, DBG, MINB, false><<<n, TX * TY, 0, st>>>(P, tiles, n, inst, F, dbg);
  }
  return cudaGetLastError();
}

template <typename T, int FLUX>
static cudaError_t flux_t(const ParamsT<T>& P, const int4* tiles, int n, KernelChoice kc, const InstanceState* inst,
                          FaceArraysT<T> F, const DebugOutT<T>* dbg, cudaStream_t st) {
  if (dbg) return flux_launch<T, FLUX, true, 1>(P, tiles, n, false, inst, F, *dbg, st);
  const DebugOutT<T> none{};
  switch (kc.variant) {
    case 1: return flux_launch<T, FLUX, false, 1>(P, tiles, n, kc.persistent, inst, F, none, st);
    case 2: return flux_launch<T, FLUX, false, 6>(P, tiles, n, kc.persistent, inst, F, none, st);
    default: return flux_launch<T, FLUX, false, 4>(P, tiles, n, kc.persistent, inst, F, none, st);
  }
}

template <typename T, int FLUX>
static cudaError_t flux_qp(const ParamsT<T>& P, const TileSet& ts, const InstanceState* inst, FaceArraysT<T> F,
                           cudaStream_t st) {
  if (P.nqp == 3) k_flux_qp<T, FLUX, 3><<<ts.nface, TX * TY, 0, st>>>(P, ts.face, inst, F);
  else k_flux_qp<T, FLUX, 2><<<ts.nface, TX * TY, 0, st>>>(P, ts.face, inst, F);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_flux(const ParamsT<T>& P, const TileSet& ts, KernelChoice kc, const InstanceState* inst,
                        FaceArraysT<T> F, const DebugOutT<T>* dbg, cudaStream_t st) {
  if (ts.nface <= 0) return cudaSuccess;
  if (P.nqp > 1) {
    switch (P.flux) {
      case E2D_FLUX_HLLL: return flux_qp<T, E2D_FLUX_HLLL>(P, ts, inst, F, st);
      case E2D_FLUX_HLLE: return flux_qp<T, E2D_FLUX_HLLE>(P, ts, inst, F, st);
      default: return flux_qp<T, E2D_FLUX_ROE>(P, ts, inst, F, st);
    }
  }
  switch (P.flux) {
    case E2D_FLUX_HLLL: return flux_t<T, E2D_FLUX_HLLL>(P, ts.face, ts.nface, kc, inst, F, dbg, st);
    case E2D_FLUX_HLLE: return flux_t<T, E2D_FLUX_HLLE>(P, ts.face, ts.nface, kc, inst, F, dbg, st);
    default: return flux_t<T, E2D_FLUX_ROE>(P, ts.face, ts.nface, kc, inst, F, dbg, st);
  }
}

template <typename T>
cudaError_t launch_update(const ParamsT<T>& P, const TileSet& ts, KernelChoice kc, FaceArraysT<T> F,
                          StateBuffersT<T> S, const StageProgram& prog, InstanceState* inst, RealizState* real,
                          T* dudt_out, cudaStream_t st) {
  const int n = ts.ncell[1];
  if (n <= 0) return cudaSuccess;
  if (kc.persistent) {
    auto kern = k_update<T, true>;
    kern<<<persistent_grid(kern, TX * TY, n), TX * TY, 0, st>>>(P, ts.cell[1], n, F, S, resolve_program(prog, S),
                                                                 inst, real, dudt_out);
  } else {
    k_update<T, false><<<n, TX * TY, 0, st>>>(P, ts.cell[1], n, F, S, resolve_program(prog, S), inst, real,
                                              dudt_out);
  }
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_dt(const ParamsT<T>& P, const int4* tiles, int n, const T* U, InstanceState* inst,
                      cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  k_dt<T><<<n, DT_THREADS, 0, st>>>(P, tiles, U, inst);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_realizable(const ParamsT<T>& P, const int4* tiles, int n, const T* U, RealizState* real,
                              cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  k_realizable<T><<<n, TX * TY, 0, st>>>(P, tiles, U, real);
  return cudaGetLastError();
}

// Conserved totals: per 8-row cell tile, the sum over its cells of A * U_v for the
// four conserved variables, accumulated in FP64 whatever the path's precision (cell
// values and areas promoted), in a fixed order (a shared-memory tree over the tile's
// 256 cells), into partial[tile][4].  The caller sums the partials of each instance in
// tile order, so the totals are reproducible run to run.
template <typename T>
__global__ void __launch_bounds__(TX * TY) k_totals(ParamsT<T> P, const int4* __restrict__ tiles,
                                                    const T* __restrict__ U, double* __restrict__ partial) {
  __shared__ double red[4][TX * TY];
  const int4 tl = tiles[blockIdx.x];
  const E2DBlock* B = P.blocks + tl.x;
  const int ty = threadIdx.x / TX, tx = threadIdx.x - (threadIdx.x / TX) * TX;
  const int i = tl.y + ty, j = tl.z + tx;
  double v[4] = {0.0, 0.0, 0.0, 0.0};
  if (i < B->ny && j < B->nx) {
    const int64_t c = cell_at(B, i, j);
    const double A = (double)P.geo.cell[E2D_G_A][c];
#pragma unroll
    for (int k = 0; k < 4; ++k) v[k] = A * (double)U[k * P.ncell + c];
  }
#pragma unroll
  for (int k = 0; k < 4; ++k) red[k][threadIdx.x] = v[k];
  __syncthreads();
  for (int w = TX * TY / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
#pragma unroll
      for (int k = 0; k < 4; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x < 4) partial[4 * (int64_t)blockIdx.x + threadIdx.x] = red[threadIdx.x][0];
}

template <typename T>
cudaError_t launch_totals(const ParamsT<T>& P, const int4* tiles, int n, const T* U, double* partial,
                          cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  k_totals<T><<<n, TX * TY, 0, st>>>(P, tiles, U, partial);
  return cudaGetLastError();
}

// Ghost layer of every block in the reconstruction variables: the values that
// Blocks.apply_boundary_condition leaves in the ghost blocks and that
// ReconstructionBlock.from_block converts (pyhype/blocks/base.py:448-471,
// pyhype/blocks/ghost.py:149-216, pyhype/blocks/quad_block.py:120-134).  Per block
// the layer is E (ny values, south to north), W (ny), N (nx, west to east), S (nx),
// starting at base[b]; out holds 4 planes of nghost values.  One thread per ghost
// cell; grid.y strides over blocks.
template <typename T, int RECON>
__global__ void k_ghost_layer(ParamsT<T> P, const T* __restrict__ U, double t, const int64_t* __restrict__ base,
                              double* __restrict__ out, int64_t nghost) {
  const Gas<T> G{P.gas[0], P.gas[1], P.gas[2], P.gas[3]};
  for (int b = blockIdx.y; b < P.nblocks; b += gridDim.y) {
    const E2DBlock* B = P.blocks + b;
    const int nx = B->nx, ny = B->ny, len = 2 * (nx + ny);
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < len; g += gridDim.x * blockDim.x) {
      int side, k;
      if (g < ny) { side = E2D_E; k = g; }
      else if (g < 2 * ny) { side = E2D_W; k = g - ny; }
      else if (g < 2 * ny + nx) { side = E2D_N; k = g - 2 * ny; }
      else { side = E2D_S; k = g - 2 * ny - nx; }
      T q[4], r[4];
      ghost_cons(P, B, side, k, U, t, q);
      to_recon<RECON>(q, G, r);
#pragma unroll
      for (int v = 0; v < 4; ++v) out[v * nghost + base[b] + g] = (double)r[v];
    }
  }
}

// maxlen: the longest layer of one block, 2 (nx + ny)
template <typename T>
cudaError_t launch_ghost_layer(const ParamsT<T>& P, const T* U, double t, const int64_t* base, double* out,
                               int64_t nghost, int maxlen, cudaStream_t st) {
  if (nghost <= 0) return cudaSuccess;
  const dim3 grid((maxlen + 255) / 256, P.nblocks < 65535 ? P.nblocks : 65535);
  if (P.recon == E2D_RECON_PRIMITIVE)
    k_ghost_layer<T, E2D_RECON_PRIMITIVE><<<grid, 256, 0, st>>>(P, U, t, base, out, nghost);
  else
    k_ghost_layer<T, E2D_RECON_CONSERVATIVE><<<grid, 256, 0, st>>>(P, U, t, base, out, nghost);
  return cudaGetLastError();
}

// PRE is empty to instantiate, `extern` to declare an instantiation made elsewhere
#define E2D_RECON_LIM_DECL(PRE, T, LIM)                                                                           \
  PRE template cudaError_t recon_lim<T, LIM>(const ParamsT<T>&, const int4* const*, const int*, int, bool,        \
                                             const T*, const InstanceState*, FaceArraysT<T>, const DebugOutT<T>*, \
                                             cudaStream_t, const TmaSet*);                                        \
  PRE template cudaError_t recon_qp_lim<T, LIM>(const ParamsT<T>&, const TileSet&, const T*, const InstanceState*, \
                                                FaceArraysT<T>, cudaStream_t);
// the per-limiter launchers are instantiated elsewhere (e2d_recon_unit.cu)
#define E2D_EXTERN_RECON_LIM(T)         \
  E2D_RECON_LIM_DECL(extern, T, 0)      \
  E2D_RECON_LIM_DECL(extern, T, 1)      \
  E2D_RECON_LIM_DECL(extern, T, 2)      \
  E2D_RECON_LIM_DECL(extern, T, 3)

#define E2D_INSTANTIATE_STAGE_LAUNCHERS(T)                                                                       \
  template cudaError_t launch_reconstruct<T>(const ParamsT<T>&, const TileSet&, KernelChoice, const T*,          \
                                             const InstanceState*, FaceArraysT<T>, const DebugOutT<T>*,          \
                                             cudaStream_t, const TmaSet*);                                       \
  template cudaError_t launch_flux<T>(const ParamsT<T>&, const TileSet&, KernelChoice, const InstanceState*,     \
                                      FaceArraysT<T>, const DebugOutT<T>*, cudaStream_t);                        \
  template cudaError_t launch_update<T>(const ParamsT<T>&, const TileSet&, KernelChoice, FaceArraysT<T>,         \
                                        StateBuffersT<T>, const StageProgram&, InstanceState*, RealizState*, T*, \
                                        cudaStream_t);                                                           \
  template cudaError_t launch_dt<T>(const ParamsT<T>&, const int4*, int, const T*, InstanceState*, cudaStream_t); \
  template cudaError_t launch_realizable<T>(const ParamsT<T>&, const int4*, int, const T*, RealizState*, cudaStream_t); \
  template cudaError_t launch_ghost_layer<T>(const ParamsT<T>&, const T*, double, const int64_t*, double*, int64_t, \
                                             int, cudaStream_t);                                                 \
  template cudaError_t launch_totals<T>(const ParamsT<T>&, const int4*, int, const T*, double*, cudaStream_t);

// for units that include this header but call the launchers instantiated elsewhere
#define E2D_EXTERN_STAGE_LAUNCHERS(T)                                                                           \
  extern template cudaError_t launch_reconstruct<T>(const ParamsT<T>&, const TileSet&, KernelChoice, const T*,   \
                                                    const InstanceState*, FaceArraysT<T>, const DebugOutT<T>*,   \
                                                    cudaStream_t, const TmaSet*);                                \
  extern template cudaError_t launch_flux<T>(const ParamsT<T>&, const TileSet&, KernelChoice, const InstanceState*, \
                                             FaceArraysT<T>, const DebugOutT<T>*, cudaStream_t);                 \
  extern template cudaError_t launch_update<T>(const ParamsT<T>&, const TileSet&, KernelChoice, FaceArraysT<T>,  \
                                               StateBuffersT<T>, const StageProgram&, InstanceState*, RealizState*, \
                                               T*, cudaStream_t);                                                \
  extern template cudaError_t launch_dt<T>(const ParamsT<T>&, const int4*, int, const T*, InstanceState*,        \
                                           cudaStream_t);                                                        \
  extern template cudaError_t launch_realizable<T>(const ParamsT<T>&, const int4*, int, const T*, RealizState*,  \
                                                   cudaStream_t);                                                \
  extern template cudaError_t launch_ghost_layer<T>(const ParamsT<T>&, const T*, double, const int64_t*, double*, \
                                                    int64_t, int, cudaStream_t);                                 \
  extern template cudaError_t launch_totals<T>(const ParamsT<T>&, const int4*, int, const T*, double*, cudaStream_t);

}  // namespace e2d
