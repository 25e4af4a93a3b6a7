// e2d_adjoint.cuh - reverse-mode kernels of the residual and of one RK step.
//
// The residual R(U) is K3(K2(K1(U))) with K1 = reconstruction (ghost cells, interface
// averages, Green-Gauss gradient, limiter, limited face states, rotation, conversion
// to primitive), K2 = one Riemann flux per face, K3 = divergence.  Its transpose runs
// the same three passes backwards:
//
//   k_flux_vjp          per face: the adjoint of the two cells' dUdt that the face
//                       feeds (K3^T, one face at a time), times 2L, rotated by the
//                       transpose of the flux un-rotation, through the Roe, HLLL or
//                       HLLE flux VJP;
//                       the face's left/right adjoints overwrite its stored states.
//   k_reconstruct_vjp   per cell: recomputes the cell's reconstruction from the stage
//                       state (the same expressions as the forward kernel, so every
//                       min/max/branch selects the same operand) and pulls the face
//                       adjoints back through conversion, rotation, limiter and
//                       gradient onto its five-point stencil; the four neighbour
//                       contributions go to per-cell slots.
//   k_adjoint_gather    per cell: sums its own slot and the slots its neighbours
//                       (or, at block edges, its own ghost images) wrote for it,
//                       transposes the ghost maps (copy, reflection, inter-block
//                       halo), converts to conservative variables and applies the
//                       RK adjoint stage program.
//
// Subgradients: min/max take the operand the forward selects (the first of equal
// operands), Harten's entropy fix differentiates the branch taken, the davg == 0
// slope branch (s = 1) is constant, and a negative limiter value clipped to 0 passes
// nothing back.
#pragma once
#include "e2d_adjoint_ops.cuh"
#include "e2d_stage.cuh"

namespace e2d {

// stencil slots of k_reconstruct_vjp: the cell itself and its E, W, N, S values
enum { ST_SELF = 0, ST_E = 1, ST_W = 2, ST_N = 3, ST_S = 4, ST_NSLOTS = 5 };

// RK adjoint program of one stage: lam_U += lam_Y and acc[q] += coef[q] * lam_Y.
template <typename T>
struct AdjProgramT {
  int n;
  T* dst[MAX_STAGES];
  double coef[MAX_STAGES];
};

// Forward limiter of one variable of one cell, the expressions of the reconstruction
// kernel (interface averages, Green-Gauss gradient, high-order terms, slopes, psi,
// minimum over faces, clip), recording the selections the reverse pass needs.
template <typename T>
struct LimiterTrace {
  int sel;       // face whose psi is phi (the first of equal values)
  T sl;          // that face's slope
  T davg;        // that face's difference
  int sign;      // +1 davg > 0, -1 davg < 0, 0 davg == 0 (slope 1)
  bool clipped;  // phi was negative and set to 0
  int imax, imin;  // stencil index (w0, we, ea, so, no) of the max and of the min
};

// interface averages and Green-Gauss gradient of one variable (forward expressions)
template <typename T>
__device__ __forceinline__ void green_gauss(T w0, T we, T ea, T so, T no, T LcE, T LsE, T LcW, T LsW, T LcN, T LsN,
                                            T LcS, T LsS, T ia, T& gx, T& gy) {
  const T ie = half(w0 + ea), iw = half(we + w0);
  const T in = half(w0 + no), is = half(so + w0);
  gx = (ie * LcE + iw * (-LcW) + in * LcN + is * (-LcS)) * ia;
  gy = (ie * LsE + iw * (-LsW) + in * LsN + is * (-LsS)) * ia;
}

template <typename T, int LIM>
__device__ __forceinline__ void limiter_forward(T w0, T we, T ea, T so, T no, T LcE, T LsE, T LcW, T LsW, T LcN,
                                                T LsN, T LcS, T LsS, T ia, const T* hx, const T* hy, T* hot, T& ph,
                                                LimiterTrace<T>* tr, T* gxo = nullptr, T* gyo = nullptr) {
  T gx, gy;
  green_gauss(w0, we, ea, so, no, LcE, LsE, LcW, LsW, LcN, LsN, LcS, LsS, ia, gx, gy);
  if (gxo) { *gxo = gx; *gyo = gy; }
  // vmax(a, b) keeps a unless a < b; vmin(a, b) keeps a unless b < a
  const T nb[4] = {we, ea, so, no};
  T mx = w0, mn = w0;
  int imx = 0, imn = 0;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    if (vlt(mx, nb[q])) { mx = nb[q]; imx = q + 1; }
    if (vlt(nb[q], mn)) { mn = nb[q]; imn = q + 1; }
  }
  const T dmax = mx - w0, dmin = mn - w0;
  int sel = 0, ssign = 0;
  T ssl = T(0), sdavg = T(0);
  T dv[4];
#pragma unroll
  for (int s = 0; s < 4; ++s) {
    hot[s] = gx * hx[s] + gy * hy[s];
    if constexpr (sizeof(T) == 4) {
      const T half_ulp64 = __int_as_float(__float_as_int(w0) & 0x7f800000) * T(1.1102230246251565e-16);
      dv[s] = (fabs(hot[s]) < half_ulp64) ? T(0) : hot[s];
    } else {
      dv[s] = (w0 + hot[s]) - w0;
    }
  }
  bool done = false;
  if constexpr (sizeof(T) == 8) {
    // FP64: psi only at the faces that decide phi, as the reconstruction kernel does;
    // the selected face is the first whose psi equals phi, as in the loop below.
    // Barth-Jespersen at phi == 1 (every face with s >= 1 gives 1: the first face is
    // selected) takes the loop.
    const SlopePick k = pick_slopes<LIM>(dmax, dmin, dv);
    if (k.ok) {
      T sl = k.ga ? qdiv(k.na, k.da) : T(1);
      T p = psi_s<LIM>(sl);
      int f = k.fa;
      T d = k.da;
      if (k.second) {
        const T slb = k.gb ? qdiv(k.nb, k.db) : T(1);
        const T pb = psi_s<LIM>(slb);
        if (vlt(pb, p) || (!vlt(p, pb) && k.fb < k.fa)) {
          p = pb; sl = slb; f = k.fb; d = k.db;
        }
      }
      if (!(LIM == E2D_LIM_BARTH_JESPERSEN && p == T(1))) {
        done = true;
        ph = p; sel = f; ssl = sl; sdavg = d;
        ssign = is_pos(d) ? 1 : (is_neg(d) ? -1 : 0);
      }
    }
  }
  if constexpr (sizeof(T) == 4) {
    // the FP32 forward's limiter (limit_cell_var): slopes from the reciprocal
    // approximation, psi at the smallest and (limiters with a maximum) the largest;
    // the selected face is the first face with the smallest (largest) slope
    T sls[4];
    int imn_s = 0, imx_s = 0;
#pragma unroll
    for (int s = 0; s < 4; ++s) {
      sls[s] = slope32(dmax, dmin, dv[s], FLOAT_TRUE_MIN);  // dv: thresholded already
      if (s > 0 && vlt(sls[s], sls[imn_s])) imn_s = s;
      if (s > 0 && vlt(sls[imx_s], sls[s])) imx_s = s;
    }
    T smin = sls[0], smax = sls[0], dmn = dv[0], dmx = dv[0];
#pragma unroll
    for (int s = 1; s < 4; ++s) {  // constant indices only (no local-memory array)
      if (s == imn_s) { smin = sls[s]; dmn = dv[s]; }
      if (s == imx_s) { smax = sls[s]; dmx = dv[s]; }
    }
    ph = psi_s<LIM>(smin);
    sel = imn_s; ssl = smin; sdavg = dmn;
    if constexpr (psi_has_peak<LIM>()) {
      const T pb = psi_s<LIM>(smax);
      if (vlt(pb, ph)) { ph = pb; sel = imx_s; ssl = smax; sdavg = dmx; }
    }
    ssign = is_pos(sdavg) ? 1 : (is_neg(sdavg) ? -1 : 0);
    done = true;
  }
  if (!done) {
#pragma unroll
    for (int s = 0; s < 4; ++s) {
      const T davg = dv[s];
      const bool pos = is_pos(davg), neg = is_neg(davg);
      const T sl = (pos || neg) ? qdiv(pos ? dmax : dmin, davg) : T(1);
      const T p = psi_s<LIM>(sl);
      if (s == 0 || vlt(p, ph)) {
        ph = p;
        sel = s;
        ssl = sl;
        sdavg = davg;
        ssign = pos ? 1 : (neg ? -1 : 0);
      }
    }
  }
  const bool clipped = is_neg(ph);
  ph = clipped ? T(0) : ph;
  if (tr) {
    tr->sel = sel;
    tr->sl = ssl;
    tr->davg = sdavg;
    tr->sign = ssign;
    tr->clipped = clipped;
    tr->imax = imx;
    tr->imin = imn;
  }
}

// ---------------------------------------------------------------------------------
// K2^T, K3^T
// ---------------------------------------------------------------------------------
template <typename T, int FLUX>
__global__ void __launch_bounds__(TX * TY) k_flux_vjp(ParamsT<T> P, const int4* __restrict__ tiles,
                                                      const InstanceState* __restrict__ inst, FaceArraysT<T> F,
                                                      const T* __restrict__ lk) {
  const int4 tl = tiles[blockIdx.x];
  const E2DBlock* B = P.blocks + tl.x;
  if (!inst[B->instance].active) return;
  const int nx = B->nx, ny = B->ny;
  const int ty = threadIdx.x / TX, tx = threadIdx.x - (threadIdx.x / TX) * TX;
  const int i = tl.y + ty, j = tl.z + tx;
  if (i > ny || j > nx) return;
  const Gas<T> G{P.gas[0], P.gas[1], P.gas[2], P.gas[3]};
  const bool cart = block_cart(P, B, tl.x);
  const T* ia = P.geo.cell[E2D_G_INV_A];
  // dUdt = 0.5*(I_W - I_E + I_S - I_N)/A: a face is the W (S) face of the cell above
  // it in index order and the E (N) face of the cell below.
  if (i < ny) {
    const int64_t f = vf_at(B, i, j);
    T lF[4];
    const T len2 = twice(P.geo.vface[E2D_F_L][f]);
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      T li = T(0);
      if (j < nx) { const int64_t c = cell_at(B, i, j); li += half(lk[v * P.ncell + c]) * ia[c]; }
      if (j > 0) { const int64_t c = cell_at(B, i, j - 1); li -= half(lk[v * P.ncell + c]) * ia[c]; }
      lF[v] = len2 * li;
    }
    if (!cart) rotate(lF, P.geo.vface[E2D_F_COS][f], P.geo.vface[E2D_F_SIN][f]);  // transpose of unrotate
    T L[4], R[4], lL[4] = {T(0), T(0), T(0), T(0)}, lR[4] = {T(0), T(0), T(0), T(0)};
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      L[v] = F.vL[v * P.nvface + f];
      R[v] = F.vR[v * P.nvface + f];
    }
    riemann_vjp<FLUX>(L, R, G, lF, lL, lR);
    store4(F.vL, P.nvface, f, lL);
    store4(F.vR, P.nvface, f, lR);
  }
  if (j < nx) {
    const int64_t f = hf_at(B, i, j);
    T lF[4];
    const T len2 = twice(P.geo.hface[E2D_F_L][f]);
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      T li = T(0);
      if (i < ny) { const int64_t c = cell_at(B, i, j); li += half(lk[v * P.ncell + c]) * ia[c]; }
      if (i > 0) { const int64_t c = cell_at(B, i - 1, j); li -= half(lk[v * P.ncell + c]) * ia[c]; }
      lF[v] = len2 * li;
    }
    if (cart) rotate90(lF);  // transpose of unrotate90
    else rotate(lF, P.geo.hface[E2D_F_COS][f], P.geo.hface[E2D_F_SIN][f]);
    T L[4], R[4], lL[4] = {T(0), T(0), T(0), T(0)}, lR[4] = {T(0), T(0), T(0), T(0)};
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      L[v] = F.hL[v * P.nhface + f];
      R[v] = F.hR[v * P.nhface + f];
    }
    riemann_vjp<FLUX>(L, R, G, lF, lL, lR);
    store4(F.hL, P.nhface, f, lL);
    store4(F.hR, P.nhface, f, lR);
  }
}

// ---------------------------------------------------------------------------------
// K1^T
// ---------------------------------------------------------------------------------
// Adjoint of a face state w = recon_to_prim(rot(q)) given lam_w: returns lam_q
// (reconstruction variables, unrotated) in lq.  rot: 0 none, 1 (c, s), 2 rotate90.
template <int RECON, typename T>
__device__ __forceinline__ void face_state_vjp(const T* q, int rot, T c, T s, const Gas<T>& G, const T* lw, T* lq) {
  T qr[4] = {q[0], q[1], q[2], q[3]};
  if (rot == 1) rotate(qr, c, s);
  else if (rot == 2) rotate90(qr);
  lq[0] = T(0); lq[1] = T(0); lq[2] = T(0); lq[3] = T(0);
  if (RECON == E2D_RECON_PRIMITIVE) {
    lq[0] = lw[0]; lq[1] = lw[1]; lq[2] = lw[2]; lq[3] = lw[3];
  } else {
    cons_to_prim_vjp(qr, G, lw, lq);
  }
  if (rot == 1) unrotate(lq, c, s);  // transpose of rotate
  else if (rot == 2) unrotate90(lq);
}

template <typename T>
__device__ __forceinline__ void load_face(const T* __restrict__ a, int64_t stride, int64_t f, T* q) {
  q[0] = a[f];
  q[1] = a[stride + f];
  q[2] = a[2 * stride + f];
  q[3] = a[3 * stride + f];
}

// tile height of the reverse reconstruction (128 threads: its per-thread shared-memory
// staging of 36 values fits the static limit)
constexpr int VTY = 4;

template <typename T, int LIM, int RECON>
__global__ void __launch_bounds__(TX * VTY, 4) k_reconstruct_vjp(ParamsT<T> P, const int4* __restrict__ tiles,
                                                              const T* __restrict__ U,
                                                              const InstanceState* __restrict__ inst,
                                                              FaceArraysT<T> F, T* __restrict__ st) {
  __shared__ T sW[4][VTY + 2][TX + 2];
  const Gas<T> G{P.gas[0], P.gas[1], P.gas[2], P.gas[3]};
  const int4 tl = tiles[blockIdx.x];
  const E2DBlock* B = P.blocks + tl.x;
  const InstanceState* I = inst + B->instance;
  if (!I->active) return;
  const double t = I->t;
  const int nx = B->nx, ny = B->ny;
  const int i0 = tl.y, j0 = tl.z;
  // stencil tile in reconstruction variables, ghosts formed as in the forward kernel;
  // a tile whose halo lies inside the block takes a uniform path without them
  const bool edge = i0 == 0 || j0 == 0 || i0 + VTY >= ny || j0 + TX >= nx;
  for (int p = threadIdx.x; p < (VTY + 2) * (TX + 2); p += TX * VTY) {
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
  T hx[4], hy[4];
#pragma unroll
  for (int s = 0; s < 4; ++s) {
    hx[s] = P.geo.cell[E2D_G_HX_E + s][c];
    hy[s] = P.geo.cell[E2D_G_HY_E + s][c];
  }
  const bool cart = block_cart(P, B, tl.x);
  const T cE = P.geo.vface[E2D_F_COS][fE], sE = P.geo.vface[E2D_F_SIN][fE];
  const T cW = P.geo.vface[E2D_F_COS][fW], sW_ = P.geo.vface[E2D_F_SIN][fW];
  const T cN = P.geo.hface[E2D_F_COS][fN], sN = P.geo.hface[E2D_F_SIN][fN];
  const T cS = P.geo.hface[E2D_F_COS][fS], sS = P.geo.hface[E2D_F_SIN][fS];
  const int rotV = cart ? 0 : 1, rotH = cart ? 2 : 1;

  // Shared-memory staging, one slot per thread: the forward limiter's result and
  // selections per variable (phase A, read again in phase C instead of a second
  // limiter evaluation), and the 16 face adjoints (phase B) that phase C consumes one
  // variable at a time.
  __shared__ T sTr[4][5][TX * VTY];   // per variable: phi, gx, gy, selected slope, its davg
  __shared__ int sTi[4][TX * VTY];    // per variable: sel | sign | clipped | imax | imin
  __shared__ T sL[16][TX * VTY];
  const int tid = threadIdx.x;

  // Phase A: forward limiter (the forward kernel's expressions)
#pragma unroll 1
  for (int v = 0; v < 4; ++v) {
    T hot[4], ph, gx, gy;
    LimiterTrace<T> tr;
    limiter_forward<T, LIM>(sW[v][ty + 1][tx + 1], sW[v][ty + 1][tx], sW[v][ty + 1][tx + 2], sW[v][ty][tx + 1],
                            sW[v][ty + 2][tx + 1], LcE, LsE, LcW, LsW, LcN, LsN, LcS, LsS, ia, hx, hy, hot, ph, &tr,
                            &gx, &gy);
    sTr[v][0][tid] = ph;
    sTr[v][1][tid] = gx;
    sTr[v][2][tid] = gy;
    sTr[v][3][tid] = tr.sl;
    sTr[v][4][tid] = tr.davg;
    sTi[v][tid] = tr.sel | ((tr.sign + 1) << 2) | (tr.clipped ? 16 : 0) | (tr.imax << 5) | (tr.imin << 8);
  }

  // Phase B: per side, the face-state adjoint through conversion and rotation, plus
  // the boundary face's outside state when it is this cell's own face state (with the
  // side's reflection); ghost-valued outside states are handled in phase D
#pragma unroll
  for (int side = 0; side < 4; ++side) {
    T q[4], lw[4], lq[4];
#pragma unroll
    for (int v = 0; v < 4; ++v) {  // the limited face state w0 + phi * hot of the forward
      const T hot = sTr[v][1][tid] * hx[side] + sTr[v][2][tid] * hy[side];
      q[v] = sW[v][ty + 1][tx + 1] + sTr[v][0][tid] * hot;
    }
    const bool vert = side == E2D_E || side == E2D_W;
    const T fc = side == E2D_E ? cE : side == E2D_W ? cW : side == E2D_N ? cN : cS;
    const T fs = side == E2D_E ? sE : side == E2D_W ? sW_ : side == E2D_N ? sN : sS;
    const int rot = vert ? rotV : rotH;
    // this cell's face state is the left state of its E/N face, the right state of W/S
    if (side == E2D_E) load_face(F.vL, P.nvface, fE, lw);
    else if (side == E2D_W) load_face(F.vR, P.nvface, fW, lw);
    else if (side == E2D_N) load_face(F.hL, P.nhface, fN, lw);
    else load_face(F.hR, P.nhface, fS, lw);
    face_state_vjp<RECON>(q, rot, fc, fs, G, lw, lq);
    const bool at = side == E2D_E ? j == nx - 1 : side == E2D_W ? j == 0 : side == E2D_N ? i == ny - 1 : i == 0;
    if (edge && at) {
      const int k = vert ? i : j;
      const double *gd, *fd;
      const int kind = side_kind_at(B, side, k, t, gd, fd);
      if (kind == E2D_SIDE_REFLECT || kind == E2D_SIDE_OUTLET) {
        T o[4] = {q[0], q[1], q[2], q[3]};
        T bc = T(0), bs = T(0);
        if (kind == E2D_SIDE_REFLECT) {
          boundary_cs(P, B, side, k, bc, bs);
          reflect(o, bc, bs);
        }
        T lo[4];
        // the outside state is the other side's state of the same face
        if (side == E2D_E) load_face(F.vR, P.nvface, fE, lw);
        else if (side == E2D_W) load_face(F.vL, P.nvface, fW, lw);
        else if (side == E2D_N) load_face(F.hR, P.nhface, fN, lw);
        else load_face(F.hL, P.nhface, fS, lw);
        face_state_vjp<RECON>(o, rot, fc, fs, G, lw, lo);
        if (kind == E2D_SIDE_REFLECT) reflect_vjp(lo, bc, bs);
#pragma unroll
        for (int v = 0; v < 4; ++v) lq[v] += lo[v];
      }
    }
#pragma unroll
    for (int v = 0; v < 4; ++v) sL[side * 4 + v][tid] = lq[v];
  }

  // Phase C: limiter and gradient reverse, one variable at a time
#pragma unroll 1
  for (int v = 0; v < 4; ++v) {
    const T ph = sTr[v][0][tid], gx = sTr[v][1][tid], gy = sTr[v][2][tid];
    LimiterTrace<T> tr;
    tr.sl = sTr[v][3][tid];
    tr.davg = sTr[v][4][tid];
    const int packed = sTi[v][tid];
    tr.sel = packed & 3;
    tr.sign = ((packed >> 2) & 3) - 1;
    tr.clipped = (packed & 16) != 0;
    tr.imax = (packed >> 5) & 7;
    tr.imin = (packed >> 8) & 7;
    T lw0 = T(0), lph = T(0), lhot[4];
#pragma unroll
    for (int s = 0; s < 4; ++s) {
      const T l = sL[s * 4 + v][tid];
      const T hot = gx * hx[s] + gy * hy[s];
      lw0 += l;
      lph += l * hot;
      lhot[s] = l * ph;
    }
    T lst[5] = {T(0), T(0), T(0), T(0), T(0)};  // w0, we, ea, so, no
    if (!tr.clipped) {
      const T lsl = lph * psi_deriv<LIM>(tr.sl);
      T ld = T(0), lden = T(0);
      // a slope in the capped region has psi constant (lsl = 0); its value may be +inf
      // (an FP32 davg below the reciprocal's range), so it passes nothing back
      if (tr.sign != 0 && lsl != T(0)) {
        ld = qdiv(lsl, tr.davg);
        lden = qdiv(-lsl * tr.sl, tr.davg);
      }
      // davg = (w0 + hot) - w0 carries hot through with derivative 1
#pragma unroll
      for (int q = 0; q < 4; ++q) lhot[q] += (q == tr.sel) ? lden : T(0);
      const int im = tr.sign > 0 ? tr.imax : (tr.sign < 0 ? tr.imin : -1);
#pragma unroll
      for (int q = 0; q < 5; ++q) lst[q] += (q == im) ? ld : T(0);
      lw0 -= (im >= 0) ? ld : T(0);
    }
    T lgx = T(0), lgy = T(0);
#pragma unroll
    for (int s = 0; s < 4; ++s) {
      lgx += lhot[s] * hx[s];
      lgy += lhot[s] * hy[s];
    }
    const T lie = (lgx * LcE + lgy * LsE) * ia, liw = -(lgx * LcW + lgy * LsW) * ia;
    const T lin = (lgx * LcN + lgy * LsN) * ia, lis = -(lgx * LcS + lgy * LsS) * ia;
    lw0 += half(lie + liw + lin + lis);
    lst[0] += lw0;
    lst[1] += half(liw);
    lst[2] += half(lie);
    lst[3] += half(lis);
    lst[4] += half(lin);
    st[(ST_SELF * 4 + v) * P.ncell + c] = lst[0];
    st[(ST_W * 4 + v) * P.ncell + c] = lst[1];
    st[(ST_E * 4 + v) * P.ncell + c] = lst[2];
    st[(ST_S * 4 + v) * P.ncell + c] = lst[3];
    st[(ST_N * 4 + v) * P.ncell + c] = lst[4];
  }

  // Phase D: outside states that are the ghost's own value (inter-block and copy
  // sides) pass their adjoint to the ghost's slot
  if (edge) {
    const int side_of[4] = {E2D_W, E2D_E, E2D_S, E2D_N};
    const int slot_of[4] = {ST_W, ST_E, ST_S, ST_N};
    const bool at[4] = {j == 0, j == nx - 1, i == 0, i == ny - 1};
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      if (!at[q]) continue;
      const int side = side_of[q];
      const double *gd, *fd;
      const int kind = side_kind_at(B, side, (side == E2D_E || side == E2D_W) ? i : j, t, gd, fd);
      if (kind != E2D_SIDE_NEIGHBOR && kind != E2D_SIDE_COPY) continue;
      T o[4], lw[4], lo[4];
      if (side == E2D_W) {
        for (int v = 0; v < 4; ++v) o[v] = sW[v][ty + 1][tx];
        load_face(F.vL, P.nvface, fW, lw);
        face_state_vjp<RECON>(o, rotV, cW, sW_, G, lw, lo);
      } else if (side == E2D_E) {
        for (int v = 0; v < 4; ++v) o[v] = sW[v][ty + 1][tx + 2];
        load_face(F.vR, P.nvface, fE, lw);
        face_state_vjp<RECON>(o, rotV, cE, sE, G, lw, lo);
      } else if (side == E2D_S) {
        for (int v = 0; v < 4; ++v) o[v] = sW[v][ty][tx + 1];
        load_face(F.hL, P.nhface, fS, lw);
        face_state_vjp<RECON>(o, rotH, cS, sS, G, lw, lo);
      } else {
        for (int v = 0; v < 4; ++v) o[v] = sW[v][ty + 2][tx + 1];
        load_face(F.hR, P.nhface, fN, lw);
        face_state_vjp<RECON>(o, rotH, cN, sN, G, lw, lo);
      }
#pragma unroll
      for (int v = 0; v < 4; ++v) st[(slot_of[q] * 4 + v) * P.ncell + c] += lo[v];
    }
  }
}

// ---------------------------------------------------------------------------------
// gather + ghost transposes + conservative conversion + RK adjoint program
// ---------------------------------------------------------------------------------
// Contribution of the ghost image of cell c beyond side `side` (position k), or of
// the neighbour block's cell that uses c as its ghost.
template <typename T>
__device__ __forceinline__ void edge_adjoint(const ParamsT<T>& P, const E2DBlock* B, int b, int side, int k,
                                             double t, int64_t c, const T* __restrict__ st, T* lr) {
  const double *gd, *fd;
  const int kind = side_kind_at(B, side, k, t, gd, fd);
  const int own_slot = side == E2D_E ? ST_E : side == E2D_W ? ST_W : side == E2D_N ? ST_N : ST_S;
  if (kind == E2D_SIDE_NEIGHBOR) {
    // the neighbour's opposite side takes its ghosts from this block
    const int opp = side == E2D_E ? E2D_W : side == E2D_W ? E2D_E : side == E2D_N ? E2D_S : E2D_N;
    const int nb = B->neighbor[side];
    const E2DBlock* N = P.blocks + nb;
    const double *gd2, *fd2;
    if (N->neighbor[opp] != b || side_kind_at(N, opp, k, t, gd2, fd2) != E2D_SIDE_NEIGHBOR) return;
    int64_t cn;
    if (side == E2D_E) cn = cell_at(N, k, 0);
    else if (side == E2D_W) cn = cell_at(N, k, N->nx - 1);
    else if (side == E2D_N) cn = cell_at(N, 0, k);
    else cn = cell_at(N, N->ny - 1, k);
    const int nslot = opp == E2D_E ? ST_E : opp == E2D_W ? ST_W : opp == E2D_N ? ST_N : ST_S;
#pragma unroll
    for (int v = 0; v < 4; ++v) lr[v] += st[(nslot * 4 + v) * P.ncell + cn];
    return;
  }
  if (kind == E2D_SIDE_DIRICHLET) return;
  T g[4];
#pragma unroll
  for (int v = 0; v < 4; ++v) g[v] = st[(own_slot * 4 + v) * P.ncell + c];
  if (kind == E2D_SIDE_REFLECT) {
    T cs, sn;
    boundary_cs(P, B, side, k, cs, sn);
    reflect_vjp(g, cs, sn);
  }
#pragma unroll
  for (int v = 0; v < 4; ++v) lr[v] += g[v];
}

template <typename T, int RECON>
__global__ void __launch_bounds__(TX * TY) k_adjoint_gather(ParamsT<T> P, const int4* __restrict__ tiles,
                                                            const T* __restrict__ U,
                                                            const InstanceState* __restrict__ inst,
                                                            const T* __restrict__ st, T* __restrict__ lamU,
                                                            AdjProgramT<T> prog) {
  const int4 tl = tiles[blockIdx.x];
  const E2DBlock* B = P.blocks + tl.x;
  const InstanceState* I = inst + B->instance;
  if (!I->active) return;
  const int ty = threadIdx.x / TX, tx = threadIdx.x - (threadIdx.x / TX) * TX;
  const int i = tl.y + ty, j = tl.z + tx;
  const int nx = B->nx, ny = B->ny;
  if (i >= ny || j >= nx) return;
  const double t = I->t;
  const int64_t c = cell_at(B, i, j);
  T lr[4];
#pragma unroll
  for (int v = 0; v < 4; ++v) lr[v] = st[(ST_SELF * 4 + v) * P.ncell + c];
  // the east neighbour holds this cell as its W value, and so on
  if (j + 1 < nx) {
    const int64_t o = cell_at(B, i, j + 1);
#pragma unroll
    for (int v = 0; v < 4; ++v) lr[v] += st[(ST_W * 4 + v) * P.ncell + o];
  } else {
    edge_adjoint(P, B, tl.x, E2D_E, i, t, c, st, lr);
  }
  if (j > 0) {
    const int64_t o = cell_at(B, i, j - 1);
#pragma unroll
    for (int v = 0; v < 4; ++v) lr[v] += st[(ST_E * 4 + v) * P.ncell + o];
  } else {
    edge_adjoint(P, B, tl.x, E2D_W, i, t, c, st, lr);
  }
  if (i + 1 < ny) {
    const int64_t o = cell_at(B, i + 1, j);
#pragma unroll
    for (int v = 0; v < 4; ++v) lr[v] += st[(ST_S * 4 + v) * P.ncell + o];
  } else {
    edge_adjoint(P, B, tl.x, E2D_N, j, t, c, st, lr);
  }
  if (i > 0) {
    const int64_t o = cell_at(B, i - 1, j);
#pragma unroll
    for (int v = 0; v < 4; ++v) lr[v] += st[(ST_N * 4 + v) * P.ncell + o];
  } else {
    edge_adjoint(P, B, tl.x, E2D_S, j, t, c, st, lr);
  }
  T ly[4];
  if (RECON == E2D_RECON_PRIMITIVE) {
    T q[4];
    load_cell(U, P.ncell, c, q);
    const Gas<T> G{P.gas[0], P.gas[1], P.gas[2], P.gas[3]};
    ly[0] = T(0); ly[1] = T(0); ly[2] = T(0); ly[3] = T(0);
    cons_to_prim_vjp(q, G, lr, ly);
  } else {
    ly[0] = lr[0]; ly[1] = lr[1]; ly[2] = lr[2]; ly[3] = lr[3];
  }
#pragma unroll
  for (int v = 0; v < 4; ++v) lamU[v * P.ncell + c] += ly[v];
#pragma unroll
  for (int q = 0; q < MAX_STAGES; ++q) {
    if (q >= prog.n) break;
    T* d = prog.dst[q];
    const T a = T(prog.coef[q]);
#pragma unroll
    for (int v = 0; v < 4; ++v) d[v * P.ncell + c] += a * ly[v];
  }
}

// acc[q] = coef[q] * lam for every stage q (start of an RK step's reverse)
template <typename T>
__global__ void k_adjoint_init(int64_t n, const T* __restrict__ lam, AdjProgramT<T> prog) {
  for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < n; x += (int64_t)gridDim.x * blockDim.x) {
    const T l = lam[x];
#pragma unroll
    for (int q = 0; q < MAX_STAGES; ++q) {
      if (q >= prog.n) break;
      prog.dst[q][x] = T(prog.coef[q]) * l;
    }
  }
}

// ---------------------------------------------------------------------------------
// objective: P(U) = sum over the cells along one block side of p * (boundary face
// length); one CTA, fixed reduction order
// ---------------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ void side_cell_face(const E2DBlock* B, int side, int k, int64_t& c, int64_t& f,
                                               bool& vertical) {
  if (side == E2D_E) { c = cell_at(B, k, B->nx - 1); f = vf_at(B, k, B->nx); vertical = true; }
  else if (side == E2D_W) { c = cell_at(B, k, 0); f = vf_at(B, k, 0); vertical = true; }
  else if (side == E2D_N) { c = cell_at(B, B->ny - 1, k); f = hf_at(B, B->ny, k); vertical = false; }
  else { c = cell_at(B, 0, k); f = hf_at(B, 0, k); vertical = false; }
}

constexpr int OBJ_THREADS = 256;

// *J += dt * P(U), dt from instance 0 (the step just taken)
template <typename T>
__global__ void __launch_bounds__(OBJ_THREADS) k_side_pressure(ParamsT<T> P, int b, int side, const T* __restrict__ U,
                                                               const InstanceState* __restrict__ inst,
                                                               double* __restrict__ J) {
  const E2DBlock* B = P.blocks + b;
  const int n = (side == E2D_E || side == E2D_W) ? B->ny : B->nx;
  const Gas<T> G{P.gas[0], P.gas[1], P.gas[2], P.gas[3]};
  double acc = 0.0;
  for (int k = threadIdx.x; k < n; k += OBJ_THREADS) {
    int64_t c, f;
    bool vert;
    side_cell_face<T>(B, side, k, c, f, vert);
    T q[4], w[4];
    load_cell(U, P.ncell, c, q);
    cons_to_prim(q, G, w);
    const T len = vert ? P.geo.vface[E2D_F_L][f] : P.geo.hface[E2D_F_L][f];
    acc += double(w[3]) * double(len);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  __shared__ double part[OBJ_THREADS / 32];
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = part[0];
    for (int w = 1; w < OBJ_THREADS / 32; ++w) s += part[w];
    *J += inst[0].dt * s;
  }
}

// lam += coef * dP/dU
template <typename T>
__global__ void k_side_pressure_grad(ParamsT<T> P, int b, int side, const T* __restrict__ U, double coef,
                                     T* __restrict__ lam) {
  const E2DBlock* B = P.blocks + b;
  const int n = (side == E2D_E || side == E2D_W) ? B->ny : B->nx;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  int64_t c, f;
  bool vert;
  side_cell_face<T>(B, side, k, c, f, vert);
  const T len = vert ? P.geo.vface[E2D_F_L][f] : P.geo.hface[E2D_F_L][f];
  const T rho = U[c], u = qdiv(U[P.ncell + c], rho), v = qdiv(U[2 * P.ncell + c], rho);
  const T g = T(coef) * len * P.gas[1];
  lam[c] += half(g) * (u * u + v * v);
  lam[P.ncell + c] -= g * u;
  lam[2 * P.ncell + c] -= g * v;
  lam[3 * P.ncell + c] += g;
}

// record the dt and t of the step about to be taken (instance 0)
__global__ void k_record_step(const InstanceState* __restrict__ inst, double* dts, double* ts, int n) {
  dts[n] = inst[0].dt;
  ts[n] = inst[0].t;
}

}  // namespace e2d
