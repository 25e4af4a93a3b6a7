// e2d_fused.cuh - the fused stage kernel: one launch per Runge-Kutta stage does what
// k_reconstruct, k_flux and k_update do in three, with the face states and fluxes kept
// in shared memory instead of face arrays in HBM (pyhype/fvm/base.py:108-190 for one
// stage of every block, plus the stage's Butcher updates of
// time_marching/explicit_runge_kutta.py:63-80).
//
// One CTA of NW warps takes a tile of FTY rows x 32 columns of one block (two shapes:
// 28 rows with 16 warps, 13 rows with 8 warps; in both the tile rows and the ring tasks
// fill whole rounds of warps, so no warp idles through a reconstruction round):
//   staging   the tile and a 2-cell halo (FTY + 4 rows x 36 columns, 4 planes) into shared memory:
//             one TMA box load for tiles whose halo lies inside the block, plain loads
//             with ghost cells formed on the fly (ghost_cons) for the others;
//   faces     gradient and limiter of every tile cell and of the ring of cells around
//             it (whose face states the tile's edge faces need); each tile cell
//             writes its four limited face states, each ring cell the one facing the
//             tile, rotated into the face frame and converted to primitive variables;
//             block-boundary faces take their outside state from the boundary condition
//             (outside_state), as in k_reconstruct;
//   fluxes    one Riemann flux per face of the tile, rotated back and integrated,
//             written over the face's left state;
//   update    dUdt of every tile cell and the stage program (partial Butcher sums,
//             Kahan-compensated last row on the FP32 path), positivity on the last stage.
// Every value is computed by the same functions the split kernels use
// (limit_cell4, vface_prim/hface_prim, vface_flux/hface_flux, cell_dudt,
// stage_program), so the two forms give the same results.
//
// The cost of fusion is the ring: gradient and limiter of the 2 (32 + FTY) ring cells
// are computed by both tiles that share them (13 % more reconstruction work at 28 rows,
// 22 % at 13), and the tile's edge faces by both tiles.  What it saves is the face
// arrays' round trip through HBM (four states and two fluxes per face) and two launches.
//
// A stage whose Butcher updates write its own input buffer (explicit Euler, a one-stage
// tableau) cannot be fused: a tile would overwrite cells that its neighbours still read
// as halo.  The host runs such stages split (E2DSolver::fusable).
#pragma once
#include "e2d_stage.cuh"

namespace e2d {

template <typename T, int FTY>
struct FusedSmem {
  // tile + 2-cell halo in reconstruction variables; block row i0 - 2 + r at row r,
  // block column j0 - XO + c at column c (XO = 16 / sizeof(T), the TMA box's start)
  T sW[4][FTY + 4][TileCols<T>::TXW];
  // face states, family 0 the vertical faces (row i0 + r, face column j0 + c; r < FTY,
  // c <= TX), family 1 the horizontal ones (face row i0 + r, column j0 + c; r <= FTY,
  // c < TX): left and right primitive state in the face frame; after the flux phase L
  // holds the integrated flux.  Both families take the same padded plane shape, so a
  // face's variables sit at fixed offsets from one address whatever its family.
  T L[2][4][FTY + 1][TX + 1];
  T R[2][4][FTY + 1][TX + 1];
};

// L2 prefetch of elements [first, last] of one plane, a line at a time (every address
// inside the plane; a bulk prefetch per range measured slower).
template <typename T>
__device__ __forceinline__ void prefetch_l2(const T* plane, int64_t first, int64_t last) {
  const char* p = reinterpret_cast<const char*>(plane);
  for (int64_t b = (first * (int64_t)sizeof(T)) & ~(int64_t)127; b <= last * (int64_t)sizeof(T); b += 128)
    asm volatile("prefetch.global.L2 [%0];" ::"l"(p + b));
}

template <typename T, int R, int C>
__device__ __forceinline__ void put4(T (&a)[4][R][C], int r, int c, const T* w) {
  a[0][r][c] = w[0]; a[1][r][c] = w[1]; a[2][r][c] = w[2]; a[3][r][c] = w[3];
}

enum { FACE_E = 1, FACE_W = 2, FACE_N = 4, FACE_S = 8 };

// The tile's first cell (i0, j0) and its west and south faces in the planes, and the
// block's shape: read from the block descriptor once per CTA, where each index
// computation would otherwise load them from global memory again.
struct TileOrigin {
  int64_t c0, vf0, hf0;
  int nx, ny;
  bool cart;
  __device__ __forceinline__ int64_t cell(int lr, int lc) const { return c0 + (int64_t)lr * nx + lc; }
  __device__ __forceinline__ int64_t vface(int lr, int lc) const { return vf0 + (int64_t)lr * (nx + 1) + lc; }
  __device__ __forceinline__ int64_t hface(int lr, int lc) const { return hf0 + (int64_t)lr * nx + lc; }
};

// Gradient, limiter and the face states `which` of the cell at tile-local (lr, lc),
// lr in [-1, FTY], lc in [-1, TX]; a tile cell (own = true) also writes the outside
// states of its block-boundary faces.
template <typename T, int LIM, int RECON, int FTY, bool CART>
__device__ __forceinline__ void fused_cell(const ParamsT<T>& P, const Gas<T>& G, const E2DBlock* B,
                                           const TileOrigin& to, FusedSmem<T, FTY>& sm, int i0, int j0, int lr,
                                           int lc, int which, bool own, double t) {
  constexpr int XO = TileCols<T>::XO;
  const int i = i0 + lr, j = j0 + lc;
  const int sr = lr + 2, sc = XO + lc;  // the cell's position in sW
  const int64_t fW = to.vface(lr, lc), fE = fW + 1;
  const int64_t fS = to.hface(lr, lc), fN = fS + to.nx;
  // the FP32 form on a block it takes as Cartesian: the gradient and the face
  // differences without cross-axis terms (limit_cell4); compiled in for the Cartesian
  // variant, chosen per block in the general one
  constexpr bool F32 = sizeof(T) == 4;
  CellGeo<T> g;
  T face[4][4];
  {
    // stencil points: the cell, W, E, S, N
    auto st = [&](int v, int p) -> T {
      return sm.sW[v][sr + (p == 3 ? -1 : p == 4 ? 1 : 0)][sc + (p == 1 ? -1 : p == 2 ? 1 : 0)];
    };
    T gx[4], gy[4], ph[4];
    load_cell_geo_at<T, CART && F32>(P, to.cell(lr, lc), fW, fS, to.nx, g);
    limit_cell4<T, LIM, CART && F32>(st, g, face, gx, gy, ph, F32 && to.cart);
  }
  const bool cart = CART || to.cart;
  // the frames of the faces to write, read before the first store
  T fc[4] = {T(1), T(1), T(0), T(0)}, fs[4] = {T(0), T(0), T(1), T(1)};
  if (!cart) {
    if (which & FACE_E) { fc[0] = P.geo.vface[E2D_F_COS][fE]; fs[0] = P.geo.vface[E2D_F_SIN][fE]; }
    if (which & FACE_W) { fc[1] = P.geo.vface[E2D_F_COS][fW]; fs[1] = P.geo.vface[E2D_F_SIN][fW]; }
    if (which & FACE_N) { fc[2] = P.geo.hface[E2D_F_COS][fN]; fs[2] = P.geo.hface[E2D_F_SIN][fN]; }
    if (which & FACE_S) { fc[3] = P.geo.hface[E2D_F_COS][fS]; fs[3] = P.geo.hface[E2D_F_SIN][fS]; }
  }
  T w[4];
  if (which & FACE_E) { vface_prim_cs<T, RECON>(G, cart, fc[0], fs[0], face[E2D_E], w); put4(sm.L[0], lr, lc + 1, w); }
  if (which & FACE_W) { vface_prim_cs<T, RECON>(G, cart, fc[1], fs[1], face[E2D_W], w); put4(sm.R[0], lr, lc, w); }
  if (which & FACE_N) { hface_prim_cs<T, RECON>(G, cart, fc[2], fs[2], face[E2D_N], w); put4(sm.L[1], lr + 1, lc, w); }
  if (which & FACE_S) { hface_prim_cs<T, RECON>(G, cart, fc[3], fs[3], face[E2D_S], w); put4(sm.R[1], lr, lc, w); }
  if (!own) return;
  // outside states of block-boundary faces (the ghost cell is staged next to the cell)
  if (j == 0) {
    const T gr[4] = {sm.sW[0][sr][sc - 1], sm.sW[1][sr][sc - 1], sm.sW[2][sr][sc - 1], sm.sW[3][sr][sc - 1]};
    T o[4];
    outside_state(P, B, E2D_W, i, t, gr, face[E2D_W], o);
    vface_prim<T, RECON>(P, G, cart, fW, o, w);
    put4(sm.L[0], lr, lc, w);
  }
  if (j == to.nx - 1) {
    const T gr[4] = {sm.sW[0][sr][sc + 1], sm.sW[1][sr][sc + 1], sm.sW[2][sr][sc + 1], sm.sW[3][sr][sc + 1]};
    T o[4];
    outside_state(P, B, E2D_E, i, t, gr, face[E2D_E], o);
    vface_prim<T, RECON>(P, G, cart, fE, o, w);
    put4(sm.R[0], lr, lc + 1, w);
  }
  if (i == 0) {
    const T gr[4] = {sm.sW[0][sr - 1][sc], sm.sW[1][sr - 1][sc], sm.sW[2][sr - 1][sc], sm.sW[3][sr - 1][sc]};
    T o[4];
    outside_state(P, B, E2D_S, j, t, gr, face[E2D_S], o);
    hface_prim<T, RECON>(P, G, cart, fS, o, w);
    put4(sm.L[1], lr, lc, w);
  }
  if (i == to.ny - 1) {
    const T gr[4] = {sm.sW[0][sr + 1][sc], sm.sW[1][sr + 1][sc], sm.sW[2][sr + 1][sc], sm.sW[3][sr + 1][sc]};
    T o[4];
    outside_state(P, B, E2D_N, j, t, gr, face[E2D_N], o);
    hface_prim<T, RECON>(P, G, cart, fN, o, w);
    put4(sm.R[1], lr + 1, lc, w);
  }
}

// Everything of the tile that the stage reads from global memory besides the staged
// state, prefetched into L2 by the whole CTA at its start: the cell geometry of the
// tile and its ring (area, 1/A, the face points' offsets), the face geometry of their
// faces (length, L cos, L sin, and the frames of a curvilinear block), and the stage
// program's sources for the tile's cells.  The geometry planes are larger than L2 and
// come from HBM every stage; prefetched, the reconstruction's loads wait for L2
// instead of HBM.  Rows and columns are clamped to the block.
template <typename T, int FTY, int NU, bool CART>
__device__ void prefetch_tile(const ParamsT<T>& P, const TileOrigin& to, int i0, int j0,
                              const StateBuffersT<T>& S, const StageProgram& prog) {
  // items by constant-sized groups (divisions by constants): cell planes x FTY + 2
  // rows, face planes x FTY + 2 (vertical) or FTY + 3 (horizontal) rows, source
  // planes x FTY rows; rows outside the block are skipped.  A Cartesian variant reads
  // no face frames, so it prefetches 3 face planes, not 5; in FP32 it reads no
  // cross-axis components either (load_cell_geo_at): A, 1/A, the east and west
  // points' x offsets and the north and south points' y offsets, and per face family
  // L and its normal's own-axis component.
  constexpr bool AX = CART && sizeof(T) == 4;
  constexpr int NCP = AX ? 6 : 10, NF = AX ? 2 : CART ? 3 : 5;
  constexpr int RR = FTY + 2, NCI = NCP * RR, NVI = NF * RR, NHI = NF * (RR + 1);
  const int r_lo = (i0 >= 1 ? -1 : 0), r_hi = min(FTY, to.ny - 1 - i0);  // tile rows and the ring, local
  const int c_lo = (j0 >= 1 ? -1 : 0), c_hi = min(TX, to.nx - 1 - j0);
  const int nfp = AX ? 2 : (CART || to.cart) ? 3 : 5;  // face planes: L, L cos, L sin (, cos, sin)
  const int tr = min(FTY, to.ny - i0), tc = min(TX, to.nx - j0);  // the tile's own cells
  int nsrc = 0;  // source plane sets: each update's source, and U^n and its compensation for a Kahan update
#pragma unroll
  for (int u = 0; u < NU; ++u) {
    if (u >= prog.nupd) break;
    nsrc += (prog.upd[u].src_zero ? 0 : 1) + (prog.upd[u].kahan ? 2 : 0);
  }
  const int total = NCI + NVI + NHI + nsrc * 4 * FTY;
  for (int it = threadIdx.x; it < total; it += blockDim.x) {
    if (it < NCI) {  // A, 1/A and the offsets (E2D_G_A .. E2D_G_HY_S; AX: HX_E, HX_W, HY_N, HY_S)
      const int k = it / RR, r = it - k * RR - 1;
      const int plane = (AX && k >= 4) ? k + 4 : k;
      if (r >= r_lo && r <= r_hi) prefetch_l2(P.geo.cell[plane], to.cell(r, c_lo), to.cell(r, c_hi));
    } else if (it < NCI + NVI) {  // L, L cos (, L sin, cos, sin)
      const int q = it - NCI, k = q / RR, r = q - k * RR - 1;
      if (k < nfp && r >= r_lo && r <= r_hi) prefetch_l2(P.geo.vface[k], to.vface(r, c_lo), to.vface(r, c_hi + 1));
    } else if (it < NCI + NVI + NHI) {  // L, L cos, L sin (, cos, sin); AX: L, L sin
      const int q = it - NCI - NVI, k = q / (RR + 1), r = q - k * (RR + 1) - 1;
      const int plane = (AX && k == 1) ? (int)E2D_F_LS : k;
      if (k < nfp && r >= r_lo && r <= r_hi + 1) prefetch_l2(P.geo.hface[plane], to.hface(r, c_lo), to.hface(r, c_hi));
    } else {
      const int q = it - NCI - NVI - NHI, v = (q / FTY) & 3, r = q - (q / FTY) * FTY;
      int n = q / (4 * FTY);  // the n-th source plane set
      const T* base = nullptr;
#pragma unroll
      for (int u = 0; u < NU; ++u) {
        if (u >= prog.nupd || base != nullptr) break;
        const StageUpdate& up = prog.upd[u];
        if (!up.src_zero) {
          if (n == 0) base = static_cast<const T*>(up.srcp);
          --n;
        }
        if (up.kahan && base == nullptr) {
          if (n == 0) base = S.comp;
          else if (n == 1) base = S.buf[0];
          n -= 2;
        }
      }
      if (base != nullptr && r < tr) prefetch_l2(base + (int64_t)v * P.ncell, to.cell(r, 0), to.cell(r, tc - 1));
    }
  }
}

// REC: record for the adjoint; CART: every block Cartesian (block_cart); FINAL: the
// stage is the step's last (1), is not (0), or reads it from the program (2); NU: the
// stage has at most NU updates
template <typename T, int LIM, int RECON, int FLUX, int FTY, int NW, int MINB, bool REC, bool CART, int FINAL, int NU>
__global__ void __launch_bounds__(NW * 32, MINB)
    k_stage_fused(ParamsT<T> P, const int4* __restrict__ tiles, const T* __restrict__ U,
                  InstanceState* __restrict__ inst, StateBuffersT<T> S, StageProgram prog,
                  RealizState* __restrict__ real, TmaTiles tma, FusedRecordT<T> rec) {
  constexpr int FTHREADS = NW * 32;
  constexpr int RING_COL_TASKS = (2 * FTY + 31) / 32;  // the W and E ring columns, 32 cells a task
  static_assert(FTY + 2 + RING_COL_TASKS <= 2 * NW, "tile rows and ring tasks must fill two rounds of warps");
  extern __shared__ __align__(128) unsigned char e2d_fused_smem[];
  FusedSmem<T, FTY>& sm = *reinterpret_cast<FusedSmem<T, FTY>*>(e2d_fused_smem);
  __shared__ __align__(8) unsigned long long bar;
  constexpr int XO = TileCols<T>::XO;
  const Gas<T> G{P.gas[0], P.gas[1], P.gas[2], P.gas[3]};
  const int4 tl = tiles[blockIdx.x];
  const E2DBlock* B = P.blocks + tl.x;
  const InstanceState* I = inst + B->instance;
  if (!I->active) return;  // uniform over the CTA
  const double t = I->t;
  const int nx = B->nx, ny = B->ny;
  const int i0 = tl.y, j0 = tl.z;
  const TileOrigin to{cell_at(B, i0, j0), vf_at(B, i0, j0), hf_at(B, i0, j0), nx, ny, block_cart(P, B, tl.x)};
  prefetch_tile<T, FTY, NU, CART>(P, to, i0, j0, S, prog);
  // the halo lies inside the block: no ghost cell is staged and every ring cell is real
  const bool interior = i0 >= 2 && j0 >= 2 && i0 + FTY + 2 <= ny && j0 + TX + 2 <= nx;

  // ---- staging ---------------------------------------------------------------------
  if (interior && tma.maps != nullptr && tma.ok[tl.x]) {
    if (threadIdx.x == 0) {
      mbar_init(&bar);
      tma_load_box(&sm.sW[0][0][0], &tma.maps[tl.x], j0 - XO, i0 - 2, 0, &bar, (unsigned)sizeof(sm.sW));
    }
    __syncthreads();  // the barrier is initialised before anyone waits on it
    if (!__syncthreads_and(mbar_wait(&bar, 0))) {
      // the wait ran out: report it and drop the tile (the host fails the step); wait once
      // more, as long again, so that the CTA does not exit while the copy is landing
      if (threadIdx.x == 0) atomicAdd(tma.timeouts, 1ULL);
      __syncthreads_and(mbar_wait(&bar, 0));
      return;
    }
    if (RECON == E2D_RECON_PRIMITIVE) {  // conversion in place, one thread per staged cell
      for (int p = threadIdx.x; p < (FTY + 4) * (TX + 4); p += FTHREADS) {
        const int ly = p / (TX + 4), lx = p - ly * (TX + 4);
        const int c = XO - 2 + lx;
        T q[4] = {sm.sW[0][ly][c], sm.sW[1][ly][c], sm.sW[2][ly][c], sm.sW[3][ly][c]}, r[4];
        to_recon<RECON>(q, G, r);
        sm.sW[0][ly][c] = r[0]; sm.sW[1][ly][c] = r[1]; sm.sW[2][ly][c] = r[2]; sm.sW[3][ly][c] = r[3];
      }
    }
  } else {
    for (int p = threadIdx.x; p < (FTY + 4) * (TX + 4); p += FTHREADS) {
      const int ly = p / (TX + 4), lx = p - ly * (TX + 4);
      const int gi = i0 + ly - 2, gj = j0 + lx - 2;
      T q[4], r[4] = {T(0), T(0), T(0), T(0)};
      if (interior) {
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
      const int c = XO - 2 + lx;
      sm.sW[0][ly][c] = r[0]; sm.sW[1][ly][c] = r[1]; sm.sW[2][ly][c] = r[2]; sm.sW[3][ly][c] = r[3];
    }
  }
  __syncthreads();

  // ---- face states: tile rows, then the ring (S row, N row, W and E columns) ---------
  // One call site for every kind of task (the reconstruction is the kernel's largest
  // piece of code; four inlined copies of it crowded the instruction cache).
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int task = warp; task < FTY + 2 + RING_COL_TASKS; task += NW) {
    int lr, lc, which;
    bool live;
    if (task < FTY) {  // a tile row: all four faces, and block-boundary outside states
      lr = task;
      lc = lane;
      which = FACE_E | FACE_W | FACE_N | FACE_S;
      live = i0 + lr < ny && j0 + lc < nx;
    } else if (task == FTY) {  // the ring row below the tile: its north faces
      lr = -1;
      lc = lane;
      which = FACE_N;
      live = i0 >= 1 && j0 + lc < nx;
    } else if (task == FTY + 1) {  // the ring row above: its south faces
      lr = FTY;
      lc = lane;
      which = FACE_S;
      live = i0 + FTY < ny && j0 + lc < nx;
    } else {  // the ring columns: west (ring cells 0..FTY-1: east faces), then east (west faces)
      const int q = (task - FTY - 2) * 32 + lane;
      const bool east = q >= FTY;
      lr = east ? q - FTY : q;
      lc = east ? TX : -1;
      which = east ? FACE_W : FACE_E;
      live = q < 2 * FTY && i0 + lr < ny && (east ? j0 + TX < nx : j0 >= 1);
    }
    if (live) fused_cell<T, LIM, RECON, FTY, CART>(P, G, B, to, sm, i0, j0, lr, lc, which, task < FTY, t);
  }
  __syncthreads();

  // ---- one flux per face of the tile (one call site for both face families) ---------
  {
    const bool cart = CART || to.cart;
    // a warp per row of faces: the horizontal face rows 0..FTY, the vertical face rows
    // 0..FTY-1 (columns 0..31), then the tile's east edge (column TX, 32 rows a job)
    constexpr int NJ = (FTY + 1) + FTY + (FTY + 31) / 32;
    for (int job = warp; job < NJ; job += NW) {
      int r, c;
      const bool vert = job > FTY;
      if (!vert) {
        r = job;
        c = lane;
      } else if (job <= 2 * FTY) {
        r = job - FTY - 1;
        c = lane;
      } else {
        r = (job - 2 * FTY - 1) * 32 + lane;
        c = TX;
      }
      const int fam = vert ? 0 : 1;
      const bool live = vert ? (r < FTY && i0 + r < ny && j0 + c <= nx) : (i0 + r <= ny && j0 + c < nx);
      if (!live) continue;
      const int64_t f = vert ? to.vface(r, c) : to.hface(r, c);
      T L[4], R[4];
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        L[v] = sm.L[fam][v][r][c];
        R[v] = sm.R[fam][v][r][c];
      }
      if (REC && rec.vL) {  // the face states for the adjoint, where the split reconstruction puts them
        T* rl = vert ? rec.vL : rec.hL;
        T* rr = vert ? rec.vR : rec.hR;
        const int64_t nf = vert ? P.nvface : P.nhface;
#pragma unroll
        for (int v = 0; v < 4; ++v) {
          rl[v * nf + f] = L[v];
          rr[v * nf + f] = R[v];
        }
      }
      T Fq[4];
      riemann<FLUX>(L, R, G, Fq);
      // rotated back to the x/y frame and integrated, as vface_flux / hface_flux
      const T* cosp = vert ? P.geo.vface[E2D_F_COS] : P.geo.hface[E2D_F_COS];
      const T* sinp = vert ? P.geo.vface[E2D_F_SIN] : P.geo.hface[E2D_F_SIN];
      const T* lenp = vert ? P.geo.vface[E2D_F_L] : P.geo.hface[E2D_F_L];
      if (!vert && cart) unrotate90(Fq);
      else if (!cart) unrotate(Fq, cosp[f], sinp[f]);
      const T len = lenp[f];
#pragma unroll
      for (int v = 0; v < 4; ++v) sm.L[fam][v][r][c] = len * twice(Fq[v]);
    }
  }
  __syncthreads();

  // ---- dUdt and the stage program of every tile cell --------------------------------
  const bool final_stage = FINAL == 2 ? prog.final_stage != 0 : FINAL == 1;
  int nbad = 0;
#pragma unroll
  for (int round = 0; round < (FTY + NW - 1) / NW; ++round) {  // every thread runs every round
    const int r = warp + round * NW;
    const int i = i0 + r, j = j0 + lane;
    bool bad = false;
    if (r < FTY && i < ny && j < nx) {
      const int64_t c = to.cell(r, lane);
      if (REC && rec.y) {  // the stage's input state for the adjoint
#pragma unroll
        for (int v = 0; v < 4; ++v) rec.y[v * P.ncell + c] = U[v * P.ncell + c];
      }
      const T A = P.geo.cell[E2D_G_A][c];
      const T iA = sizeof(T) == 8 ? P.geo.cell[E2D_G_INV_A][c] : T(0);
      T k[4];
#pragma unroll
      for (int v = 0; v < 4; ++v) k[v] = cell_dudt(sm.L[0][v][r][lane], sm.L[0][v][r][lane + 1], sm.L[1][v][r][lane],
                                                   sm.L[1][v][r + 1][lane], A, iA);
      stage_program<T, NU>(P, S, prog, I->dt, c, k);
      if (final_stage) {
        const T rho = S.buf[0][c], E = S.buf[0][3 * P.ncell + c];
        bad = !(rho > T(0)) || !(E > T(0));
        if (bad) atomicMin(&real->first, ((unsigned long long)tl.x << 40) | (unsigned long long)(c - B->cell_offset));
      }
    }
    if (final_stage) nbad += __syncthreads_count(bad);
  }
  if (final_stage && threadIdx.x == 0 && nbad) {
    atomicAdd(&real->nbad, (unsigned long long)nbad);
    atomicAdd(&inst[B->instance].nbad, nbad);  // halts this instance only
  }
}

// ---- launchers --------------------------------------------------------------------------
template <typename T, int LIM, int RECON, int FLUX, int FORM>
static cudaError_t fused_launch(const ParamsT<T>& P, const TileSet& ts, const T* U, InstanceState* inst,
                                StateBuffersT<T> S, const StageProgram& prog, RealizState* real, cudaStream_t st,
                                const TmaSet* tset, bool prepare_only, const FusedRecordT<T>& rec) {
  constexpr int FTY = FUSED_TY[FORM], NW = FUSED_WARPS[FORM];
  // CTAs an SM holds at 64 registers a thread (FP32) or 128 (FP64): 65536 / (regs x NW x 32)
  constexpr int MINB = (sizeof(T) == 4 ? 32 : 16) / NW;
  // variants: any blocks (everything read at run time); all blocks Cartesian, and for
  // FP32 also the stage's place and update count compiled in; recording for the adjoint
  // (FP32 only: the adjoint recomputes FP64 segments split)
  constexpr bool F32 = sizeof(T) == 4;
  auto kern = k_stage_fused<T, LIM, RECON, FLUX, FTY, NW, MINB, false, false, 2, MAX_STAGES>;
  auto kern_cart = k_stage_fused<T, LIM, RECON, FLUX, FTY, NW, MINB, false, true, 2, MAX_STAGES>;
  auto kern_c0 = k_stage_fused<T, LIM, RECON, FLUX, FTY, NW, MINB, false, true, F32 ? 0 : 2, F32 ? 2 : MAX_STAGES>;
  auto kern_c1 = k_stage_fused<T, LIM, RECON, FLUX, FTY, NW, MINB, false, true, F32 ? 1 : 2, F32 ? 2 : MAX_STAGES>;
  auto kern_rec = k_stage_fused<T, LIM, RECON, FLUX, FTY, NW, MINB, F32, false, 2, MAX_STAGES>;
  auto kern_rec_cart = k_stage_fused<T, LIM, RECON, FLUX, FTY, NW, MINB, F32, true, 2, MAX_STAGES>;
  constexpr int bytes = (int)sizeof(FusedSmem<T, FTY>);
  if (prepare_only) {
    cudaError_t e = cudaSuccess;
    for (auto k : {kern, kern_cart, kern_c0, kern_c1, kern_rec, kern_rec_cart})
      if (e == cudaSuccess) e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    return e;
  }
  const TmaTiles tma = tset ? tset->fused[FORM] : TmaTiles{nullptr, nullptr, nullptr};
  if (ts.nfused[FORM] <= 0) return cudaSuccess;
  const bool record = rec.y != nullptr || rec.vL != nullptr;
  if (record && !F32) return cudaErrorInvalidValue;
  auto k = record ? (ts.all_cartesian ? kern_rec_cart : kern_rec)
                  : !ts.all_cartesian ? kern
                  : (F32 && prog.nupd <= 2) ? (prog.final_stage ? kern_c1 : kern_c0) : kern_cart;
  k<<<ts.nfused[FORM], NW * 32, bytes, st>>>(P, ts.fused[FORM], U, inst, S, resolve_program(prog, S), real, tma, rec);
  return cudaGetLastError();
}

template <typename T, int LIM, int RECON, int FLUX>
static cudaError_t fused_form(const ParamsT<T>& P, const TileSet& ts, int form, const T* U, InstanceState* inst,
                              StateBuffersT<T> S, const StageProgram& prog, RealizState* real, cudaStream_t st,
                              const TmaSet* tma, bool prepare_only, const FusedRecordT<T>& rec) {
  if (form == 2) return fused_launch<T, LIM, RECON, FLUX, 1>(P, ts, U, inst, S, prog, real, st, tma, prepare_only, rec);
  return fused_launch<T, LIM, RECON, FLUX, 0>(P, ts, U, inst, S, prog, real, st, tma, prepare_only, rec);
}

template <typename T, int LIM>
cudaError_t fused_lim(const ParamsT<T>& P, const TileSet& ts, int form, const T* U, InstanceState* inst,
                      StateBuffersT<T> S, const StageProgram& prog, RealizState* real, cudaStream_t st,
                      const TmaSet* tma, bool prepare_only, const FusedRecordT<T>& rec) {
#define E2D_FUSED_FLUX(RC)                                                                                          \
  switch (P.flux) {                                                                                                 \
    case E2D_FLUX_HLLL: return fused_form<T, LIM, RC, E2D_FLUX_HLLL>(P, ts, form, U, inst, S, prog, real, st, tma, prepare_only, rec); \
    case E2D_FLUX_HLLE: return fused_form<T, LIM, RC, E2D_FLUX_HLLE>(P, ts, form, U, inst, S, prog, real, st, tma, prepare_only, rec); \
    default: return fused_form<T, LIM, RC, E2D_FLUX_ROE>(P, ts, form, U, inst, S, prog, real, st, tma, prepare_only, rec);   \
  }
  if (P.recon == E2D_RECON_PRIMITIVE) {
    E2D_FUSED_FLUX(E2D_RECON_PRIMITIVE)
  }
  E2D_FUSED_FLUX(E2D_RECON_CONSERVATIVE)
#undef E2D_FUSED_FLUX
}

#define E2D_FUSED_LIM_DECL(PRE, T, LIM)                                                                           \
  PRE template cudaError_t fused_lim<T, LIM>(const ParamsT<T>&, const TileSet&, int, const T*, InstanceState*,    \
                                             StateBuffersT<T>, const StageProgram&, RealizState*, cudaStream_t,   \
                                             const TmaSet*, bool, const FusedRecordT<T>&);
#define E2D_EXTERN_FUSED_LIM(T)    \
  E2D_FUSED_LIM_DECL(extern, T, 0) \
  E2D_FUSED_LIM_DECL(extern, T, 1) \
  E2D_FUSED_LIM_DECL(extern, T, 2) \
  E2D_FUSED_LIM_DECL(extern, T, 3)

// One stage (one-point face rule) in one launch at stage form `form` (1: FUSED_TY[0]
// rows, 2: FUSED_TY[1] rows); prepare_only sets the kernel's shared memory limit and
// launches nothing (done once when a handle is created, outside any stream capture).
template <typename T>
cudaError_t launch_stage_fused(const ParamsT<T>& P, const TileSet& ts, int form, const T* U, InstanceState* inst,
                               StateBuffersT<T> S, const StageProgram& prog, RealizState* real, cudaStream_t st,
                               const TmaSet* tma, bool prepare_only, const FusedRecordT<T>& rec) {
  switch (P.limiter) {
    case E2D_LIM_BARTH_JESPERSEN:
      return fused_lim<T, E2D_LIM_BARTH_JESPERSEN>(P, ts, form, U, inst, S, prog, real, st, tma, prepare_only, rec);
    case E2D_LIM_VAN_ALBADA:
      return fused_lim<T, E2D_LIM_VAN_ALBADA>(P, ts, form, U, inst, S, prog, real, st, tma, prepare_only, rec);
    case E2D_LIM_VAN_LEER: return fused_lim<T, E2D_LIM_VAN_LEER>(P, ts, form, U, inst, S, prog, real, st, tma, prepare_only, rec);
    default: return fused_lim<T, E2D_LIM_VENKATAKRISHNAN>(P, ts, form, U, inst, S, prog, real, st, tma, prepare_only, rec);
  }
}

#define E2D_INSTANTIATE_FUSED_LAUNCHER(T)                                                                        \
  template cudaError_t launch_stage_fused<T>(const ParamsT<T>&, const TileSet&, int, const T*, InstanceState*,    \
                                             StateBuffersT<T>, const StageProgram&, RealizState*, cudaStream_t,  \
                                             const TmaSet*, bool, const FusedRecordT<T>&);

}  // namespace e2d
