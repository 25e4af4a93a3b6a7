/*
 * e2d_oracle.c - CPU restatement of pyHype's 2D Euler MUSCL residual and explicit
 * Runge-Kutta stepping.  TEST INFRASTRUCTURE ONLY: it is the checker the CUDA path
 * is compared with (tests, the smoke check and the CPU baseline of the benchmark),
 * never part of the product.
 *
 * It follows the reference's own sequence of array passes per block, in the
 * reference's floating-point operation order, with no contraction
 * (built with -ffp-contract=off) so that every value is the one the reference's
 * float64 code produces:
 *
 *   reconstruction-type copy of state and ghosts  pyhype/blocks/quad_block.py:120-134
 *   ghost fill + BC                                pyhype/blocks/ghost.py:149-278
 *   interface averages                             pyhype/blocks/quad_block.py:181-218
 *   Green-Gauss gradient                           pyhype/gradients/greengauss.py:110-155
 *   high-order term                                pyhype/blocks/base.py:261-289
 *   limiter (min/max, slope, psi, phi)             pyhype/limiters/base.py:47-221,
 *                                                  pyhype/limiters/limiters.py:25-62
 *   limited face / boundary states                 pyhype/fvm/SecondOrderMUSCL.py:106-126,
 *                                                  pyhype/fvm/base.py:305-325
 *   sweeps, rotations, L/R primitive states        pyhype/fvm/base.py:255-486,
 *                                                  pyhype/utils/utils.py:49-185
 *   Roe flux                                       pyhype/flux/Roe.py:175-304,
 *                                                  pyhype/flux/eigen_system.py:24-252,
 *                                                  pyhype/flux/base.py:50-146,
 *                                                  pyhype/states/primitive.py:223-320
 *   HLLL flux                                      pyhype/flux/HLLL.py:24-103
 *   flux integration + dUdt                        pyhype/fvm/base.py:108-190
 *   RK update                                      pyhype/time_marching/explicit_runge_kutta.py:47-89
 *   CFL time step                                  pyhype/blocks/quad_block.py:423-436,
 *                                                  pyhype/solvers/base.py:114-136
 *
 * Pinned against fixtures produced by running the reference itself
 * (tests/golden/make_golden.py).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/euler2d.h"

#define OR_API __attribute__((visibility("default")))

/* Work arrays kept across calls, one per slot, grown when a larger problem needs more
   and never freed: a residual of a 1024 x 1024 block needs about 512 MB of them, and
   allocating that afresh in every call made the oracle's timings measure page faults,
   not arithmetic.  The contents do not carry over (every use writes before it reads).
   Not thread-safe: the oracle is driven from one host thread. */
enum { WORK_SLOTS = 32 };
static void* work_get(int slot, size_t bytes) {
  static void* ptr[WORK_SLOTS];
  static size_t cap[WORK_SLOTS];
  if (bytes > cap[slot]) {
    free(ptr[slot]);
    ptr[slot] = malloc(bytes);
    cap[slot] = ptr[slot] ? bytes : 0;
  }
  return ptr[slot];
}

typedef struct {
  const E2DConfig* cfg;
  const E2DBlock* blk;
  const E2DGeometry* geo;
  int64_t ncell, nvface, nhface;
} Ctx;

static void ctx_init(Ctx* c, const E2DConfig* cfg, const E2DBlock* blk, const E2DGeometry* geo) {
  c->cfg = cfg;
  c->blk = blk;
  c->geo = geo;
  c->ncell = c->nvface = c->nhface = 0;
  for (int b = 0; b < cfg->nblocks; ++b) {
    const E2DBlock* B = &blk[b];
    int64_t e1 = B->cell_offset + (int64_t)B->nx * B->ny;
    int64_t e2 = B->vface_offset + (int64_t)B->ny * (B->nx + 1);
    int64_t e3 = B->hface_offset + (int64_t)(B->ny + 1) * B->nx;
    if (e1 > c->ncell) c->ncell = e1;
    if (e2 > c->nvface) c->nvface = e2;
    if (e3 > c->nhface) c->nhface = e3;
  }
}

/* ---------------------------------------------------------------- state algebra -- */

/* conservative -> primitive, pyhype/states/converter/concrete_defs.py:85-100 with
   u = rhou/rho, Ek = 0.5*(u*u+v*v), ek = rho*Ek (pyhype/states/conservative.py:85-124) */
static void cons_to_prim(const double* U, double gm1, double* W) {
  double rho = U[0];
  double u = U[1] / rho;
  double v = U[2] / rho;
  double Ek = 0.5 * (u * u + v * v);
  double ek = rho * Ek;
  W[0] = rho;
  W[1] = u;
  W[2] = v;
  W[3] = gm1 * (U[3] - ek);
}

/* primitive -> conservative, concrete_defs.py:128-141 with the primitive kinetic
   energy (0.5*rho)*(u*u+v*v) of pyhype/states/primitive.py:93-103 */
static void prim_to_cons(const double* W, double gm1, double* U) {
  double ek = 0.5 * W[0] * (W[1] * W[1] + W[2] * W[2]);
  U[0] = W[0];
  U[1] = W[0] * W[1];
  U[2] = W[0] * W[2];
  U[3] = W[3] / gm1 + ek;
}

static void to_recon(const double* U, int recon, double gm1, double* R) {
  if (recon == E2D_RECON_PRIMITIVE) {
    cons_to_prim(U, gm1, R);
  } else {
    R[0] = U[0]; R[1] = U[1]; R[2] = U[2]; R[3] = U[3];
  }
}

static void recon_to_prim(const double* R, int recon, double gm1, double* W) {
  if (recon == E2D_RECON_PRIMITIVE) {
    W[0] = R[0]; W[1] = R[1]; W[2] = R[2]; W[3] = R[3];
  } else {
    cons_to_prim(R, gm1, W);
  }
}

/* pyhype/utils/utils.py:75-85 */
static void rotate(double* q, double c, double s) {
  double u = q[1], v = q[2];
  q[1] = u * c + v * s;
  q[2] = v * c - u * s;
}
/* pyhype/utils/utils.py:151-158 */
static void unrotate(double* q, double c, double s) {
  double u = q[1], v = q[2];
  q[1] = u * c - v * s;
  q[2] = v * c + u * s;
}
/* pyhype/utils/utils.py:88-112 and 161-185 */
static void rotate90(double* q) {
  double u = q[2], v = q[1];
  q[1] = u;
  q[2] = -v;
}
static void unrotate90(double* q) {
  double u = q[2], v = q[1];
  q[1] = -u;
  q[2] = v;
}
/* pyhype/boundary_conditions/funcs.py:28-43 */
static void reflect(double* q, double c, double s) {
  rotate(q, c, s);
  q[1] = -q[1];
  unrotate(q, c, s);
}

/* numpy.maximum / numpy.minimum semantics (NaN propagates) */
static double np_max(double a, double b) {
  if (isnan(a)) return a;
  if (isnan(b)) return b;
  return a >= b ? a : b;
}
static double np_min(double a, double b) {
  if (isnan(a)) return a;
  if (isnan(b)) return b;
  return a <= b ? a : b;
}

/* numpy.linalg.norm of a float64 4-vector in the reference's environment: sqrt of
   x.dot(x), which OpenBLAS evaluates as a sequential fused multiply-add chain for
   vectors this short (verified bit for bit against numpy in the fixture container) */
static double norm4(const double* x) {
  double r = fma(x[0], x[0], 0.0);
  r = fma(x[1], x[1], r);
  r = fma(x[2], x[2], r);
  r = fma(x[3], x[3], r);
  return sqrt(r);
}

/* ---------------------------------------------------------------- flux functions - */

/* PrimitiveState F (pyhype/states/primitive.py:223-237) */
static void flux_from_prim(const double* W, double k, double* F) {
  double ek = 0.5 * W[0] * (W[1] * W[1] + W[2] * W[2]);
  double u = W[1];
  double ru = W[0] * u;
  F[0] = ru;
  F[1] = ru * u + W[3];
  F[2] = ru * W[2];
  F[3] = u * (k * W[3] + ek + W[3]);
}

/* RoePrimitiveState (pyhype/states/primitive.py:301-320) */
static void roe_average(const double* L, const double* R, double* Q) {
  double sqL = sqrt(L[0]);
  double sqR = sqrt(R[0]);
  double inv = 1.0 / (sqL + sqR);
  Q[0] = sqrt(L[0] * R[0]);
  Q[1] = (L[1] * sqL + R[1] * sqR) * inv;
  Q[2] = (L[2] * sqL + R[2] * sqR) * inv;
  Q[3] = (L[3] * sqL + R[3] * sqR) * inv;
}

/* PrimitiveState.a (primitive.py:158-171) */
static double sound(const double* W, double g) { return sqrt(g * W[3] / W[0]); }

/* FluxFunction._harten_correction_JIT (pyhype/flux/base.py:119-146) applied to one
   face: slow/fast wave speeds u-a, u+a of the right, left and Roe states.  Returns the
   corrected Roe slow (lm) and fast (lp) speeds. */
static void harten(double slowR, double fastR, double slowL, double fastL, double* lm, double* lp) {
  double tp = 2 * (slowR - slowL);
  double tm = 2 * (fastR - fastL);
  tp = (tp <= 0) ? 1e-8 : tp;
  tm = (tm <= 0) ? 1e-8 : tm;
  double rp = *lm, rm = *lp;
  if (fabs(rp) < tp) *lm = 0.5 * ((rp * rp) / tp + tp);
  if (fabs(rm) < tm) *lp = 0.5 * ((rm * rm) / tm + tm);
}

/* FluxRoe.compute_flux (pyhype/flux/Roe.py:262-304).  The upwind term is the product
   0.5 * Rc (|Lambda| (Lp dW)) of the reference's sparse eigen-system, each row summed in
   the storage order of its COO data (pyhype/flux/eigen_system.py:150-252, Roe.py:176-260). */
static void roe_flux(const double* WL, const double* WR, double g, double gm, double k, double* F) {
  double Q[4];
  roe_average(WL, WR, Q);
  double aR = sound(WR, g), aL = sound(WL, g), aQ = sound(Q, g);
  double slowR = WR[1] - aR, fastR = WR[1] + aR;
  double slowL = WL[1] - aL, fastL = WL[1] + aL;
  double Lm = Q[1] - aQ, Lp = Q[1] + aQ;
  harten(slowR, fastR, slowL, fastL, &Lm, &Lp);

  double Ek = 0.5 * (Q[1] * Q[1] + Q[2] * Q[2]);
  double H = gm * Q[3] / Q[0] + Ek;
  double ua = Q[1] * aQ;
  double ia = 1.0 / aQ;
  double one_a2 = ia * ia;
  double h = 0.5 * one_a2;
  double r2a = 0.5 * Q[0] * ia;

  double dW[4];
  for (int v = 0; v < 4; ++v) dW[v] = WR[v] - WL[v];
  /* y = Lp dW */
  double y0 = 0.0 + (-r2a) * dW[1];
  y0 = y0 + h * dW[3];
  double y1 = 0.0 + 1.0 * dW[0];
  y1 = y1 + (-one_a2) * dW[3];
  double y2 = 0.0 + 1.0 * dW[2];
  double y3 = 0.0 + r2a * dW[1];
  y3 = y3 + h * dW[3];
  /* z = |Lambda| y */
  double z0 = 0.0 + fabs(Lm) * y0;
  double z1 = 0.0 + fabs(Q[1]) * y1;
  double z2 = 0.0 + fabs(Q[1]) * y2;
  double z3 = 0.0 + fabs(Lp) * y3;
  /* Rc z */
  double r0 = 0.0 + 1.0 * z0;
  r0 = r0 + 1.0 * z1;
  r0 = r0 + 1.0 * z3;
  double r1 = 0.0 + Lm * z0;
  r1 = r1 + Q[1] * z1;
  r1 = r1 + Lp * z3;
  double r2 = 0.0 + Q[2] * z0;
  r2 = r2 + Q[2] * z1;
  r2 = r2 + 1.0 * z2;
  r2 = r2 + Q[2] * z3;
  double r3 = 0.0 + (H - ua) * z0;
  r3 = r3 + Ek * z1;
  r3 = r3 + Q[2] * z2;
  r3 = r3 + (H + ua) * z3;
  double up[4] = {0.5 * r0, 0.5 * r1, 0.5 * r2, 0.5 * r3};

  double FL[4], FR[4];
  flux_from_prim(WL, k, FL);
  flux_from_prim(WR, k, FR);
  for (int v = 0; v < 4; ++v) F[v] = 0.5 * (FL[v] + FR[v]) - up[v];
}

/* FluxHLLL.compute_flux + _HLLL_flux_JIT (pyhype/flux/HLLL.py:25-103) */
static void hlll_flux(const double* WL, const double* WR, double g, double gm1, double* F) {
  double Q[4];
  roe_average(WL, WR, Q);
  double aL = sound(WL, g), aR = sound(WR, g), aQ = sound(Q, g);
  double slowL = WL[1] - aL, fastL = WL[1] + aL;
  double slowR = WR[1] - aR, fastR = WR[1] + aR;
  double rs = Q[1] - aQ, rf = Q[1] + aQ;
  harten(slowR, fastR, slowL, fastL, &rs, &rf);
  double Lplus = np_max(fastR, rf);
  double Lminus = np_min(slowL, rs);

  double UL[4], UR[4], FL[4], FR[4];
  prim_to_cons(WL, gm1, UL);
  prim_to_cons(WR, gm1, UR);
  /* PrimitiveState.F(U=...) (primitive.py:203-209) */
  FL[0] = UL[1]; FL[1] = UL[1] * WL[1] + WL[3]; FL[2] = UL[1] * WL[2]; FL[3] = WL[1] * (UL[3] + WL[3]);
  FR[0] = UR[1]; FR[1] = UR[1] * WR[1] + WR[3]; FR[2] = UR[1] * WR[2]; FR[3] = WR[1] * (UR[3] + WR[3]);

  if (Lminus >= 0) {
    for (int v = 0; v < 4; ++v) F[v] = FL[v];
    return;
  }
  if (Lplus <= 0) {
    for (int v = 0; v < 4; ++v) F[v] = FR[v];
    return;
  }
  double u = Q[1];
  double dU[4], dF[4], r[4];
  for (int v = 0; v < 4; ++v) {
    dU[v] = UR[v] - UL[v];
    dF[v] = FR[v] - FL[v];
  }
  double kk = aQ * norm4(dU);
  for (int v = 0; v < 4; ++v) r[v] = dF[v] - u * dU[v];
  double alpha;
  if (kk < 1e-16)
    alpha = np_max(0.0, 1 - norm4(r) / (kk + 1e-14));
  else
    alpha = np_max(0.0, 1 - norm4(r) / kk);
  double sc = Lminus * Lplus * (1 - alpha * (1 - np_max(u / Lminus, u / Lplus)));
  double den = Lplus - Lminus;
  for (int v = 0; v < 4; ++v) F[v] = (Lplus * FL[v] - Lminus * FR[v] + sc * dU[v]) / den;
}

/* FluxHLLE.compute_flux (pyhype/flux/HLLE.py:22-47): the HLL flux (Harten, Lax and van
   Leer 1983) on Einfeldt's bounds (SIAM J. Numer. Anal. 25(2), 1988; Toro, Riemann
   Solvers and Numerical Methods for Fluid Dynamics, 3rd ed., 10.3 and 10.6)
   L+ = max(u_R + a_R, u~ + a~), L- = min(u_L - a_L, u~ - a~) with the Roe speeds
   Harten-corrected (HLLE.py:27-33).  The reference applies np.where(L- >= 0, F_L, .)
   and then np.where(L+ <= 0, F_R, .) (HLLE.py:41-43), so F_R wins where both hold.
   The reference's class cannot be constructed (HLLE.py:25 passes the config as the
   fluid), so there is no reference output to pin this against. */
static void hlle_flux(const double* WL, const double* WR, double g, double gm1, double* F) {
  double Q[4];
  roe_average(WL, WR, Q);
  double aL = sound(WL, g), aR = sound(WR, g), aQ = sound(Q, g);
  double slowL = WL[1] - aL, fastL = WL[1] + aL;
  double slowR = WR[1] - aR, fastR = WR[1] + aR;
  double rs = Q[1] - aQ, rf = Q[1] + aQ;
  harten(slowR, fastR, slowL, fastL, &rs, &rf);
  double Lplus = np_max(fastR, rf);
  double Lminus = np_min(slowL, rs);
  double UL[4], UR[4], FL[4], FR[4];
  prim_to_cons(WL, gm1, UL);
  prim_to_cons(WR, gm1, UR);
  FL[0] = UL[1]; FL[1] = UL[1] * WL[1] + WL[3]; FL[2] = UL[1] * WL[2]; FL[3] = WL[1] * (UL[3] + WL[3]);
  FR[0] = UR[1]; FR[1] = UR[1] * WR[1] + WR[3]; FR[2] = UR[1] * WR[2]; FR[3] = WR[1] * (UR[3] + WR[3]);
  if (Lplus <= 0) { for (int v = 0; v < 4; ++v) F[v] = FR[v]; return; }
  if (Lminus >= 0) { for (int v = 0; v < 4; ++v) F[v] = FL[v]; return; }
  double den = Lplus - Lminus;
  double LL = Lminus * Lplus;
  for (int v = 0; v < 4; ++v) F[v] = (Lplus * FL[v] - Lminus * FR[v] + LL * (UR[v] - UL[v])) / den;
}

static void face_flux(const Ctx* C, const double* WL, const double* WR, double* F) {
  double g = C->cfg->gamma, gm1 = C->cfg->gm1;
  switch (C->cfg->flux) {
    case E2D_FLUX_HLLL: hlll_flux(WL, WR, g, gm1, F); break;
    case E2D_FLUX_HLLE: hlle_flux(WL, WR, g, gm1, F); break;
    default: roe_flux(WL, WR, g, g / (g - 1.0), 1.0 / (g - 1.0), F); break;
  }
}

/* ---------------------------------------------------------------- limiter psi ----- */
/* pyhype/limiters/limiters.py:25-62.  Van Albada and Venkatakrishnan form s*s, which
   overflows for s > 1.34e154 and makes the reference return inf/inf = NaN; both already
   equal 1.0 exactly from s ~ 1e17, so the slope is capped at 1e30: every finite value of
   the reference is unchanged and its NaN becomes 1 (the one deliberate deviation). */
#define SLOPE_CAP 1e30
static double psi(int lim, double s) {
  switch (lim) {
    case E2D_LIM_BARTH_JESPERSEN: return np_min(1.0, s);
    case E2D_LIM_VAN_ALBADA: { if (s > SLOPE_CAP) s = SLOPE_CAP; double s2 = s * s; return (s2 + s) / (s2 + 1); }
    case E2D_LIM_VAN_LEER: return (fabs(s) + s) / (s + 1);
    default: { if (s > SLOPE_CAP) s = SLOPE_CAP; double s2 = s * s; return (s2 + 2 * s) / (s2 + s + 2); }
  }
}

/* ---------------------------------------------------------------- block geometry -- */
#define CELL(B, i, j) ((B)->cell_offset + (int64_t)(i) * (B)->nx + (j))
#define VF(B, i, j) ((B)->vface_offset + (int64_t)(i) * ((B)->nx + 1) + (j))
#define HF(B, i, j) ((B)->hface_offset + (int64_t)(i) * (B)->nx + (j))

static void load_cons(const Ctx* C, const double* U, int64_t cell, double* q) {
  for (int v = 0; v < 4; ++v) q[v] = U[v * C->ncell + cell];
}

/* cos/sin of the boundary angle at position k along side s (quad_mesh.py:362-369) */
static void boundary_cs(const Ctx* C, const E2DBlock* B, int side, int k, double* c, double* s) {
  int64_t f;
  switch (side) {
    case E2D_E: f = VF(B, k, B->nx); *c = C->geo->vface[E2D_F_COS][f]; *s = C->geo->vface[E2D_F_SIN][f]; return;
    case E2D_W: f = VF(B, k, 0); *c = C->geo->vface[E2D_F_COS][f]; *s = C->geo->vface[E2D_F_SIN][f]; return;
    case E2D_N: f = HF(B, B->ny, k); *c = C->geo->hface[E2D_F_COS][f]; *s = C->geo->hface[E2D_F_SIN][f]; return;
    default: f = HF(B, 0, k); *c = C->geo->hface[E2D_F_COS][f]; *s = C->geo->hface[E2D_F_SIN][f]; return;
  }
}

static int64_t own_boundary_cell(const E2DBlock* B, int side, int k) {
  switch (side) {
    case E2D_E: return CELL(B, k, B->nx - 1);
    case E2D_W: return CELL(B, k, 0);
    case E2D_N: return CELL(B, B->ny - 1, k);
    default: return CELL(B, 0, k);
  }
}

/* the per-cell kind of a side (resolves MIXED) and its Dirichlet vectors */
static int side_cell_kind(const E2DBlock* B, int side, int k, double t, const double** gd, const double** fd) {
  int kind = B->side_kind[side];
  *gd = B->dirichlet_ghost[side];
  *fd = B->dirichlet_face[side];
  if (kind == E2D_SIDE_MIXED) {
    const E2DMixedSide* m = &B->mixed[side];
    double coord = B->side_coord[side][k];
    if (coord < m->x0 + m->speed * t) {
      kind = m->kind_below; *gd = m->ghost_below; *fd = m->face_below;
    } else {
      kind = m->kind_above; *gd = m->ghost_above; *fd = m->face_above;
    }
  }
  return kind;
}

/* Ghost cell (conservative) at position k of side s: GhostBlock.send_boundary_data +
   apply_boundary_condition (pyhype/blocks/ghost.py:149-158,187-216). */
static void ghost_cons(const Ctx* C, int b, int side, int k, const double* U, double t, double* g) {
  const E2DBlock* B = &C->blk[b];
  const double *gd, *fd;
  int kind = side_cell_kind(B, side, k, t, &gd, &fd);
  if (kind == E2D_SIDE_NEIGHBOR) {
    const E2DBlock* N = &C->blk[B->neighbor[side]];
    int64_t cell;
    switch (side) {
      case E2D_E: cell = CELL(N, k, 0); break;
      case E2D_W: cell = CELL(N, k, N->nx - 1); break;
      case E2D_N: cell = CELL(N, 0, k); break;
      default: cell = CELL(N, N->ny - 1, k); break;
    }
    load_cons(C, U, cell, g);
    return;
  }
  if (kind == E2D_SIDE_DIRICHLET) {
    for (int v = 0; v < 4; ++v) g[v] = gd[v];
    return;
  }
  load_cons(C, U, own_boundary_cell(B, side, k), g);
  if (kind == E2D_SIDE_REFLECT) {
    double c, s;
    boundary_cs(C, B, side, k, &c, &s);
    reflect(g, c, s);
  }
}

/* ------------------------------------------------------------- block residual ----- */
typedef struct {
  double* W;        /* recon state, [v][n]                       */
  double* gE; double* gW; double* gN; double* gS;   /* recon ghosts [k][4] */
  double* iEW;      /* interface values [v][ny][nx+1]            */
  double* iNS;      /* [v][ny+1][nx]                             */
  double* gx; double* gy;
  double* hot;      /* high-order terms [side][v][n]            */
  double* phi;
  double* face;     /* limited face states [side][v][n]          */
  double* oE; double* oW; double* oN; double* oS; /* outside states [k][4] */
  double* vf;       /* vertical face flux [v][ny][nx+1]          */
  double* hf;       /* [v][ny+1][nx]                             */
} Scratch;

static void block_residual(const Ctx* C, int b, const double* U, double t, double* dudt, const E2DDebug* dbg) {
  const E2DBlock* B = &C->blk[b];
  const int nx = B->nx, ny = B->ny;
  const int64_t n = (int64_t)nx * ny;
  const int recon = C->cfg->recon;
  const double gm1 = C->cfg->gm1;
  const E2DGeometry* G = C->geo;
  const int64_t nv = (int64_t)ny * (nx + 1), nh = (int64_t)(ny + 1) * nx;
  /* face quadrature (pyhype/mesh/quadratures.py:33-37): points in the reference's order,
     weights as Python forms them; the one-point rule's offsets are the HX/HY planes */
  const int nqp = C->cfg->nqp > 1 ? C->cfg->nqp : 1;
  const double wq[3][3] = {{2.0, 0.0, 0.0}, {1.0, 1.0, 0.0}, {5.0 / 9.0, 8.0 / 9.0, 5.0 / 9.0}};
  const double* qw = wq[nqp - 1];
#define HOT(side, q, v) ((((side) * nqp + (q)) * 4 + (v)) * n)

  Scratch S;
  S.W = work_get(0, sizeof(double) * 4 * n);
  S.gE = work_get(1, sizeof(double) * 4 * ny); S.gW = work_get(2, sizeof(double) * 4 * ny);
  S.gN = work_get(3, sizeof(double) * 4 * nx); S.gS = work_get(4, sizeof(double) * 4 * nx);
  S.oE = work_get(5, sizeof(double) * 4 * nqp * ny); S.oW = work_get(6, sizeof(double) * 4 * nqp * ny);
  S.oN = work_get(7, sizeof(double) * 4 * nqp * nx); S.oS = work_get(8, sizeof(double) * 4 * nqp * nx);
  S.iEW = work_get(9, sizeof(double) * 4 * nv);
  S.iNS = work_get(10, sizeof(double) * 4 * nh);
  S.gx = work_get(11, sizeof(double) * 4 * n); S.gy = work_get(12, sizeof(double) * 4 * n);
  S.hot = work_get(13, sizeof(double) * 16 * nqp * n);
  S.phi = work_get(14, sizeof(double) * 4 * n);
  S.face = work_get(15, sizeof(double) * 16 * nqp * n);
  S.vf = work_get(16, sizeof(double) * 4 * nqp * nv);
  S.hf = work_get(17, sizeof(double) * 4 * nqp * nh);

  /* 1. reconstruction-type state (QuadBlock -> ReconstructionBlock.from_block) */
#pragma omp parallel for schedule(static)
  for (int i = 0; i < ny; ++i)
    for (int j = 0; j < nx; ++j) {
      double q[4], r[4];
      load_cons(C, U, CELL(B, i, j), q);
      to_recon(q, recon, gm1, r);
      for (int v = 0; v < 4; ++v) S.W[v * n + (int64_t)i * nx + j] = r[v];
    }
  /* 2. ghosts: conservative ghost + BC, then converted to the reconstruction type */
  for (int side = 0; side < 4; ++side) {
    int len = (side == E2D_E || side == E2D_W) ? ny : nx;
    double* dst = side == E2D_E ? S.gE : side == E2D_W ? S.gW : side == E2D_N ? S.gN : S.gS;
    for (int k = 0; k < len; ++k) {
      double g[4];
      ghost_cons(C, b, side, k, U, t, g);
      to_recon(g, recon, gm1, dst + 4 * k);
    }
  }
#define Wv(v, i, j) S.W[(v) * n + (int64_t)(i) * nx + (j)]
  /* 3. interface averages */
#pragma omp parallel for schedule(static)
  for (int i = 0; i < ny; ++i)
    for (int v = 0; v < 4; ++v) {
      S.iEW[v * nv + (int64_t)i * (nx + 1) + 0] = 0.5 * (S.gW[4 * i + v] + Wv(v, i, 0));
      S.iEW[v * nv + (int64_t)i * (nx + 1) + nx] = 0.5 * (S.gE[4 * i + v] + Wv(v, i, nx - 1));
      for (int j = 1; j < nx; ++j)
        S.iEW[v * nv + (int64_t)i * (nx + 1) + j] = 0.5 * (Wv(v, i, j - 1) + Wv(v, i, j));
    }
#pragma omp parallel for schedule(static)
  for (int i = 0; i <= ny; ++i)
    for (int v = 0; v < 4; ++v)
      for (int j = 0; j < nx; ++j) {
        double val;
        if (i == 0) val = 0.5 * (S.gS[4 * j + v] + Wv(v, 0, j));
        else if (i == ny) val = 0.5 * (S.gN[4 * j + v] + Wv(v, ny - 1, j));
        else val = 0.5 * (Wv(v, i - 1, j) + Wv(v, i, j));
        S.iNS[v * nh + (int64_t)i * nx + j] = val;
      }
  /* 4. Green-Gauss gradient and high-order terms */
#pragma omp parallel for schedule(static)
  for (int i = 0; i < ny; ++i)
    for (int j = 0; j < nx; ++j) {
      int64_t c = CELL(B, i, j), loc = (int64_t)i * nx + j;
      double xlE = G->vface[E2D_F_LC][VF(B, i, j + 1)], ylE = G->vface[E2D_F_LS][VF(B, i, j + 1)];
      double xlW = -G->vface[E2D_F_LC][VF(B, i, j)], ylW = -G->vface[E2D_F_LS][VF(B, i, j)];
      double xlN = G->hface[E2D_F_LC][HF(B, i + 1, j)], ylN = G->hface[E2D_F_LS][HF(B, i + 1, j)];
      double xlS = -G->hface[E2D_F_LC][HF(B, i, j)], ylS = -G->hface[E2D_F_LS][HF(B, i, j)];
      double a = G->cell[E2D_G_INV_A][c];
      for (int v = 0; v < 4; ++v) {
        double e = S.iEW[v * nv + (int64_t)i * (nx + 1) + j + 1];
        double w = S.iEW[v * nv + (int64_t)i * (nx + 1) + j];
        double nn = S.iNS[v * nh + (int64_t)(i + 1) * nx + j];
        double s = S.iNS[v * nh + (int64_t)i * nx + j];
        double gx = (e * xlE + w * xlW + nn * xlN + s * xlS) * a;
        double gy = (e * ylE + w * ylW + nn * ylN + s * ylS) * a;
        S.gx[v * n + loc] = gx;
        S.gy[v * n + loc] = gy;
        for (int side = 0; side < 4; ++side)
          for (int q = 0; q < nqp; ++q) {
            double dx = nqp == 1 ? G->cell[E2D_G_HX_E + side][c] : G->qp[q][side][c];
            double dy = nqp == 1 ? G->cell[E2D_G_HY_E + side][c] : G->qp[q][4 + side][c];
            S.hot[HOT(side, q, v) + loc] = gx * dx + gy * dy;
          }
      }
    }
  /* 5. limiter */
  const int lim = C->cfg->limiter;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < ny; ++i)
    for (int j = 0; j < nx; ++j) {
      int64_t loc = (int64_t)i * nx + j;
      for (int v = 0; v < 4; ++v) {
        double u0 = Wv(v, i, j);
        double we = j > 0 ? Wv(v, i, j - 1) : S.gW[4 * i + v];
        double ea = j < nx - 1 ? Wv(v, i, j + 1) : S.gE[4 * i + v];
        double so = i > 0 ? Wv(v, i - 1, j) : S.gS[4 * j + v];
        double no = i < ny - 1 ? Wv(v, i + 1, j) : S.gN[4 * j + v];
        double mx = np_max(np_max(np_max(np_max(u0, we), ea), so), no);
        double mn = np_min(np_min(np_min(np_min(u0, we), ea), so), no);
        double dmax = mx - u0, dmin = mn - u0;
        /* minimum over the E, W, N, S quadrature points in that order */
        double ph = 0.0;
        for (int side = 0; side < 4; ++side)
          for (int q = 0; q < nqp; ++q) {
            double davg = (u0 + S.hot[HOT(side, q, v) + loc]) - u0;
            double s = 1.0;
            if (davg > 0) s = dmax / davg;
            else if (davg < 0) s = dmin / davg;
            double p = psi(lim, s);
            ph = (side == 0 && q == 0) ? p : np_min(ph, p);
          }
        S.phi[v * n + loc] = (ph < 0) ? 0.0 : ph;
      }
    }
  /* 6. limited face states */
#pragma omp parallel for schedule(static)
  for (int i = 0; i < ny; ++i)
    for (int j = 0; j < nx; ++j) {
      int64_t loc = (int64_t)i * nx + j;
      for (int side = 0; side < 4; ++side)
        for (int q = 0; q < nqp; ++q)
          for (int v = 0; v < 4; ++v)
            S.face[HOT(side, q, v) + loc] = Wv(v, i, j) + S.phi[v * n + loc] * S.hot[HOT(side, q, v) + loc];
    }
  /* 7. outside states of the block boundary faces (fvm/base.py:305-325 + BC) */
  for (int side = 0; side < 4; ++side) {
    int len = (side == E2D_E || side == E2D_W) ? ny : nx;
    double* dst = side == E2D_E ? S.oE : side == E2D_W ? S.oW : side == E2D_N ? S.oN : S.oS;
    const double* gh = side == E2D_E ? S.gE : side == E2D_W ? S.gW : side == E2D_N ? S.gN : S.gS;
    for (int q = 0; q < nqp; ++q)
      for (int k = 0; k < len; ++k) {
        const double *gd, *fd;
        int kind = side_cell_kind(B, side, k, t, &gd, &fd);
        double* o = dst + 4 * ((int64_t)q * len + k);
        if (kind == E2D_SIDE_NEIGHBOR || kind == E2D_SIDE_COPY) {
          for (int v = 0; v < 4; ++v) o[v] = gh[4 * k + v];
        } else if (kind == E2D_SIDE_DIRICHLET) {
          for (int v = 0; v < 4; ++v) o[v] = fd[v];
        } else {
          int64_t loc = own_boundary_cell(B, side, k) - B->cell_offset;
          for (int v = 0; v < 4; ++v) o[v] = S.face[HOT(side, q, v) + loc];
          if (kind == E2D_SIDE_REFLECT) {
            double c, s;
            boundary_cs(C, B, side, k, &c, &s);
            reflect(o, c, s);
          }
        }
      }
  }
  /* 8. east-west sweep */
#pragma omp parallel for schedule(static)
  for (int i = 0; i < ny; ++i)
    for (int j = 0; j <= nx; ++j)
     for (int q = 0; q < nqp; ++q) {
      double L[4], R[4], WL[4], WR[4], F[4];
      for (int v = 0; v < 4; ++v) {
        L[v] = j == 0 ? S.oW[4 * ((int64_t)q * ny + i) + v] : S.face[HOT(E2D_E, q, v) + (int64_t)i * nx + j - 1];
        R[v] = j == nx ? S.oE[4 * ((int64_t)q * ny + i) + v] : S.face[HOT(E2D_W, q, v) + (int64_t)i * nx + j];
      }
      int64_t f = VF(B, i, j);
      double c = G->vface[E2D_F_COS][f], s = G->vface[E2D_F_SIN][f];
      if (!B->is_cartesian) { rotate(L, c, s); rotate(R, c, s); }
      recon_to_prim(L, recon, gm1, WL);
      recon_to_prim(R, recon, gm1, WR);
      face_flux(C, WL, WR, F);
      if (dbg && q == 0) {  /* intermediates of the first quadrature point */
        for (int v = 0; v < 4; ++v) {
          if (dbg->vL) dbg->vL[v * C->nvface + f] = WL[v];
          if (dbg->vR) dbg->vR[v * C->nvface + f] = WR[v];
          if (dbg->vflux_raw) dbg->vflux_raw[v * C->nvface + f] = F[v];
        }
      }
      if (!B->is_cartesian) unrotate(F, c, s);
      for (int v = 0; v < 4; ++v) {
        S.vf[((int64_t)q * 4 + v) * nv + (int64_t)i * (nx + 1) + j] = F[v];
        if (dbg && dbg->vflux && q == 0) dbg->vflux[v * C->nvface + f] = F[v];
      }
     }
  /* 9. north-south sweep */
#pragma omp parallel for schedule(static)
  for (int j = 0; j < nx; ++j)
    for (int i = 0; i <= ny; ++i)
     for (int q = 0; q < nqp; ++q) {
      double L[4], R[4], WL[4], WR[4], F[4];
      for (int v = 0; v < 4; ++v) {
        L[v] = i == 0 ? S.oS[4 * ((int64_t)q * nx + j) + v] : S.face[HOT(E2D_N, q, v) + (int64_t)(i - 1) * nx + j];
        R[v] = i == ny ? S.oN[4 * ((int64_t)q * nx + j) + v] : S.face[HOT(E2D_S, q, v) + (int64_t)i * nx + j];
      }
      int64_t f = HF(B, i, j);
      double c = G->hface[E2D_F_COS][f], s = G->hface[E2D_F_SIN][f];
      if (B->is_cartesian) { rotate90(L); rotate90(R); }
      else { rotate(L, c, s); rotate(R, c, s); }
      recon_to_prim(L, recon, gm1, WL);
      recon_to_prim(R, recon, gm1, WR);
      face_flux(C, WL, WR, F);
      if (dbg && q == 0) {
        for (int v = 0; v < 4; ++v) {
          if (dbg->hL) dbg->hL[v * C->nhface + f] = WL[v];
          if (dbg->hR) dbg->hR[v * C->nhface + f] = WR[v];
          if (dbg->hflux_raw) dbg->hflux_raw[v * C->nhface + f] = F[v];
        }
      }
      if (B->is_cartesian) unrotate90(F);
      else unrotate(F, c, s);
      for (int v = 0; v < 4; ++v) {
        S.hf[((int64_t)q * 4 + v) * nh + (int64_t)i * nx + j] = F[v];
        if (dbg && dbg->hflux && q == 0) dbg->hflux[v * C->nhface + f] = F[v];
      }
     }
  /* 10. Gauss integration over faces, L * (sum_q w_q F_q) summed from 0 in point order
     (fvm/base.py:171-190), and dUdt */
#pragma omp parallel for schedule(static)
  for (int i = 0; i < ny; ++i)
    for (int j = 0; j < nx; ++j) {
      int64_t c = CELL(B, i, j);
      double LW = G->vface[E2D_F_L][VF(B, i, j)], LE = G->vface[E2D_F_L][VF(B, i, j + 1)];
      double LS = G->hface[E2D_F_L][HF(B, i, j)], LN = G->hface[E2D_F_L][HF(B, i + 1, j)];
      double A = G->cell[E2D_G_A][c];
      for (int v = 0; v < 4; ++v) {
        double sW = 0.0, sE = 0.0, sS = 0.0, sN = 0.0;
        for (int q = 0; q < nqp; ++q) {
          sW = sW + qw[q] * S.vf[((int64_t)q * 4 + v) * nv + (int64_t)i * (nx + 1) + j];
          sE = sE + qw[q] * S.vf[((int64_t)q * 4 + v) * nv + (int64_t)i * (nx + 1) + j + 1];
          sS = sS + qw[q] * S.hf[((int64_t)q * 4 + v) * nh + (int64_t)i * nx + j];
          sN = sN + qw[q] * S.hf[((int64_t)q * 4 + v) * nh + (int64_t)(i + 1) * nx + j];
        }
        double IW = LW * sW, IE = LE * sE, IS = LS * sS, IN = LN * sN;
        dudt[v * C->ncell + c] = 0.5 * (IW - IE + IS - IN) / A;
      }
    }
#undef HOT
  if (dbg) {
    for (int v = 0; v < 4; ++v)
      for (int64_t l = 0; l < n; ++l) {
        if (dbg->gx) dbg->gx[v * C->ncell + B->cell_offset + l] = S.gx[v * n + l];
        if (dbg->gy) dbg->gy[v * C->ncell + B->cell_offset + l] = S.gy[v * n + l];
        if (dbg->phi) dbg->phi[v * C->ncell + B->cell_offset + l] = S.phi[v * n + l];
      }
  }
#undef Wv
}

/* ------------------------------------------------------------------ public API ---- */
OR_API void oracle_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

OR_API int oracle_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* The face flux function alone, for property tests: n face-frame primitive pairs
   (WL[4 k .. 4 k + 3], WR[...]) -> F[4 k ..], flux code as in E2DConfig.flux. */
OR_API int oracle_flux(int flux, int64_t n, const double* WL, const double* WR, double gamma, double gm1,
                       double* F) {
  E2DConfig cfg;
  memset(&cfg, 0, sizeof cfg);
  cfg.flux = flux;
  cfg.gamma = gamma;
  cfg.gm1 = gm1;
  Ctx C;
  memset(&C, 0, sizeof C);
  C.cfg = &cfg;
  for (int64_t k = 0; k < n; ++k) face_flux(&C, WL + 4 * k, WR + 4 * k, F + 4 * k);
  return 0;
}

OR_API int oracle_residual(const E2DConfig* cfg, const E2DBlock* blk, const E2DGeometry* geo,
                           const double* U, double t, double* dudt, const E2DDebug* dbg) {
  Ctx C;
  ctx_init(&C, cfg, blk, geo);
  for (int b = 0; b < cfg->nblocks; ++b) block_residual(&C, b, U, t, dudt, dbg);
  return 0;
}

/* Ghost layer of every block in the reconstruction variables, the values
   ReconstructionBlock.from_block holds after Blocks.apply_boundary_condition
   (pyhype/blocks/base.py:448-471, pyhype/blocks/ghost.py:149-216,
   pyhype/blocks/quad_block.py:120-134).  out: 4 planes of nghost = sum of 2 (nx + ny)
   values; per block E (ny), W (ny), N (nx), S (nx), blocks in table order. */
OR_API int oracle_ghost_layer(const E2DConfig* cfg, const E2DBlock* blk, const E2DGeometry* geo,
                              const double* U, double t, double* out) {
  Ctx C;
  ctx_init(&C, cfg, blk, geo);
  int64_t nghost = 0;
  for (int b = 0; b < cfg->nblocks; ++b) nghost += 2 * (int64_t)(blk[b].nx + blk[b].ny);
  int64_t o = 0;
  for (int b = 0; b < cfg->nblocks; ++b) {
    const int sides[4] = {E2D_E, E2D_W, E2D_N, E2D_S};
    for (int si = 0; si < 4; ++si) {
      const int side = sides[si];
      const int len = (side == E2D_E || side == E2D_W) ? blk[b].ny : blk[b].nx;
      for (int k = 0; k < len; ++k, ++o) {
        double g[4], r[4];
        ghost_cons(&C, b, side, k, U, t, g);
        to_recon(g, cfg->recon, cfg->gm1, r);
        for (int v = 0; v < 4; ++v) out[v * nghost + o] = r[v];
      }
    }
  }
  return 0;
}

/* ExplicitRungeKutta.integrate (explicit_runge_kutta.py:47-80): stage s evaluates
   k_s at the current stage state, then forms U^n + (dt*a[s][0])*k_0 + ... term by
   term in order, skipping zero coefficients. */
OR_API int oracle_step(const E2DConfig* cfg, const E2DBlock* blk, const E2DGeometry* geo,
                       double* U, int nstages, const double* a, double dt, double t) {
  Ctx C;
  ctx_init(&C, cfg, blk, geo);
  const int64_t N = 4 * C.ncell;
  double* U0 = work_get(20, sizeof(double) * N);
  double* cur = work_get(21, sizeof(double) * N);
  double* k = work_get(22, sizeof(double) * N * nstages);
  memcpy(U0, U, sizeof(double) * N);
  memcpy(cur, U, sizeof(double) * N);
  for (int s = 0; s < nstages; ++s) {
    for (int b = 0; b < cfg->nblocks; ++b) block_residual(&C, b, cur, t, k + (int64_t)s * N, NULL);
    memcpy(cur, U0, sizeof(double) * N);
    for (int j = 0; j <= s; ++j) {
      double aj = a[s * nstages + j];
      if (aj != 0) {
        double dta = dt * aj;
        const double* kj = k + (int64_t)j * N;
#pragma omp parallel for schedule(static)
        for (int64_t e = 0; e < N; ++e) cur[e] = cur[e] + dta * kj[e];
      }
    }
  }
  memcpy(U, cur, sizeof(double) * N);
  return 0;
}

/* QuadBlock.get_dt (quad_block.py:423-436) reduced over blocks (solvers/base.py:
   114-136), per instance; no t_final clamp. */
OR_API int oracle_dt(const E2DConfig* cfg, const E2DBlock* blk, const E2DGeometry* geo,
                     const double* U, double* dt_out) {
  Ctx C;
  ctx_init(&C, cfg, blk, geo);
  int ninst = cfg->ninstances > 0 ? cfg->ninstances : 1;
  for (int q = 0; q < ninst; ++q) dt_out[q] = INFINITY;
  for (int b = 0; b < cfg->nblocks; ++b) {
    const E2DBlock* B = &blk[b];
    double m = INFINITY;
#pragma omp parallel for reduction(min : m) schedule(static)
    for (int i = 0; i < B->ny; ++i)
      for (int j = 0; j < B->nx; ++j) {
        int64_t c = CELL(B, i, j);
        double q[4], W[4];
        load_cons(&C, U, c, q);
        cons_to_prim(q, cfg->gm1, W);
        double a = sqrt(cfg->gamma * W[3] / W[0]);
        double tx = geo->cell[E2D_G_CFL_DX][c] / (fabs(W[1]) + a);
        double ty = geo->cell[E2D_G_CFL_DY][c] / (fabs(W[2]) + a);
        double mm = np_min(tx, ty);
        if (mm < m || isnan(mm)) m = mm;
      }
    double dtb = cfg->cfl * m;
    int q = B->instance;
    if (dtb < dt_out[q]) dt_out[q] = dtb;
  }
  return 0;
}

OR_API int oracle_realizable(const E2DConfig* cfg, const E2DBlock* blk, const E2DGeometry* geo,
                             const double* U, E2DRealizability* out) {
  Ctx C;
  ctx_init(&C, cfg, blk, geo);
  out->ok = 1; out->block = -1; out->cell = -1; out->nbad = 0;
  for (int b = 0; b < cfg->nblocks; ++b) {
    const E2DBlock* B = &blk[b];
    for (int64_t l = 0; l < (int64_t)B->nx * B->ny; ++l) {
      double rho = U[B->cell_offset + l], E = U[3 * C.ncell + B->cell_offset + l];
      if (!(rho > 0) || !(E > 0)) {
        if (out->ok) { out->ok = 0; out->block = b; out->cell = l; }
        out->nbad++;
      }
    }
  }
  return out->ok ? 0 : E2D_ERR_UNREALIZABLE;
}
