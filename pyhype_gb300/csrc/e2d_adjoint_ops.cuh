// e2d_adjoint_ops.cuh - hand-written reverse-mode (vector-Jacobian) products of the
// pointwise pieces of the scheme: the Roe, HLLL and HLLE fluxes, the conservative->primitive
// conversion, the rotations and the reflection, and the limiter functions.
//
// Each *_vjp recomputes the forward intermediates it needs from the forward inputs
// and accumulates lambda^T * d(output)/d(input) into the input adjoints.  Branches
// (Harten's entropy fix, |x|) take the derivative of the branch the forward took;
// at a tie the forward's own selection decides.
#pragma once
#include "e2d_device.cuh"

namespace e2d {

// Divisions of the reverse state algebra by positive divisors (densities and their
// square roots, sound speeds, Q0, the limiter functions' denominators, the Harten
// width, gamma - 1): FP64 as the forward's qdiv/pdiv; the FP32 form without div32's
// range test (rdiv: the same quotient for operands within 2^-60..2^61).  The HLL
// family's divisions by wave speeds, which may approach zero, keep qdiv/pdiv.
template <typename T>
__device__ __forceinline__ T aqdiv(T a, T b) {
  if constexpr (sizeof(T) == 4) return rdiv(a, b);
  else return qdiv(a, b);
}
template <typename T>
__device__ __forceinline__ T apdiv(T a, T b) {
  if constexpr (sizeof(T) == 4) return rdiv(a, b);
  else return pdiv(a, b);
}

template <typename T>
__device__ __forceinline__ T sgn(T x) { return x > T(0) ? T(1) : (x < T(0) ? T(-1) : T(0)); }

// W = cons_to_prim(U): lamU += (dW/dU)^T lamW
template <typename T>
__device__ __forceinline__ void cons_to_prim_vjp(const T* U, const Gas<T>& G, const T* lW, T* lU) {
  const T rho = U[0];
  const T u = aqdiv(U[1], rho), v = aqdiv(U[2], rho);
  // p = gm1 * (E - rho * 0.5 * (u*u + v*v))
  const T lp = lW[3];
  T lu = lW[1] - lp * G.gm1 * rho * u;
  T lv = lW[2] - lp * G.gm1 * rho * v;
  T lrho = lW[0] - half(lp * G.gm1) * (u * u + v * v);
  // u = rhou / rho, v = rhov / rho
  lU[1] += aqdiv(lu, rho);
  lU[2] += aqdiv(lv, rho);
  lU[0] += lrho - aqdiv(lu * u + lv * v, rho);
  lU[3] += lp * G.gm1;
}

// q <- rotate(q, c, s) is orthogonal: its transpose is unrotate (and vice versa).
template <typename T>
__device__ __forceinline__ void rotate_vjp(T* lq, T c, T s) { unrotate(lq, c, s); }
template <typename T>
__device__ __forceinline__ void rotate90_vjp(T* lq) { unrotate90(lq); }
// reflect = unrotate * diag(1,-1 on the normal) * rotate is symmetric
template <typename T>
__device__ __forceinline__ void reflect_vjp(T* lq, T c, T s) { reflect(lq, c, s); }

// d psi / d s of the limiter functions (s >= 0 here: the slope is dmax/davg with
// davg > 0 or dmin/davg with davg < 0).  The rational derivatives are written as
// ((numerator)/d)/d so that large s does not overflow; beyond s = 1e100 (and in the
// capped region of the slope) they are zero to working precision.
template <int LIM, typename T>
__device__ __forceinline__ T psi_deriv(T s) {
  if (LIM == E2D_LIM_BARTH_JESPERSEN) return (s < T(1)) ? T(1) : T(0);  // min(1, s)
  if (LIM == E2D_LIM_VAN_LEER) {  // (|s| + s)/(s + 1), with d|s|/ds = 0 at s = 0
    const T d = s + T(1);
    return apdiv((sgn(s) + T(1)) - aqdiv(fabs(s) + s, d), d);
  }
  if (vlt(sizeof(T) == 4 ? T(SLOPE_CAP_FP32) : T(SLOPE_CAP_FP64), s)) return T(0);  // capped: constant
  if (LIM == E2D_LIM_VAN_ALBADA) {  // (s^2 + s)/(s^2 + 1)
    const T d = s * s + T(1);
    return apdiv(apdiv(T(1) + twice(s) - s * s, d), d);
  }
  const T d = s * s + s + T(2);  // Venkatakrishnan (s^2 + 2s)/(s^2 + s + 2)
  return apdiv(apdiv(T(4) + T(4) * s - s * s, d), d);
}

// F = roe_flux(WL, WR): lamWL += (dF/dWL)^T lamF, lamWR += (dF/dWR)^T lamF
template <typename T>
__device__ void roe_flux_vjp(const T* L, const T* R, const Gas<T>& G, const T* lF, T* lL, T* lR) {
  // ---- forward (same expressions as roe_flux) ----
  const T sqL = sqrt(L[0]), sqR = sqrt(R[0]);
  const T inv = apdiv(T(1), sqL + sqR);
  const T Q0 = sqrt(L[0] * R[0]);
  const T n1 = L[1] * sqL + R[1] * sqR, n2 = L[2] * sqL + R[2] * sqR, n3 = L[3] * sqL + R[3] * sqR;
  const T Q1 = n1 * inv, Q2 = n2 * inv, Q3 = n3 * inv;
  const T aR = sqrt(apdiv(G.g * R[3], R[0])), aL = sqrt(apdiv(G.g * L[3], L[0])), aQ = sqrt(apdiv(G.g * Q3, Q0));
  const T Lm0 = Q1 - aQ, Lp0 = Q1 + aQ;
  const T slowR = R[1] - aR, fastR = R[1] + aR, slowL = L[1] - aL, fastL = L[1] + aL;
  const T tp0 = twice(slowR - slowL), tm0 = twice(fastR - fastL);
  const bool tp_pos = is_pos(tp0), tm_pos = is_pos(tm0);
  const T tp = tp_pos ? tp0 : T(1e-8), tm = tm_pos ? tm0 : T(1e-8);
  const bool cm = vlt(T(fabs(Lm0)), tp), cp = vlt(T(fabs(Lp0)), tm);
  const T Lm = cm ? half(aqdiv(Lm0 * Lm0, tp) + tp) : Lm0;
  const T Lp = cp ? half(aqdiv(Lp0 * Lp0, tm) + tm) : Lp0;
  const T Ek = half(Q1 * Q1 + Q2 * Q2);
  const T H = apdiv(G.gm * Q3, Q0) + Ek;
  const T ua = Q1 * aQ;
  const T ia = apdiv(T(1), aQ);
  const T one_a2 = ia * ia;
  const T h = half(one_a2);
  const T r2a = half(Q0) * ia;
  const T d0 = R[0] - L[0], d1 = R[1] - L[1], d2 = R[2] - L[2], d3 = R[3] - L[3];
  const T y0 = (-r2a) * d1 + h * d3, y1 = d0 + (-one_a2) * d3, y2 = d2, y3 = r2a * d1 + h * d3;
  const T sLm = sgn(Lm), sQ1 = sgn(Q1), sLp = sgn(Lp);  // d|x|/dx, 0 at x = 0
  const T z0 = fabs(Lm) * y0, z1 = fabs(Q1) * y1, z2 = fabs(Q1) * y2, z3 = fabs(Lp) * y3;
  // ---- reverse ----
  const T lr0 = T(-0.5) * lF[0], lr1 = T(-0.5) * lF[1], lr2 = T(-0.5) * lF[2], lr3 = T(-0.5) * lF[3];
  T lz0 = lr0 + lr1 * Lm + lr2 * Q2 + lr3 * (H - ua);
  T lz1 = lr0 + lr1 * Q1 + lr2 * Q2 + lr3 * Ek;
  T lz2 = lr2 + lr3 * Q2;
  T lz3 = lr0 + lr1 * Lp + lr2 * Q2 + lr3 * (H + ua);
  T lLm = lr1 * z0, lLp = lr1 * z3;
  T lQ1 = lr1 * z1;
  T lQ2 = lr2 * (z0 + z1 + z3) + lr3 * z2;
  T lH = lr3 * (z0 + z3);
  T lua = lr3 * (z3 - z0);
  T lEk = lr3 * z1;
  // z = |lambda| * y
  lLm += lz0 * y0 * sLm;
  lLp += lz3 * y3 * sLp;
  lQ1 += (lz1 * y1 + lz2 * y2) * sQ1;
  const T ly0 = lz0 * fabs(Lm), ly1 = lz1 * fabs(Q1), ly2 = lz2 * fabs(Q1), ly3 = lz3 * fabs(Lp);
  // y = Lp * dW
  const T lr2a = (ly3 - ly0) * d1;
  const T lh = (ly0 + ly3) * d3;
  const T lone_a2 = -ly1 * d3 + half(lh);
  T ld0 = ly1, ld1 = (ly3 - ly0) * r2a, ld2 = ly2, ld3 = (ly0 + ly3) * h - ly1 * one_a2;
  // r2a = 0.5*Q0*ia, one_a2 = ia*ia, ia = 1/aQ
  T lQ0 = half(ia) * lr2a;
  const T lia = half(Q0) * lr2a + twice(ia) * lone_a2;
  T laQ = -ia * ia * lia;
  // ua = Q1*aQ ; H = gm*Q3/Q0 + Ek ; Ek = 0.5*(Q1^2 + Q2^2)
  lQ1 += aQ * lua;
  laQ += Q1 * lua;
  T lQ3 = apdiv(G.gm, Q0) * lH;
  lQ0 += apdiv(-G.gm * Q3, Q0 * Q0) * lH;
  lEk += lH;
  lQ1 += Q1 * lEk;
  lQ2 += Q2 * lEk;
  // Harten
  T lLm0 = lLm, lLp0 = lLp, ltp = T(0), ltm = T(0);
  if (cm) {
    lLm0 = lLm * aqdiv(Lm0, tp);
    ltp = half(lLm) * (T(1) - aqdiv(Lm0 * Lm0, tp * tp));
  }
  if (cp) {
    lLp0 = lLp * aqdiv(Lp0, tm);
    ltm = half(lLp) * (T(1) - aqdiv(Lp0 * Lp0, tm * tm));
  }
  if (!tp_pos) ltp = T(0);
  if (!tm_pos) ltm = T(0);
  lQ1 += lLm0 + lLp0;
  laQ += lLp0 - lLm0;
  // tp = 2*(slowR - slowL), tm = 2*(fastR - fastL)
  const T lslowR = twice(ltp), lslowL = -twice(ltp), lfastR = twice(ltm), lfastL = -twice(ltm);
  T lR1 = lslowR + lfastR, lL1 = lslowL + lfastL;
  const T laR = lfastR - lslowR, laL = lfastL - lslowL;
  // sound speeds a = sqrt(g p / rho)
  T lR0 = aqdiv(-laR * G.g * R[3], twice(aR) * R[0] * R[0]);
  T lR3 = aqdiv(laR * G.g, twice(aR) * R[0]);
  T lL0 = aqdiv(-laL * G.g * L[3], twice(aL) * L[0] * L[0]);
  T lL3 = aqdiv(laL * G.g, twice(aL) * L[0]);
  lQ3 += aqdiv(laQ * G.g, twice(aQ) * Q0);
  lQ0 += aqdiv(-laQ * G.g * Q3, twice(aQ) * Q0 * Q0);
  // Roe averages
  const T linv = lQ1 * n1 + lQ2 * n2 + lQ3 * n3;
  lL1 += lQ1 * inv * sqL;
  lR1 += lQ1 * inv * sqR;
  T lL2 = lQ2 * inv * sqL, lR2 = lQ2 * inv * sqR;
  lL3 += lQ3 * inv * sqL;
  lR3 += lQ3 * inv * sqR;
  T lsqL = (lQ1 * L[1] + lQ2 * L[2] + lQ3 * L[3]) * inv - inv * inv * linv;
  T lsqR = (lQ1 * R[1] + lQ2 * R[2] + lQ3 * R[3]) * inv - inv * inv * linv;
  lL0 += aqdiv(lQ0 * R[0], twice(Q0)) + aqdiv(lsqL, twice(sqL));
  lR0 += aqdiv(lQ0 * L[0], twice(Q0)) + aqdiv(lsqR, twice(sqR));
  // dW = R - L
  lR0 += ld0; lR1 += ld1; lR2 += ld2; lR3 += ld3;
  lL0 -= ld0; lL1 -= ld1; lL2 -= ld2; lL3 -= ld3;
  // physical fluxes, each weighted 0.5
  const T* W[2] = {L, R};
  T* lW[2] = {nullptr, nullptr};
  T acc[2][4] = {{lL0, lL1, lL2, lL3}, {lR0, lR1, lR2, lR3}};
#pragma unroll
  for (int side = 0; side < 2; ++side) {
    const T* w = W[side];
    const T u = w[1], ru = w[0] * w[1];
    const T ek = half(w[0]) * (w[1] * w[1] + w[2] * w[2]);
    const T f0 = half(lF[0]), f1 = half(lF[1]), f2 = half(lF[2]), f3 = half(lF[3]);
    const T lru = f0 + f1 * u + f2 * w[2];
    const T lek = f3 * u;
    acc[side][0] += lru * w[1] + half(lek) * (w[1] * w[1] + w[2] * w[2]);
    acc[side][1] += lru * w[0] + f1 * ru + f3 * (G.k * w[3] + ek + w[3]) + lek * w[0] * w[1];
    acc[side][2] += f2 * ru + lek * w[0] * w[2];
    acc[side][3] += f1 + f3 * u * (G.k + T(1));
  }
  (void)lW;
#pragma unroll
  for (int v = 0; v < 4; ++v) {
    lL[v] += acc[0][v];
    lR[v] += acc[1][v];
  }
}

// ---- HLL-type fluxes (HLLL, HLLE) --------------------------------------------------
// The forward pieces both share: Roe average (u and a only), sound speeds, the
// Harten-corrected Roe speeds and the bounds L+ = max(u_R + a_R, rf), L- = min(u_L -
// a_L, rs), with the selections the forward makes (vmax keeps its first operand on
// ties, vmin its first).
template <typename T>
struct HllBounds {
  T sqL, sqR, inv, Q0, n1, n3, Q1, Q3, aL, aR, aQ;
  T rs0, rf0, tp, tm;
  bool tp_pos, tm_pos, cs, cf, plus_fastR, minus_slowL;
  T Lp, Lm;
};

template <typename T>
__device__ __forceinline__ void hll_bounds(const T* L, const T* R, const Gas<T>& G, HllBounds<T>& b) {
  b.sqL = sqrt(L[0]);
  b.sqR = sqrt(R[0]);
  b.inv = apdiv(T(1), b.sqL + b.sqR);
  b.Q0 = sqrt(L[0] * R[0]);
  b.n1 = L[1] * b.sqL + R[1] * b.sqR;
  b.n3 = L[3] * b.sqL + R[3] * b.sqR;
  b.Q1 = b.n1 * b.inv;
  b.Q3 = b.n3 * b.inv;
  b.aL = sqrt(apdiv(G.g * L[3], L[0]));
  b.aR = sqrt(apdiv(G.g * R[3], R[0]));
  b.aQ = sqrt(apdiv(G.g * b.Q3, b.Q0));
  b.rs0 = b.Q1 - b.aQ;
  b.rf0 = b.Q1 + b.aQ;
  const T slowL = L[1] - b.aL, fastL = L[1] + b.aL, slowR = R[1] - b.aR, fastR = R[1] + b.aR;
  const T tp0 = twice(slowR - slowL), tm0 = twice(fastR - fastL);
  b.tp_pos = is_pos(tp0);
  b.tm_pos = is_pos(tm0);
  b.tp = b.tp_pos ? tp0 : T(1e-8);
  b.tm = b.tm_pos ? tm0 : T(1e-8);
  b.cs = vlt(T(fabs(b.rs0)), b.tp);
  b.cf = vlt(T(fabs(b.rf0)), b.tm);
  const T rs = b.cs ? half(aqdiv(b.rs0 * b.rs0, b.tp) + b.tp) : b.rs0;
  const T rf = b.cf ? half(aqdiv(b.rf0 * b.rf0, b.tm) + b.tm) : b.rf0;
  b.plus_fastR = !vlt(fastR, rf);
  b.minus_slowL = !vlt(rs, slowL);
  b.Lp = b.plus_fastR ? fastR : rf;
  b.Lm = b.minus_slowL ? slowL : rs;
}

// reverse of hll_bounds (+ the Roe average's u and a~): lL, lR += the adjoints of
// L+, L-, u and a~ pulled back to the states
template <typename T>
__device__ __forceinline__ void hll_bounds_vjp(const T* L, const T* R, const Gas<T>& G, const HllBounds<T>& b, T lLp,
                                               T lLm, T lu, T laQ_in, T* lL, T* lR) {
  T lslowL = T(0), lfastL = T(0), lslowR = T(0), lfastR = T(0), lrs = T(0), lrf = T(0);
  if (b.plus_fastR) lfastR += lLp; else lrf += lLp;
  if (b.minus_slowL) lslowL += lLm; else lrs += lLm;
  // Harten's correction of the Roe speeds
  T lrs0 = lrs, lrf0 = lrf, ltp = T(0), ltm = T(0);
  if (b.cs) {
    lrs0 = lrs * aqdiv(b.rs0, b.tp);
    ltp = half(lrs) * (T(1) - aqdiv(b.rs0 * b.rs0, b.tp * b.tp));
  }
  if (b.cf) {
    lrf0 = lrf * aqdiv(b.rf0, b.tm);
    ltm = half(lrf) * (T(1) - aqdiv(b.rf0 * b.rf0, b.tm * b.tm));
  }
  if (!b.tp_pos) ltp = T(0);
  if (!b.tm_pos) ltm = T(0);
  lslowR += twice(ltp);
  lslowL -= twice(ltp);
  lfastR += twice(ltm);
  lfastL -= twice(ltm);
  // rs0 = u - aQ, rf0 = u + aQ; slow/fast = W1 -/+ a
  const T lQ1 = lu + lrs0 + lrf0;
  const T laQ = laQ_in + lrf0 - lrs0;
  lR[1] += lslowR + lfastR;
  lL[1] += lslowL + lfastL;
  const T laR = lfastR - lslowR, laL = lfastL - lslowL;
  // sound speeds a = sqrt(g p / rho)
  lR[0] += aqdiv(-laR * G.g * R[3], twice(b.aR) * R[0] * R[0]);
  lR[3] += aqdiv(laR * G.g, twice(b.aR) * R[0]);
  lL[0] += aqdiv(-laL * G.g * L[3], twice(b.aL) * L[0] * L[0]);
  lL[3] += aqdiv(laL * G.g, twice(b.aL) * L[0]);
  const T lQ3 = aqdiv(laQ * G.g, twice(b.aQ) * b.Q0);
  const T lQ0 = aqdiv(-laQ * G.g * b.Q3, twice(b.aQ) * b.Q0 * b.Q0);
  // Roe average (Q2 does not enter these fluxes)
  const T linv = lQ1 * b.n1 + lQ3 * b.n3;
  lL[1] += lQ1 * b.inv * b.sqL;
  lR[1] += lQ1 * b.inv * b.sqR;
  lL[3] += lQ3 * b.inv * b.sqL;
  lR[3] += lQ3 * b.inv * b.sqR;
  const T lsqL = (lQ1 * L[1] + lQ3 * L[3]) * b.inv - b.inv * b.inv * linv;
  const T lsqR = (lQ1 * R[1] + lQ3 * R[3]) * b.inv - b.inv * b.inv * linv;
  lL[0] += aqdiv(lQ0 * R[0], twice(b.Q0)) + aqdiv(lsqL, twice(b.sqL));
  lR[0] += aqdiv(lQ0 * L[0], twice(b.Q0)) + aqdiv(lsqR, twice(b.sqR));
}

// U = prim_to_cons(W) and F = {U1, U1 W1 + W3, U1 W2, W1 (U3 + W3)} (PrimitiveState.F
// with U): the forward values, and lW += (dU/dW)^T lU + (dF/dW)^T lF.
template <typename T>
__device__ __forceinline__ void cons_and_flux(const T* W, const Gas<T>& G, T* U, T* F) {
  prim_to_cons(W, G, U);
  F[0] = U[1];
  F[1] = U[1] * W[1] + W[3];
  F[2] = U[1] * W[2];
  F[3] = W[1] * (U[3] + W[3]);
}
template <typename T>
__device__ __forceinline__ void cons_and_flux_vjp(const T* W, const Gas<T>& G, const T* U, const T* lF, const T* lU_in,
                                                  T* lW) {
  T lU[4] = {lU_in[0], lU_in[1], lU_in[2], lU_in[3]};
  lU[1] += lF[0] + lF[1] * W[1] + lF[2] * W[2];
  lU[3] += lF[3] * W[1];
  lW[1] += lF[1] * U[1] + lF[3] * (U[3] + W[3]);
  lW[2] += lF[2] * U[1];
  lW[3] += lF[1] + lF[3] * W[1];
  // U = {W0, W0 W1, W0 W2, W3 / gm1 + 0.5 W0 (W1^2 + W2^2)}
  lW[0] += lU[0] + lU[1] * W[1] + lU[2] * W[2] + lU[3] * half(W[1] * W[1] + W[2] * W[2]);
  lW[1] += lU[1] * W[0] + lU[3] * W[0] * W[1];
  lW[2] += lU[2] * W[0] + lU[3] * W[0] * W[2];
  lW[3] += apdiv(lU[3], G.gm1);
}

// F = hlll_flux(WL, WR) (pyhype/flux/HLLL.py:25-103).  Subgradients: the branch the
// forward takes; alpha = max(0, 1 - |r|/k) passes nothing back where it is 0; the
// norms pass nothing back at a zero vector; max(u/L-, u/L+) the operand selected.
template <typename T>
__device__ void hlll_flux_vjp(const T* L, const T* R, const Gas<T>& G, const T* lF, T* lL, T* lR) {
  HllBounds<T> b;
  hll_bounds(L, R, G, b);
  T UL[4], UR[4], FL[4], FR[4];
  cons_and_flux(L, G, UL, FL);
  cons_and_flux(R, G, UR, FR);
  const T zero4[4] = {T(0), T(0), T(0), T(0)};
  if (b.Lm >= T(0)) {
    cons_and_flux_vjp(L, G, UL, lF, zero4, lL);
    return;
  }
  if (b.Lp <= T(0)) {
    cons_and_flux_vjp(R, G, UR, lF, zero4, lR);
    return;
  }
  const T Lp = b.Lp, Lm = b.Lm, u = b.Q1;
  T dU[4], rr[4];
#pragma unroll
  for (int v = 0; v < 4; ++v) {
    dU[v] = UR[v] - UL[v];
    rr[v] = (FR[v] - FL[v]) - u * dU[v];
  }
  const T nd = norm4(dU[0], dU[1], dU[2], dU[3]);
  const T kk = b.aQ * nd;
  const T nr = norm4(rr[0], rr[1], rr[2], rr[3]);
  const T den_k = (kk < T(1e-16)) ? kk + T(1e-14) : kk;
  const T x = T(1) - qdiv(nr, den_k);
  const bool alpha_pos = vlt(T(0), x);
  const T alpha = alpha_pos ? x : T(0);
  const T qm = qdiv(u, Lm), qp = qdiv(u, Lp);
  const bool m_sel = !vlt(qm, qp);
  const T M = m_sel ? qm : qp;
  const T Bv = T(1) - alpha * (T(1) - M);
  const T sc = Lm * Lp * Bv;
  const T den = Lp - Lm;
  // reverse
  T g[4], lFL[4], lFR[4], ldU[4];
  T lsc = T(0), lden = T(0), lLp = T(0), lLm = T(0);
#pragma unroll
  for (int v = 0; v < 4; ++v) {
    g[v] = pdiv(lF[v], den);
    const T Fv = pdiv(Lp * FL[v] - Lm * FR[v] + sc * dU[v], den);
    lFL[v] = Lp * g[v];
    lFR[v] = -Lm * g[v];
    ldU[v] = sc * g[v];
    lsc += g[v] * dU[v];
    lden -= g[v] * Fv;
    lLp += g[v] * FL[v];
    lLm -= g[v] * FR[v];
  }
  lLp += lden;
  lLm -= lden;
  lLm += lsc * Lp * Bv;
  lLp += lsc * Lm * Bv;
  const T lB = lsc * Lm * Lp;
  const T lalpha = -lB * (T(1) - M);
  const T lM = lB * alpha;
  T lu = T(0);
  if (m_sel) {
    lu += qdiv(lM, Lm);
    lLm -= lM * qdiv(qm, Lm);
  } else {
    lu += qdiv(lM, Lp);
    lLp -= lM * qdiv(qp, Lp);
  }
  T lnr = T(0), lkk = T(0);
  if (alpha_pos) {
    lnr = -qdiv(lalpha, den_k);
    lkk = lalpha * qdiv(qdiv(nr, den_k), den_k);
  }
  const T laQ_k = lkk * nd;
  const T lnd = lkk * b.aQ;
  if (nd > T(0)) {
#pragma unroll
    for (int v = 0; v < 4; ++v) ldU[v] += lnd * qdiv(dU[v], nd);
  }
  if (nr > T(0)) {
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const T lr = lnr * qdiv(rr[v], nr);
      lFR[v] += lr;
      lFL[v] -= lr;
      lu -= lr * dU[v];
      ldU[v] -= u * lr;
    }
  }
  T lUL[4], lUR[4];
#pragma unroll
  for (int v = 0; v < 4; ++v) {
    lUR[v] = ldU[v];
    lUL[v] = -ldU[v];
  }
  cons_and_flux_vjp(L, G, UL, lFL, lUL, lL);
  cons_and_flux_vjp(R, G, UR, lFR, lUR, lR);
  hll_bounds_vjp(L, R, G, b, lLp, lLm, lu, laQ_k, lL, lR);  // a~ also enters k = a~ |dU|
}

// F = hlle_flux(WL, WR) (pyhype/flux/HLLE.py:22-47): F_R where L+ <= 0, else F_L where
// L- >= 0, else (L+ F_L - L- F_R + L- L+ (U_R - U_L)) / (L+ - L-).
template <typename T>
__device__ void hlle_flux_vjp(const T* L, const T* R, const Gas<T>& G, const T* lF, T* lL, T* lR) {
  HllBounds<T> b;
  hll_bounds(L, R, G, b);
  T UL[4], UR[4], FL[4], FR[4];
  cons_and_flux(L, G, UL, FL);
  cons_and_flux(R, G, UR, FR);
  const T zero4[4] = {T(0), T(0), T(0), T(0)};
  if (b.Lp <= T(0)) {
    cons_and_flux_vjp(R, G, UR, lF, zero4, lR);
    return;
  }
  if (b.Lm >= T(0)) {
    cons_and_flux_vjp(L, G, UL, lF, zero4, lL);
    return;
  }
  const T Lp = b.Lp, Lm = b.Lm;
  const T den = Lp - Lm, LL = Lm * Lp;
  T lFL[4], lFR[4], lUL[4], lUR[4];
  T lLL = T(0), lden = T(0), lLp = T(0), lLm = T(0);
#pragma unroll
  for (int v = 0; v < 4; ++v) {
    const T dU = UR[v] - UL[v];
    const T gv = pdiv(lF[v], den);
    const T Fv = pdiv(Lp * FL[v] - Lm * FR[v] + LL * dU, den);
    lFL[v] = Lp * gv;
    lFR[v] = -Lm * gv;
    lUR[v] = LL * gv;
    lUL[v] = -LL * gv;
    lLL += gv * dU;
    lden -= gv * Fv;
    lLp += gv * FL[v];
    lLm -= gv * FR[v];
  }
  lLp += lden + lLL * Lm;
  lLm += -lden + lLL * Lp;
  cons_and_flux_vjp(L, G, UL, lFL, lUL, lL);
  cons_and_flux_vjp(R, G, UR, lFR, lUR, lR);
  hll_bounds_vjp(L, R, G, b, lLp, lLm, T(0), T(0), lL, lR);
}

template <int FLUX, typename T>
__device__ __forceinline__ void riemann_vjp(const T* L, const T* R, const Gas<T>& G, const T* lF, T* lL, T* lR) {
  if (FLUX == E2D_FLUX_HLLL) hlll_flux_vjp(L, R, G, lF, lL, lR);
  else if (FLUX == E2D_FLUX_HLLE) hlle_flux_vjp(L, R, G, lF, lL, lR);
  else roe_flux_vjp(L, R, G, lF, lL, lR);
}

}  // namespace e2d
