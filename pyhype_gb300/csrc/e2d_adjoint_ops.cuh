// e2d_adjoint_ops.cuh - hand-written reverse-mode (vector-Jacobian) products of the
// pointwise pieces of the scheme: the Roe flux, the conservative->primitive
// conversion, the rotations and the reflection, and the limiter functions.
//
// Each *_vjp recomputes the forward intermediates it needs from the forward inputs
// and accumulates lambda^T * d(output)/d(input) into the input adjoints.  Branches
// (Harten's entropy fix, |x|) take the derivative of the branch the forward took;
// at a tie the forward's own selection decides.
#pragma once
#include "e2d_device.cuh"

namespace e2d {

template <typename T>
__device__ __forceinline__ T sgn(T x) { return x > T(0) ? T(1) : (x < T(0) ? T(-1) : T(0)); }

// W = cons_to_prim(U): lamU += (dW/dU)^T lamW
template <typename T>
__device__ __forceinline__ void cons_to_prim_vjp(const T* U, const Gas<T>& G, const T* lW, T* lU) {
  const T rho = U[0];
  const T u = qdiv(U[1], rho), v = qdiv(U[2], rho);
  // p = gm1 * (E - rho * 0.5 * (u*u + v*v))
  const T lp = lW[3];
  T lu = lW[1] - lp * G.gm1 * rho * u;
  T lv = lW[2] - lp * G.gm1 * rho * v;
  T lrho = lW[0] - half(lp * G.gm1) * (u * u + v * v);
  // u = rhou / rho, v = rhov / rho
  lU[1] += qdiv(lu, rho);
  lU[2] += qdiv(lv, rho);
  lU[0] += lrho - qdiv(lu * u + lv * v, rho);
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
    return pdiv((sgn(s) + T(1)) - qdiv(fabs(s) + s, d), d);
  }
  if (vlt(sizeof(T) == 4 ? T(SLOPE_CAP_FP32) : T(SLOPE_CAP_FP64), s)) return T(0);  // capped: constant
  if (LIM == E2D_LIM_VAN_ALBADA) {  // (s^2 + s)/(s^2 + 1)
    const T d = s * s + T(1);
    return pdiv(pdiv(T(1) + twice(s) - s * s, d), d);
  }
  const T d = s * s + s + T(2);  // Venkatakrishnan (s^2 + 2s)/(s^2 + s + 2)
  return pdiv(pdiv(T(4) + T(4) * s - s * s, d), d);
}

// F = roe_flux(WL, WR): lamWL += (dF/dWL)^T lamF, lamWR += (dF/dWR)^T lamF
template <typename T>
__device__ void roe_flux_vjp(const T* L, const T* R, const Gas<T>& G, const T* lF, T* lL, T* lR) {
  // ---- forward (same expressions as roe_flux) ----
  const T sqL = sqrt(L[0]), sqR = sqrt(R[0]);
  const T inv = pdiv(T(1), sqL + sqR);
  const T Q0 = sqrt(L[0] * R[0]);
  const T n1 = L[1] * sqL + R[1] * sqR, n2 = L[2] * sqL + R[2] * sqR, n3 = L[3] * sqL + R[3] * sqR;
  const T Q1 = n1 * inv, Q2 = n2 * inv, Q3 = n3 * inv;
  const T aR = sqrt(pdiv(G.g * R[3], R[0])), aL = sqrt(pdiv(G.g * L[3], L[0])), aQ = sqrt(pdiv(G.g * Q3, Q0));
  const T Lm0 = Q1 - aQ, Lp0 = Q1 + aQ;
  const T slowR = R[1] - aR, fastR = R[1] + aR, slowL = L[1] - aL, fastL = L[1] + aL;
  const T tp0 = twice(slowR - slowL), tm0 = twice(fastR - fastL);
  const bool tp_pos = is_pos(tp0), tm_pos = is_pos(tm0);
  const T tp = tp_pos ? tp0 : T(1e-8), tm = tm_pos ? tm0 : T(1e-8);
  const bool cm = vlt(T(fabs(Lm0)), tp), cp = vlt(T(fabs(Lp0)), tm);
  const T Lm = cm ? half(qdiv(Lm0 * Lm0, tp) + tp) : Lm0;
  const T Lp = cp ? half(qdiv(Lp0 * Lp0, tm) + tm) : Lp0;
  const T Ek = half(Q1 * Q1 + Q2 * Q2);
  const T H = pdiv(G.gm * Q3, Q0) + Ek;
  const T ua = Q1 * aQ;
  const T ia = pdiv(T(1), aQ);
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
  T lQ3 = pdiv(G.gm, Q0) * lH;
  lQ0 += pdiv(-G.gm * Q3, Q0 * Q0) * lH;
  lEk += lH;
  lQ1 += Q1 * lEk;
  lQ2 += Q2 * lEk;
  // Harten
  T lLm0 = lLm, lLp0 = lLp, ltp = T(0), ltm = T(0);
  if (cm) {
    lLm0 = lLm * qdiv(Lm0, tp);
    ltp = half(lLm) * (T(1) - qdiv(Lm0 * Lm0, tp * tp));
  }
  if (cp) {
    lLp0 = lLp * qdiv(Lp0, tm);
    ltm = half(lLp) * (T(1) - qdiv(Lp0 * Lp0, tm * tm));
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
  T lR0 = qdiv(-laR * G.g * R[3], twice(aR) * R[0] * R[0]);
  T lR3 = qdiv(laR * G.g, twice(aR) * R[0]);
  T lL0 = qdiv(-laL * G.g * L[3], twice(aL) * L[0] * L[0]);
  T lL3 = qdiv(laL * G.g, twice(aL) * L[0]);
  lQ3 += qdiv(laQ * G.g, twice(aQ) * Q0);
  lQ0 += qdiv(-laQ * G.g * Q3, twice(aQ) * Q0 * Q0);
  // Roe averages
  const T linv = lQ1 * n1 + lQ2 * n2 + lQ3 * n3;
  lL1 += lQ1 * inv * sqL;
  lR1 += lQ1 * inv * sqR;
  T lL2 = lQ2 * inv * sqL, lR2 = lQ2 * inv * sqR;
  lL3 += lQ3 * inv * sqL;
  lR3 += lQ3 * inv * sqR;
  T lsqL = (lQ1 * L[1] + lQ2 * L[2] + lQ3 * L[3]) * inv - inv * inv * linv;
  T lsqR = (lQ1 * R[1] + lQ2 * R[2] + lQ3 * R[3]) * inv - inv * inv * linv;
  lL0 += qdiv(lQ0 * R[0], twice(Q0)) + qdiv(lsqL, twice(sqL));
  lR0 += qdiv(lQ0 * L[0], twice(Q0)) + qdiv(lsqR, twice(sqR));
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

}  // namespace e2d
