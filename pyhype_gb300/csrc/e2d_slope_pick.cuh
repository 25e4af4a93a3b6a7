// e2d_slope_pick.cuh - which faces' limiter values decide a cell's phi (FP64 path).
//
// The limiter (pyhype/limiters/base.py:47-221) evaluates psi at the slope of each of
// the four faces, s_F = dmax/davg_F (davg_F > 0), dmin/davg_F (davg_F < 0) or 1
// (davg_F == 0), and keeps the minimum: phi = min_F psi(s_F).  In FP64 on GB300 every
// slope and every psi costs a correctly rounded division on the FP64 pipe, the
// scheme's binding resource, so evaluating all four faces is the largest single cost
// of the reconstruction kernel.
//
// All four limiter functions are unimodal in s >= 0 (every slope is >= 0: dmax >= 0,
// dmin <= 0, davg of the same sign):
//   Venkatakrishnan (s^2+2s)/(s^2+s+2)  rises to 1.094 at s = 2+2*sqrt(2), then falls to 1;
//                                       below 1 exactly for s < 2;
//   van Albada      (s^2+s)/(s^2+1)     rises to 1.207 at s = 1+sqrt(2), then falls to 1;
//                                       below 1 exactly for s < 1;
//   van Leer        2s/(s+1)            increasing;
//   Barth-Jespersen min(1, s)           non-decreasing, and exactly so after rounding.
// So the minimum over the faces is psi at the smallest slope, or (for the two peaked
// functions when the smallest slope is already at or above the point where psi
// reaches 1) the smaller of psi at the smallest and at the largest slope.  Which face
// has the smallest and largest slope is decided from FP32 estimates of the slopes
// formed from the doubles' bits (integer and FP32 pipes); only the chosen faces get
// the FP64 slope division and psi.
//
// The pick is exact, not approximate, because it only chooses which faces to
// evaluate and gives up whenever that choice could change phi's bits:
//   * estimate error: mantissas truncated to 23 bits and an approximate reciprocal
//     (1 ulp) keep |s_est/s - 1| < 5e-7;
//   * a face whose estimate lies within a relative TAU = 1e-5 of the chosen smallest
//     (or largest) one is a near tie: unless its slope is provably the same double
//     (same |numerator| and |denominator| bits, both exactly 1, or both exactly 0)
//     the pick gives up;
//   * every other face then has an exact slope at least 0.88*TAU (relative) away from
//     the chosen ones, where psi differs by at least 8.8e-14 relative (2.6e-7 on the
//     rising branch below s = 4, 5.6e-12 at the flat peak, second order, and
//     0.88*TAU/s >= 8.8e-14 on the falling branch up to s = 1e8), far above the
//     7e-16 that the rounding of two psi evaluations can account for: its computed
//     psi is strictly larger than the chosen minimum;
//   * on the falling branch psi - 1 ~ 1/s, so the difference TAU/s must stay above the
//     rounding: the pick gives up when it would need psi at a slope above 1e8
//     (van Leer: when the smallest slope is above 1e8);
//   * operands that are zero-exponent (other than an exact zero numerator), infinite,
//     NaN, or whose ratio leaves 2^-100..2^100 have no estimate: the pick gives up;
//   * Barth-Jespersen passes a zero slope's sign through (psi(-0) = -0): zero slopes
//     of both signs make the pick give up.
// When it gives up the caller evaluates all four faces as before.  The division and
// psi expressions are unchanged, so phi is the same double in every case.
#pragma once
#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define E2D_HD __host__ __device__ __forceinline__
#else
#define E2D_HD inline
#endif

namespace e2d {

struct SlopePick {
  double na, da;  // slope operands of the face to evaluate
  double nb, db;  // and of the largest slope, needed too when `second`
  bool ga, gb;    // false: that slope is exactly 1 (davg == 0), not na/da
  bool second;    // phi = min(psi(na/da), psi(nb/db)); else phi = psi(na/da)
  bool ok;        // false: evaluate all four faces
  int fa, fb;     // their indices in den: the first candidate whose psi equals phi is
                  // fa, or with `second` the one of fa, fb whose psi is smaller (the
                  // lower index when both are equal)
};

namespace slope_pick_detail {

constexpr uint64_t kOneBits = 0x3ff0000000000000ULL;
constexpr uint64_t kInfBits = 0x7ff0000000000000ULL;
constexpr float kTau = 1e-5f;
constexpr float kFallingLimit = 1e8f;
constexpr float kPsiSep = 1e-5f;

E2D_HD uint64_t abs_bits(double x) {
#if defined(__CUDA_ARCH__)
  return (uint64_t)__double_as_longlong(x) & 0x7fffffffffffffffULL;
#else
  uint64_t b;
  std::memcpy(&b, &x, sizeof b);
  return b & 0x7fffffffffffffffULL;
#endif
}

E2D_HD float from_bits(uint32_t u) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(u);
#else
  float f;
  std::memcpy(&f, &u, sizeof f);
  return f;
#endif
}

E2D_HD float approx_rcp(float x) {
#if defined(__CUDA_ARCH__)
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
#elif defined(E2D_SLOPE_PICK_HOST_RCP)
  return E2D_SLOPE_PICK_HOST_RCP(x);  // a host test's stand-in for the approximate reciprocal
#else
  return 1.0f / x;
#endif
}

E2D_HD bool signbit_of(double x) {
#if defined(__CUDA_ARCH__)
  return __double2hiint(x) < 0;
#else
  uint64_t b;
  std::memcpy(&b, &x, sizeof b);
  return (b >> 63) != 0;
#endif
}

// davg > 0 or davg < 0 (the slope is a quotient; false for zeros and NaN)
E2D_HD bool nonzero(double x) {
  const uint64_t b = abs_bits(x);
  return b != 0 && b <= kInfBits;
}

// FP32 estimate of the slope |n|/|d| from absolute bit patterns.  The exponent
// difference goes into the numerator's float exponent and the denominator is scaled
// to [1, 2), so the estimate is a normal float for ratios within 2^-100..2^100.
E2D_HD float estimate(uint64_t n, uint64_t d, bool& ok) {
  if (n == d && n < kInfBits) { ok = true; return 1.0f; }  // s == 1 exactly (davg == 0, or n == d)
  if (n == 0 && d < kInfBits) { ok = true; return 0.0f; }  // s == +-0 exactly
  const uint32_t nh = (uint32_t)(n >> 32), nl = (uint32_t)n;
  const uint32_t dh = (uint32_t)(d >> 32), dl = (uint32_t)d;
  const int en = (int)(nh >> 20), ed = (int)(dh >> 20);
  const int diff = en - ed;
  ok = en >= 1 && en <= 2046 && ed >= 1 && ed <= 2046 && diff >= -100 && diff <= 100;
  const uint32_t mn = ((nh & 0xfffffu) << 3) | (nl >> 29);
  const uint32_t md = ((dh & 0xfffffu) << 3) | (dl >> 29);
  const float fn = from_bits(((uint32_t)(diff + 127) << 23) | mn);
  const float fd = from_bits((127u << 23) | md);
  return fn * approx_rcp(fd);
}

// FP32 value of the peaked limiter functions at a slope estimate (slopes above 1e15,
// where both equal 1 in FP32, are clamped so the squares stay finite)
template <int LIM>
E2D_HD float psi_estimate(float x) {
  x = x < 1e15f ? x : 1e15f;
  const float x2 = x * x;
  return LIM == 0 ? (x2 + 2.0f * x) * approx_rcp(x2 + x + 2.0f) : (x2 + x) * approx_rcp(x2 + 1.0f);
}

// The two slopes are the same double: same operand magnitudes (the quotient of
// magnitudes is sign-symmetric), both exactly 1, or both exactly 0.
E2D_HD bool same_slope(uint64_t n0, uint64_t d0, uint64_t n1, uint64_t d1) {
  return (n0 == n1 && d0 == d1 && n0 < kInfBits && d0 < kInfBits) || (n0 == d0 && n1 == d1 && n0 < kInfBits && n1 < kInfBits) ||
         (n0 == 0 && n1 == 0 && d0 < kInfBits && d1 < kInfBits);
}

}  // namespace slope_pick_detail

// LIM: E2D_LIM_* of euler2d.h (0 Venkatakrishnan, 1 Barth-Jespersen, 2 van Albada,
// 3 van Leer).  dmax >= 0, dmin <= 0: the cell's stencil extremes minus its value;
// den: davg of the N candidate points in the limiter's order (the E, W, N, S faces;
// with several face quadrature points, every point of E, then of W, N, S).  A slope
// is dmax/davg (davg > 0), dmin/davg (davg < 0) or exactly 1 (davg == 0).  fa, fb
// index den.
template <int LIM, int N = 4>
E2D_HD SlopePick pick_slopes(double dmax, double dmin, const double (&den)[N]) {
  using namespace slope_pick_detail;
  const uint64_t amax = abs_bits(dmax), amin = abs_bits(dmin);
  // per face: |numerator| and |denominator| bits (1, 1 for davg == 0) and the estimate
  auto operands = [&](int k, uint64_t& n, uint64_t& d) {
    const uint64_t b = abs_bits(den[k]);
    const bool gen = nonzero(den[k]);
    const bool pos = gen && !signbit_of(den[k]);
    n = gen ? (pos ? amax : amin) : kOneBits;
    d = gen ? b : kOneBits;
  };
  float se[N];
  bool ok = true, zpos = false, zneg = false;
#pragma unroll
  for (int k = 0; k < N; ++k) {
    uint64_t n, d;
    operands(k, n, d);
    bool okk;
    se[k] = estimate(n, d, okk);
    ok = ok && okk;
    if (LIM == 1 && n == 0) {  // a zero slope's sign: that of the numerator times den's
      const bool neg = signbit_of(den[k]) != signbit_of(signbit_of(den[k]) ? dmin : dmax);
      zneg = zneg || neg;
      zpos = zpos || !neg;
    }
  }
  // Barth-Jespersen's psi is min(1, s), so zero slopes of both signs give psi = +0 and
  // -0 and the ordered minimum keeps -0: give up rather than pick one of them
  if (LIM == 1 && zpos && zneg) ok = false;
  float smin = se[0], smax = se[0];
  int ia = 0, ib = 0;
#pragma unroll
  for (int k = 1; k < N; ++k) {
    if (se[k] < smin) { smin = se[k]; ia = k; }
    if (se[k] > smax) { smax = se[k]; ib = k; }
  }
  // psi(s) >= 1 from this slope on (both peaked functions); below it psi < 1 and only
  // the smallest slope matters.  Above it both ends are candidates; FP32 values of psi
  // at the two estimates decide which end is smaller when they differ by more than
  // kPsiSep (their error is below 1.5e-6), and both are evaluated when they do not.
  constexpr bool peaked = LIM == 0 || LIM == 2;
  constexpr float reach_one = LIM == 0 ? 1.99f : 0.99f;
  const bool ends = peaked && smin >= reach_one && ia != ib;
  bool use_a = true, use_b = false;
  if (ends) {
    const float pa = psi_estimate<LIM>(smin), pb = psi_estimate<LIM>(smax);
    use_a = !(pb < pa * (1.0f - kPsiSep));
    use_b = !(pa < pb * (1.0f - kPsiSep));
  }
  if (use_b && smax > kFallingLimit) ok = false;
  if (LIM == 3 && smin > kFallingLimit) ok = false;
  uint64_t nA = 0, dA = 0, nB = 0, dB = 0;  // operands of the two ends
#pragma unroll
  for (int k = 0; k < N; ++k) {  // unrolled selects: no indexed access to den
    uint64_t n, d;
    operands(k, n, d);
    if (k == ia) { nA = n; dA = d; }
    if (k == ib) { nB = n; dB = d; }
  }
  const float lo = smin * (1.0f + kTau), hi = smax * (1.0f - kTau);
#pragma unroll
  for (int k = 0; k < N; ++k) {
    uint64_t n, d;
    operands(k, n, d);
    if (use_a && k != ia && se[k] <= lo && !same_slope(n, d, nA, dA)) ok = false;
    if (use_b && k != ib && se[k] >= hi && !same_slope(n, d, nB, dB)) ok = false;
  }
  // first: the end to evaluate (a unless only b is needed); second: b as well
  SlopePick p;
  const int i1 = use_a ? ia : ib;
  p.da = den[0]; p.db = den[0];
#pragma unroll
  for (int k = 1; k < N; ++k) {
    if (k == i1) p.da = den[k];
    if (k == ib) p.db = den[k];
  }
  p.second = use_a && use_b;
  p.fa = i1;
  p.fb = ib;
  p.ga = nonzero(p.da);
  p.gb = nonzero(p.db);
  p.na = signbit_of(p.da) ? dmin : dmax;
  p.nb = signbit_of(p.db) ? dmin : dmax;
  p.ok = ok;
  return p;
}

}  // namespace e2d
