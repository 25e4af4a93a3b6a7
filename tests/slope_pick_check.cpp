// Host check of pick_slopes (pyhype_gb300/csrc/e2d_slope_pick.cuh): for random and
// adversarial cells, phi from psi at the picked faces equals phi from all four faces,
// bit for bit, and the picked face is the first face whose psi is phi (the selection
// the adjoint differentiates), for all four limiters.  The approximate reciprocal of the device is
// replaced by the correctly rounded one perturbed by up to +-2 ulp at random, which is
// wider than the device instruction's stated 1 ulp.
//
// Build: g++ -O2 -std=c++17 -ffp-contract=off slope_pick_check.cpp
// Run:   ./a.out <cases per limiter> <seed>     prints two lines per limiter, four
//        candidates ("<lim> cases=...") and 8 or 12 ("<lim>+ cases=..."):
//        "<lim> cases=<n> mismatches=<m> fallback=<f> second=<s>"
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>

static std::mt19937_64 g_rng;

// Like the device instruction, the stand-in is a function of its input: the
// perturbation (-2..+2 ulp) is drawn from a hash of the input bits and a per-run salt.
static uint32_t g_salt = 0;
static float perturbed_rcp(float x) {
  float y = 1.0f / x;
  uint32_t u, xb;
  std::memcpy(&u, &y, sizeof u);
  std::memcpy(&xb, &x, sizeof xb);
  uint32_t hsh = (xb ^ g_salt) * 0x9e3779b1u;
  hsh ^= hsh >> 15;
  u += (int)(hsh % 5) - 2;
  std::memcpy(&y, &u, sizeof y);
  return y;
}
#define E2D_SLOPE_PICK_HOST_RCP perturbed_rcp
#include "../pyhype_gb300/csrc/e2d_slope_pick.cuh"

static uint64_t bits(double x) {
  uint64_t b;
  std::memcpy(&b, &x, sizeof b);
  return b;
}
static double from(uint64_t b) {
  double x;
  std::memcpy(&x, &b, sizeof x);
  return x;
}
// the device's ordered min/max and sign tests (e2d_device.cuh)
static long long okey(double x) {
  const long long b = (long long)bits(x);
  return b ^ ((b >> 63) & 0x7fffffffffffffffLL);
}
static double vmin(double a, double b) { return okey(a) <= okey(b) ? a : b; }
static double vmax(double a, double b) { return okey(a) >= okey(b) ? a : b; }
static bool is_pos(double x) {
  const long long b = (long long)bits(x);
  return b > 0 && b <= 0x7ff0000000000000LL;
}
static bool is_neg(double x) {
  const long long k = okey(x);
  return k < -1 && k >= (long long)0x800fffffffffffffULL;
}

// psi of pyhype/limiters/limiters.py:25-62 with the 1e30 slope cap, as the device has it
template <int LIM>
static double psi(double s) {
  if (LIM == 0 || LIM == 2) s = vmin(s, 1e30);
  if (LIM == 1) return vmin(1.0, s);
  if (LIM == 2) {
    const double s2 = s * s;
    return (s2 + s) / (s2 + 1.0);
  }
  if (LIM == 3) return (std::fabs(s) + s) / (s + 1.0);
  const double s2 = s * s;
  return (s2 + 2.0 * s) / (s2 + s + 2.0);
}
template <int LIM>
static double psi_s(double s) {
  if (bits(s) == 0x3ff0000000000000ULL) return LIM == 0 ? 0.75 : 1.0;
  return psi<LIM>(s);
}

// phi over all four faces, and the first face whose psi is phi (the selection the
// adjoint differentiates)
template <int LIM, int N>
static double phi_all(double dmax, double dmin, const double (&davg)[N], int& sel) {
  double ph = 0.0;
  sel = 0;
  for (int s = 0; s < N; ++s) {
    const bool pos = is_pos(davg[s]), neg = is_neg(davg[s]);
    const double p = psi_s<LIM>((pos || neg) ? (pos ? dmax : dmin) / davg[s] : 1.0);
    if (s > 0 && okey(p) < okey(ph)) sel = s;
    ph = (s == 0) ? p : vmin(ph, p);
  }
  return ph;
}

struct Counts {
  long cases = 0, mismatches = 0, fallback = 0, second = 0;
};

template <int LIM, int N>
static void check_cell(double w0, const double (&nb)[4], const double (&hot)[N], Counts& c) {
  const double dmax = vmax(vmax(vmax(vmax(w0, nb[0]), nb[1]), nb[2]), nb[3]) - w0;
  const double dmin = vmin(vmin(vmin(vmin(w0, nb[0]), nb[1]), nb[2]), nb[3]) - w0;
  double davg[N];
  for (int s = 0; s < N; ++s) davg[s] = (w0 + hot[s]) - w0;
  int sel_ref;
  const double ref = phi_all<LIM, N>(dmax, dmin, davg, sel_ref);
  const e2d::SlopePick k = e2d::pick_slopes<LIM, N>(dmax, dmin, davg);
  ++c.cases;
  if (!k.ok) {
    ++c.fallback;
    return;
  }
  double ph = psi_s<LIM>(k.ga ? k.na / k.da : 1.0);
  int sel = k.fa;
  if (LIM == 1 && bits(ph) == bits(1.0)) sel = 0;  // Barth-Jespersen's plateau: every face gives 1
  if (k.second) {
    ++c.second;
    const double pb = psi_s<LIM>(k.gb ? k.nb / k.db : 1.0);
    if (okey(pb) < okey(ph) || (bits(pb) == bits(ph) && k.fb < k.fa)) sel = k.fb;
    ph = vmin(ph, pb);
  }
  if (!std::isnan(ref) && sel != sel_ref) {
    if (c.mismatches < 5) std::fprintf(stderr, "LIM %d face %d, all faces %d\n", LIM, sel, sel_ref);
    ++c.mismatches;
  }
  if (bits(ph) != bits(ref) && !(std::isnan(ph) && std::isnan(ref))) {
    if (c.mismatches < 5)
      std::fprintf(stderr, "LIM %d N %d mismatch: w0=%a nb=%a %a %a %a hot0=%a phi=%a ref=%a\n", LIM, N, w0, nb[0],
                   nb[1], nb[2], nb[3], hot[0], ph, ref);
    ++c.mismatches;
  }
}

static double unif(double a, double b) { return a + (b - a) * ((g_rng() >> 11) * 0x1.0p-53); }
static double logu(double lo_exp, double hi_exp) { return std::ldexp(1.0, 0) * std::exp2(unif(lo_exp, hi_exp)); }
static double sgn() { return (g_rng() & 1) ? 1.0 : -1.0; }
static double ulps(double x, long n) { return from(bits(x) + n); }

// one random cell of kind `kind`
static void make_cell(int kind, double& w0, double (&nb)[4], double (&hot)[4]) {
  const double scale = (g_rng() % 8 == 0) ? std::exp2(std::floor(unif(-1070, 1020))) : logu(-20, 20);
  w0 = sgn() * scale * unif(0.1, 10);
  const double g = scale * logu(-20, 2);
  switch (kind) {
    case 0:  // unrelated neighbours and face terms
      for (int s = 0; s < 4; ++s) {
        nb[s] = w0 + sgn() * scale * logu(-30, 1);
        hot[s] = sgn() * g * unif(0, 1);
      }
      break;
    case 1: {  // smooth: linear profile plus small noise, mirror-symmetric face terms
      const double gx = sgn() * g, gy = sgn() * g * unif(0, 1);
      const double eps = (g_rng() & 1) ? 0.0 : g * logu(-40, -5);
      nb[0] = w0 + gx + eps * unif(-1, 1);
      nb[1] = w0 - gx + eps * unif(-1, 1);
      nb[2] = w0 + gy + eps * unif(-1, 1);
      nb[3] = w0 - gy + eps * unif(-1, 1);
      hot[0] = 0.5 * gx; hot[1] = -0.5 * gx; hot[2] = 0.5 * gy; hot[3] = -0.5 * gy;
      break;
    }
    case 2: {  // exact and 1-ulp ties between faces
      const double h = sgn() * g * unif(0.1, 1);
      for (int s = 0; s < 4; ++s) {
        nb[s] = w0 + sgn() * g * unif(0.5, 2);
        const long d = (long)(g_rng() % 7) - 3;
        hot[s] = (g_rng() % 3 == 0) ? -h : ulps(h, (g_rng() & 1) ? 0 : d);
      }
      break;
    }
    case 3:  // uniform region: round-off sized face terms, some exactly zero
      for (int s = 0; s < 4; ++s) {
        nb[s] = (g_rng() & 1) ? w0 : ulps(w0, (long)(g_rng() % 5) - 2);
        hot[s] = (g_rng() % 3 == 0) ? 0.0 : sgn() * std::fabs(w0) * logu(-60, -48);
      }
      break;
    case 4: {  // slopes near the limiters' special points (1, 2, the peaks, 1e8, the cap)
      static const double targets[] = {0.0, 1.0, 2.0, 4.828427124746190, 2.414213562373095, 1e8, 1e30, 1e17};
      const double d = g;
      nb[0] = w0 + d; nb[1] = w0 - d * unif(0.5, 2); nb[2] = w0; nb[3] = w0;
      for (int s = 0; s < 4; ++s) {
        const double t = targets[g_rng() % 8] * (1 + sgn() * logu(-52, -3) * (g_rng() & 1));
        const double num = (s & 1) ? -d : d;
        hot[s] = t > 0 ? num / t : 0.0;
      }
      break;
    }
    case 5: {  // several slopes on the falling branch, a little apart
      const double d = g, sb = std::exp2(unif(3, 60));
      nb[0] = w0 + d; nb[1] = w0 - d; nb[2] = w0; nb[3] = w0;
      for (int s = 0; s < 4; ++s) {
        const double t = (s == 0 && (g_rng() & 1)) ? unif(2, 6) : sb * (1 - logu(-20, -4));
        hot[s] = ((s & 1) ? -d : d) / t;
      }
      break;
    }
    default: {  // special values: zeros of both signs, subnormals, infinities, NaN
      static const double sp[] = {0.0, -0.0, 0x1p-1074, -0x1p-1060, INFINITY, -INFINITY, NAN, 1e308};
      for (int s = 0; s < 4; ++s) {
        nb[s] = (g_rng() % 4 == 0) ? sp[g_rng() % 8] : w0 + sgn() * g;
        hot[s] = (g_rng() % 4 == 0) ? sp[g_rng() % 8] : sgn() * g * unif(0, 1);
      }
      if (g_rng() % 4 == 0) w0 = sp[g_rng() % 8];
    }
  }
}

// N > 4 candidates (several face quadrature points): the cell's four face terms,
// then more made from them: exact copies, one-ulp neighbours, relative 1e-6 and
// 1e-4 changes, sign flips and unrelated values
template <int N>
static void extend(const double (&h4)[4], double (&hot)[N]) {
  for (int s = 0; s < 4; ++s) hot[s] = h4[s];
  for (int s = 4; s < N; ++s) {
    const double b = h4[g_rng() % 4];
    switch (g_rng() % 6) {
      case 0: hot[s] = b; break;
      case 1: hot[s] = ulps(b, (long)(g_rng() % 5) - 2); break;
      case 2: hot[s] = b * (1 + 1e-6 * sgn()); break;
      case 3: hot[s] = b * (1 + 1e-4 * sgn()); break;
      case 4: hot[s] = -b; break;
      default: hot[s] = b * unif(-3, 3);
    }
  }
}

template <int LIM, int N>
static Counts run(long n) {
  Counts c;
  g_salt = (uint32_t)g_rng();
  for (long i = 0; i < n; ++i) {
    double w0, nb[4], h4[4], hot[N];
    make_cell((int)(i % 7), w0, nb, h4);
    extend<N>(h4, hot);
    check_cell<LIM, N>(w0, nb, hot, c);
  }
  return c;
}

int main(int argc, char** argv) {
  const long n = argc > 1 ? std::atol(argv[1]) : 1000000;
  g_rng.seed(argc > 2 ? std::strtoull(argv[2], nullptr, 10) : 1);
  // the four faces, and 2 and 3 face quadrature points (8 and 12 candidates)
  const Counts c[4] = {run<0, 4>(n), run<1, 4>(n), run<2, 4>(n), run<3, 4>(n)};
  const Counts q[4] = {run<0, 12>(n / 2), run<1, 8>(n / 2), run<2, 12>(n / 2), run<3, 8>(n / 2)};
  long bad = 0;
  for (int l = 0; l < 4; ++l) {
    std::printf("%d cases=%ld mismatches=%ld fallback=%ld second=%ld\n", l, c[l].cases, c[l].mismatches,
                c[l].fallback, c[l].second);
    std::printf("%d+ cases=%ld mismatches=%ld fallback=%ld second=%ld\n", l, q[l].cases, q[l].mismatches,
                q[l].fallback, q[l].second);
    bad += c[l].mismatches + q[l].mismatches;
  }
  return bad ? 1 : 0;
}
