// Host check of half()/twice() (pyhype_gb300/csrc/e2d_pow2.cuh) against the IEEE
// multiplications x * 0.5 and x * 2.0: every exponent field, random significands and
// signs, plus the boundary patterns.  Prints "cases=<n> mismatches=<m>".
// Build: g++ -O2 -std=c++17 -ffp-contract=off pow2_check.cpp
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <random>

#include "../pyhype_gb300/csrc/e2d_pow2.cuh"

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

int main(int argc, char** argv) {
  const long per_exp = argc > 1 ? std::atol(argv[1]) : 2000;
  std::mt19937_64 rng(argc > 2 ? std::strtoull(argv[2], nullptr, 10) : 1);
  long cases = 0, bad = 0;
  auto check = [&](uint64_t b) {
    const double x = from(b);
    const double h = e2d::half(x), t = e2d::twice(x);
    const double rh = x * 0.5, rt = x * 2.0;
    ++cases;
    const bool ok_h = std::isnan(rh) ? std::isnan(h) : bits(h) == bits(rh);
    const bool ok_t = std::isnan(rt) ? std::isnan(t) : bits(t) == bits(rt);
    if (!ok_h || !ok_t) {
      if (bad < 5) std::fprintf(stderr, "x=%a half=%a (%a) twice=%a (%a)\n", x, h, rh, t, rt);
      ++bad;
    }
  };
  const uint64_t edge_m[] = {0, 1, 2, 3, 0x000fffffffffffffULL, 0x0008000000000000ULL, 0x0007ffffffffffffULL,
                             0x000ffffffffffffeULL, 0x0008000000000001ULL};
  for (uint64_t s = 0; s < 2; ++s)
    for (uint64_t e = 0; e < 2048; ++e) {
      for (uint64_t m : edge_m) check((s << 63) | (e << 52) | m);
      for (long k = 0; k < per_exp; ++k) check((s << 63) | (e << 52) | (rng() & 0x000fffffffffffffULL));
    }
  std::printf("cases=%ld mismatches=%ld\n", cases, bad);
  return bad ? 1 : 0;
}
