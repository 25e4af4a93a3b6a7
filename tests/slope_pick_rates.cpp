// How often the limiter's face pick (pyhype_gb300/csrc/e2d_slope_pick.cuh) gives up on
// real cell data.  Reads records of 6 doubles (dmax, dmin, davg of the E, W, N, S
// faces) from the file named by argv[1], in warp order (32 consecutive records are
// one warp's lanes for one variable), runs the Venkatakrishnan pick on each and prints
// "lanes=<n> fallback=<f> second=<s> warps=<w> warp_fallback=<wf> warp_second=<ws>".
// Build: g++ -O2 -std=c++17 -ffp-contract=off slope_pick_rates.cpp
#include <cstdio>
#include <vector>

#include "../pyhype_gb300/csrc/e2d_slope_pick.cuh"

int main(int argc, char** argv) {
  if (argc < 2) return 2;
  FILE* f = std::fopen(argv[1], "rb");
  if (!f) return 2;
  std::vector<double> r;
  double buf[6];
  while (std::fread(buf, sizeof(double), 6, f) == 6) r.insert(r.end(), buf, buf + 6);
  std::fclose(f);
  const long n = (long)r.size() / 6;
  long fb = 0, sec = 0, warps = 0, wfb = 0, wsec = 0;
  for (long w = 0; w < n; w += 32) {
    bool any_fb = false, any_sec = false;
    for (long k = w; k < n && k < w + 32; ++k) {
      const double* x = &r[6 * k];
      const double den[4] = {x[2], x[3], x[4], x[5]};
      const e2d::SlopePick p = e2d::pick_slopes<0>(x[0], x[1], den);
      if (!p.ok) { ++fb; any_fb = true; }
      else if (p.second) { ++sec; any_sec = true; }
    }
    ++warps;
    wfb += any_fb;
    wsec += any_sec;
  }
  std::printf("lanes=%ld fallback=%ld second=%ld warps=%ld warp_fallback=%ld warp_second=%ld\n", n, fb, sec, warps,
              wfb, wsec);
  return 0;
}
