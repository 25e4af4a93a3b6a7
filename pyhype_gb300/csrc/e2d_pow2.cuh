// e2d_pow2.cuh - x * 0.5 and x * 2 for doubles without the FP64 pipe.
//
// The scheme scales by 1/2 and 2 in many places (interface averages, kinetic energy,
// the Roe flux's 0.5 (F_L + F_R) - 0.5 |A| dW, the one-point rule's 2 F, the
// divergence's 0.5 sum).  On GB300 the FP64 pipe is the binding resource (one FP64
// instruction costs as much issue time on it as dozens of integer instructions), and
// a power-of-two scaling is an exponent change: these functions return the IEEE
// result of x * 0.5 and x * 2 (round to nearest even, signed zeros, subnormals,
// overflow to infinity, infinities; NaN stays NaN) computed on the integer pipe.
// They are host-callable so a CPU test can compare them with the multiplication.
#pragma once
#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define E2D_POW2_HD __host__ __device__ __forceinline__
#else
#define E2D_POW2_HD inline
#endif

namespace e2d {

// bits of x * 0.5
E2D_POW2_HD uint64_t half_bits(uint64_t b) {
  const uint32_t e = (uint32_t)(b >> 52) & 0x7ffu;
  if (e - 2u < 2045u) return b - (1ULL << 52);  // normal result: exponent - 1
  if (e == 0x7ffu) return b;                    // infinity or NaN
  // zero, subnormal or smallest-exponent input: the result is subnormal; halve the
  // significand (with its leading 1 when e == 1), ties to even
  uint64_t m = b & 0x000fffffffffffffULL;
  if (e == 1u) m |= 1ULL << 52;
  const uint64_t r = (m >> 1) + (m & (m >> 1) & 1ULL);
  return (b & 0x8000000000000000ULL) | r;
}

// bits of x * 2
E2D_POW2_HD uint64_t twice_bits(uint64_t b) {
  const uint32_t e = (uint32_t)(b >> 52) & 0x7ffu;
  if (e - 1u < 2045u) return b + (1ULL << 52);                           // normal result
  if (e == 2046u) return (b & 0x8000000000000000ULL) | 0x7ff0000000000000ULL;  // overflow
  if (e == 0x7ffu) return b;                                              // infinity or NaN
  return (b & 0x8000000000000000ULL) | ((b & 0x000fffffffffffffULL) << 1);  // zero or subnormal
}

template <typename T>
E2D_POW2_HD T half(T x) { return T(0.5) * x; }
template <typename T>
E2D_POW2_HD T twice(T x) { return T(2) * x; }

template <>
E2D_POW2_HD double half<double>(double x) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)half_bits((uint64_t)__double_as_longlong(x)));
#else
  uint64_t b;
  std::memcpy(&b, &x, sizeof b);
  b = half_bits(b);
  std::memcpy(&x, &b, sizeof b);
  return x;
#endif
}
template <>
E2D_POW2_HD double twice<double>(double x) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)twice_bits((uint64_t)__double_as_longlong(x)));
#else
  uint64_t b;
  std::memcpy(&b, &x, sizeof b);
  b = twice_bits(b);
  std::memcpy(&x, &b, sizeof b);
  return x;
#endif
}

}  // namespace e2d
