// x / (2^32 - 1) in double precision, correctly rounded (the same bits as
// the IEEE division (double)x / 4294967295.0 the draws of std::mt19937 words
// go through), without a division: for 0 < x < 2^32 - 1 the binary expansion
// of x / (2^32 - 1) is x's 32 bits repeated, 0.[x][x][x]..., so the 64 bits
// from its leading one are known exactly, the rest is non-zero, and rounding
// them to 53 bits with that rest as a sticky bit is one conversion. Checked
// against the division for every 32-bit x (tests/test_unit_draw.py).
// Compiles as CUDA device code and as C (the check). Also the Metropolis
// test of those draws.
#pragma once
#include <stdint.h>
#ifndef __CUDACC__
#include <math.h>
#include <stdbool.h>
#endif

#ifdef __CUDACC__
__device__ __forceinline__ double unit_draw(uint32_t x) {
  if (x == 0u) return 0.0;
  if (x == 0xFFFFFFFFu) return 1.0;
  const int lz = __clz((int)x);
  const unsigned long long two = ((unsigned long long)x << 32) | x;  // [x][x]
  const unsigned long long w = lz ? (two << lz) | (x >> (32 - lz)) : two;
  const double d = __ull2double_rn(w | 1ull);  // rounds with the rest as sticky
  return __longlong_as_double(__double_as_longlong(d) - ((long long)(64 + lz) << 52));
}
#else
#include <string.h>
static inline double unit_draw(uint32_t x) {
  if (x == 0u) return 0.0;
  if (x == 0xFFFFFFFFu) return 1.0;
  const int lz = __builtin_clz(x);
  const uint64_t two = ((uint64_t)x << 32) | x;
  const uint64_t w = lz ? (two << lz) | (x >> (32 - lz)) : two;
  double d = (double)(w | 1u);
  int64_t b;
  memcpy(&b, &d, sizeof b);
  b -= (int64_t)(64 + lz) << 52;
  memcpy(&d, &b, sizeof d);
  return d;
}
#endif

#ifdef __CUDACC__
#define PLUM_DRAW_FN __device__ __forceinline__
#else
#define PLUM_DRAW_FN static inline
#endif

// Metropolis' u < exp(-x) (simulation.cc:324-332), the same decision without
// the exponential where it is certain: x <= 0 gives exp(-x) >= 1 > u for
// u < 1; above x = 23, exp(-x) < 1.03e-10 is below every non-zero draw
// (the least is 1 / (2^32 - 1) = 2.33e-10), so only u = 0 needs it. A NaN x
// fails both tests and compares false with the exponential, as before.
PLUM_DRAW_FN bool metropolis(double u, double x) {
  if (x <= 0.0 && u < 1.0) return true;
  if (x > 23.0) return u == 0.0 && 0.0 < exp(-x);
  return u < exp(-x);
}
