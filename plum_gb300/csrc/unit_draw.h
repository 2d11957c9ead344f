// x / (2^32 - 1) in double precision, correctly rounded (the same bits as
// the IEEE division (double)x / 4294967295.0 the draws of std::mt19937 words
// go through), without a division: for 0 < x < 2^32 - 1 the binary expansion
// of x / (2^32 - 1) is x's 32 bits repeated, 0.[x][x][x]..., so the 64 bits
// from its leading one are known exactly, the rest is non-zero, and rounding
// them to 53 bits with that rest as a sticky bit is one conversion. Checked
// against the division for every 32-bit x (tests/test_unit_draw.py).
// Compiles as CUDA device code and as C (the check).
#pragma once
#include <stdint.h>

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
