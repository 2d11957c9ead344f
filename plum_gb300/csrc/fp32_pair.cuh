// FP32 pair functions of the precision form, shared by the move kernels
// (kern_fp32.cu) and the configurational-bias trial kernel (kern_cbmc32.cu).
// Positions are 32-bit fixed-point fractions of the Ewald box (fix_point):
// a minimum-image difference is one integer subtraction.
#pragma once

#include "device_common.cuh"
#include "engine.h"

namespace plum {

__device__ __forceinline__ float fdiff(int a, int b, float scale) {
  return (float)(int)((unsigned)b - (unsigned)a) * scale;
}

// erfc for x >= 0 by the Chebyshev fit of Press et al., Numerical Recipes
// (2nd ed., section 6.2, "erfcc"): erfc(x) = t exp(-x^2 + P9(t)),
// t = 1 / (1 + x/2), fractional error below 1.2e-7 for every x >= 0 -- at the
// level of FP32 rounding, for about a third of erfcf's instructions.
__device__ __forceinline__ float erfc_nr(float x) {
  const float t = __fdividef(1.0f, fmaf(0.5f, x, 1.0f));
  float p = 0.17087277f;
  p = fmaf(p, t, -0.82215223f);
  p = fmaf(p, t, 1.48851587f);
  p = fmaf(p, t, -1.13520398f);
  p = fmaf(p, t, 0.27886807f);
  p = fmaf(p, t, -0.18628806f);
  p = fmaf(p, t, 0.09678418f);
  p = fmaf(p, t, 0.37409196f);
  p = fmaf(p, t, 1.00002368f);
  p = fmaf(p, t, -1.26551223f);
  return t * __expf(fmaf(-x, x, p));
}

static_assert(kH32Per == 32, "bin index below assumes 5 mantissa bits per octave");
constexpr int kH32LoBits = (127 + kH32ELo) << 23;  // float bits of 2^kH32ELo

// h(u) = erfc(sqrt u) / sqrt u from the table (in shared memory) at the
// float bits of u: the exponent and top five mantissa bits pick the bin, the
// remaining 18 bits are the bin-local fraction f; placed under the exponent
// of 1 they make the float 1 + f/32 exactly, and w = f/32 is exact too. The
// bin's cubic is in w. Bins outside the table are clamped to the last one
// (one unsigned minimum; a u below the table wraps to a huge index): the
// caller replaces values below the table, and values above it are cut off.
__device__ __forceinline__ float h32_tab(const float4* tab, int bits) {
  const unsigned idx = min((unsigned)((bits >> 18) - ((127 + kH32ELo) << 5)),
                           (unsigned)(kH32Bins - 1));
  const float4 c = tab[idx];
  const float w = __int_as_float((bits & 0x3FFFF) | 0x3F800000) - 1.0f;
  return fmaf(fmaf(fmaf(c.w, w, c.z), w, c.y), w, c.x);
}

// Below the table (u < 2^kH32ELo: r under 1/128 of 1/sqrt(alpha)): the erfc
// fit; 0 at r = 0 (the reference's r > 0 test).
static __device__ __noinline__ float h32_small(float u) {
  return u > 0.0f ? erfc_nr(sqrtf(u)) * rsqrtf(u) : 0.0f;
}

// h(u) for any u >= 0 from a table in shared or global memory.
__device__ __forceinline__ float h32(const float4* tab, float u) {
  const int bits = __float_as_int(u);
  float h = h32_tab(tab, bits);
  if (bits < kH32LoBits) h = h32_small(u);
  return h;
}

// erfc(sqrt(alpha) r) / r at squared distance r2 > 0 (0 at r2 = 0): from the
// context's h(u) table when it has one (alpha r_c^2 inside the table), else
// the erfc fit.
__device__ __forceinline__ float real_term32(const DevParams& P, float r2) {
  if (P.htab) return P.f_sqrt_alpha * h32(P.htab, P.f_sqrt_alpha * P.f_sqrt_alpha * r2);
  if (!(r2 > 0.0f)) return 0.0f;
  const float ir = rsqrtf(r2);
  return erfc_nr(P.f_sqrt_alpha * r2 * ir) * ir;
}

__device__ __forceinline__ float lj32(const DevParams& P, int k, float r2) {
  if (P.pair_kind == 1) return sqrtf(r2) <= P.f_hs_sum[k] ? (float)kVeryLarge : 0.0f;
  if (r2 <= 0.0f) return (float)kVeryLarge;
  if (r2 < P.f_lj_rc2[k]) {
    float s2 = __fdividef(P.f_lj_sig2[k], r2);
    float s6 = s2 * s2 * s2;
    return P.f_lj_eps4[k] * (s6 * s6 - s6) - P.f_lj_eref[k];
  }
  return 0.0f;
}

__device__ __forceinline__ float real_images32(const DevParams& P, float dx, float dy,
                                               float dz) {
  float e = 0.0f;
  const float rc = P.f_real_cut;
  if (P.single_image) {
    // r_c <= L/2 on every axis: only the minimum image can be inside r_c
    const float r2 = dx * dx + dy * dy + dz * dz;
    if (r2 <= rc * rc) e = real_term32(P, r2);
    return e;
  }
  for (int a = -P.real_cell[0]; a <= P.real_cell[0]; a++) {
    float x = dx + a * P.f_box[0];
    if (fabsf(x) > rc) continue;
    for (int b = -P.real_cell[1]; b <= P.real_cell[1]; b++) {
      float y = dy + b * P.f_box[1];
      if (fabsf(y) > rc) continue;
      for (int c = -P.real_cell[2]; c <= P.real_cell[2]; c++) {
        float z = dz + c * P.f_box[2];
        if (fabsf(z) > rc) continue;
        float r2 = x * x + y * y + z * z;
        if (r2 <= rc * rc) e += real_term32(P, r2);
      }
    }
  }
  return e;
}

__device__ __forceinline__ void pair32(const DevParams& P, int4 a, float qa, int4 b,
                                       float qb, float& lj, float& re) {
  const float dx = fdiff(a.x, b.x, P.f_scale[0]);
  const float dy = fdiff(a.y, b.y, P.f_scale[1]);
  const float dz = fdiff(a.z, b.z, P.f_scale[2]);
  if (P.use_pair) lj += lj32(P, a.w * P.n_type + b.w, dx * dx + dy * dy + dz * dz);
  if (P.use_ewald) {
    const float qq = qa * qb;
    if (qq != 0.0f) re += P.f_lB * qq * real_images32(P, dx, dy, dz);
  }
}

}  // namespace plum
