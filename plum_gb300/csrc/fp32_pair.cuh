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
    if (r2 > 0.0f) {
      const float ir = rsqrtf(r2);
      const float r = r2 * ir;
      if (r <= rc) e = erfc_nr(P.f_sqrt_alpha * r) * ir;
    }
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
        if (r2 > 0.0f) {
          float ir = rsqrtf(r2);
          float r = r2 * ir;
          if (r <= rc) e += erfc_nr(P.f_sqrt_alpha * r) * ir;
        }
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
