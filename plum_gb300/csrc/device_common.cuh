// Device helpers shared by the kernel translation units. They are inlined
// where they are used: a DevParams kernel argument passed by reference into a
// separately compiled function would be copied to local memory per thread.
#pragma once

#include "engine.h"

namespace plum {

// Wall energy of one bead at height z (potential_truncated_lj_wall.cc:46-134).
__device__ __forceinline__ double wall64(const DevParams& P, double z, int ty) {
  if (P.ext_kind == 1) {  // PotentialHardWall::BeadEnergy (potential_hard_wall.cc:36-47)
    const double rad = P.wall_rad[ty];
    return (z <= rad || z + rad >= P.box[2]) ? kVeryLarge : 0.0;
  }
  if (P.ext_kind == 2) {  // PotentialWellWall::BeadEnergy (potential_well_wall.cc:41-55)
    const double rad = P.wall_rad[ty];
    if (z <= rad || z >= P.box[2] - rad) return kVeryLarge;
    if (z < P.well_width || z > P.box[2] - P.well_width) return P.well_depth;
    return 0.0;
  }
  double energy = 0.0;
  const double sigma = P.wall_sig[ty], eps = P.wall_eps[ty];
  const double R0 = 3 * 1.25992104989 * sigma, K = 1.0;
  const double lz = P.box[2];
  const double k213 = 1.25992104989, c93 = 2.59807621135;
  const int g = P.graft[ty];
  if (eps == 0.0) return 0.0;
  if (z <= 0.0 || z >= lz) return kVeryLarge;
  if (P.wall_cut < 0 && g == 0) {
    double r3r = pow(1.0 / k213, 3.0);
    double eref = c93 * eps * (r3r * r3r - r3r);
    if (z < k213 * sigma) {
      double r3 = pow(sigma / z, 3.0);
      energy += c93 * eps * (r3 * r3 - r3) - eref;
    }
    if (lz - z < k213 * sigma) {
      double r3 = pow(sigma / (lz - z), 3.0);
      energy += c93 * eps * (r3 * r3 - r3) - eref;
    }
  } else if (g == 1) {
    double r3 = pow(sigma / z, 3.0);
    energy += c93 * eps * (r3 * r3 - r3);
    energy += -0.5 * K * R0 * R0 * log(1 - pow(z / R0, 2.0));
    if (lz - z < k213 * sigma) {
      r3 = pow(sigma / (lz - z), 3.0);
      energy += c93 * eps * (r3 * r3 - r3);
    } else {
      r3 = pow(1.0 / k213, 3.0);
      energy += c93 * eps * (r3 * r3 - r3);
    }
  } else if (g == 2) {
    double r3 = pow(sigma / (lz - z), 3.0);
    energy += c93 * eps * (r3 * r3 - r3);
    energy += -0.5 * K * R0 * R0 * log(1 - pow((lz - z) / R0, 2.0));
    if (z < k213 * sigma) {
      r3 = pow(sigma / z, 3.0);
      energy += c93 * eps * (r3 * r3 - r3);
    } else {
      r3 = pow(1.0 / k213, 3.0);
      energy += c93 * eps * (r3 * r3 - r3);
    }
  } else {
    double r3r = pow(1.0 / P.wall_cut, 3.0);
    double eref = c93 * eps * (r3r * r3r - r3r);
    if (z < P.wall_cut) {
      double r3 = pow(sigma / z, 3.0);
      energy += c93 * eps * (r3 * r3 - r3) - eref;
    }
    if (lz - z < P.wall_cut) {
      double r3 = pow(sigma / (lz - z), 3.0);
      energy += c93 * eps * (r3 * r3 - r3) - eref;
    }
  }
  return energy;
}

__device__ __forceinline__ int fix_axis(double x, double L, double inv_fix, bool periodic) {
  double w = periodic ? x - L * floor(x / L) : x;
  long long v = llrint(w * inv_fix);
  return (int)(unsigned int)(unsigned long long)v;
}

// 64-bit fixed-point fraction of the box: frac(x / L) 2^64.
__device__ __forceinline__ unsigned long long fix64(double x, double inv) {
  double f = x * inv;
  f -= floor(f);
  if (f >= 1.0) f = 0.0;  // a tiny negative x / L rounds up to 1
  return __double2ull_rn(f * 0x1p64);
}

// A bead as the plain form's 64-bit mirror holds it (cubic box).
__device__ __forceinline__ ulonglong4_32a fix64x4(const DevParams& P, double4_32a p) {
  const double inv = P.inv_ebox[0];
  return make_ulonglong4_32a(fix64(p.x, inv), fix64(p.y, inv), fix64(p.z, inv),
                         (unsigned long long)__double_as_longlong(p.w));
}

__device__ __forceinline__ int4 fix_point(const DevParams& P, double4_32a p, int type) {
  return make_int4(fix_axis(p.x, P.ebox[0], P.inv_fix[0], true),
                   fix_axis(p.y, P.ebox[1], P.inv_fix[1], true),
                   fix_axis(p.z, P.ebox[2], P.inv_fix[2], P.npbc > 2), type);
}

// Hard spheres leave out the pair energy of a chain's bonded neighbours
// (potential_pair.cc:64-67, 163-167): beads i and j = i +- 1 of the same
// molecule (the higher index does not start a molecule; mol_start holds
// n_mol + 1 ascending entries).
__device__ __forceinline__ bool hs_bonded(const DevParams& P, const int* mol_start, int i,
                                          int j) {
  if (P.pair_kind != 1 || (j - i != 1 && i - j != 1)) return false;
  const int hi = i > j ? i : j;
  int lo = 0, up = P.n_mol;
  while (lo < up) {
    const int mid = (lo + up) >> 1;
    if (mol_start[mid] < hi) lo = mid + 1; else up = mid;
  }
  return mol_start[lo] != hi;
}

// Cell of a bead of the descriptor's cell list from its fixed-point
// coordinates (fractions of the Ewald box in [0, 2^32)).
__device__ __forceinline__ int cell_axis(unsigned x, int nc) {
  return (int)(((unsigned long long)x * (unsigned)nc) >> 32);
}
__device__ __forceinline__ int cell_index(const DevParams& P, int4 f) {
  return cell_axis((unsigned)f.x, P.cell_nc[0]) +
         P.cell_nc[0] * (cell_axis((unsigned)f.y, P.cell_nc[1]) +
                         P.cell_nc[1] * cell_axis((unsigned)f.z, P.cell_nc[2]));
}

// ------------------------------------------------------- FP64 real space
static_assert(kH64Per == 32, "bin index below assumes 5 mantissa bits per octave");
constexpr long long kH64LoBits = (long long)(1023 + kH64ELo) << 52;

// h(u) = erfc(sqrt u) / sqrt u from the FP64 table at the bits of u >= 2^kH64ELo:
// the exponent and top five mantissa bits pick the bin, the remaining 47 bits
// shifted into a double of [1, 2) give 1 + f exactly, y = f - 1/2.
__device__ __forceinline__ double h64_tab(const double* __restrict__ tab, long long bits) {
  int idx = (int)(bits >> 47) - ((1023 + kH64ELo) << 5);
  idx = min(max(idx, 0), kH64Bins - 1);
  const double2* c = reinterpret_cast<const double2*>(tab + (size_t)idx * kH64Stride);
  const double2 c01 = __ldg(c), c23 = __ldg(c + 1), c45 = __ldg(c + 2), c67 = __ldg(c + 3),
                c89 = __ldg(c + 4);
  const double y = __longlong_as_double(((bits << 5) & 0xFFFFFFFFFFFFFLL) |
                                        0x3FF0000000000000LL) - 1.5;
  double h = fma(c89.x, y, c67.y);
  h = fma(h, y, c67.x);
  h = fma(h, y, c45.y);
  h = fma(h, y, c45.x);
  h = fma(h, y, c23.y);
  h = fma(h, y, c23.x);
  h = fma(h, y, c01.y);
  return fma(h, y, c01.x);
}

// erfc(sqrt(alpha) r) / r at squared distance r2 > 0 (the caller excludes
// r2 = 0, as the reference's r > 0 test does): sqrt(alpha) h(alpha r2) from
// the table, or directly where there is none or u is below it.
__device__ __forceinline__ double real_term64(const DevParams& P, double r2) {
  if (P.htab64) {
    const long long bits = __double_as_longlong(P.alpha * r2);
    if (bits >= kH64LoBits) return P.sqrt_alpha * h64_tab(P.htab64, bits);
  }
  const double r = sqrt(r2);
  return erfc(P.sqrt_alpha * r) / r;
}

}  // namespace plum
