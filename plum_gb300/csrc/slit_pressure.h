// The wall-force pressure of slit systems, ForceField::CalcPressureForceLJELSlit
// (pressure.cc:404-488): the z force between the wall sites (the first
// `phantom` molecules, half on the wall at z = 0, half on the wall at
// z = box_l[2]; each site is its molecule's first bead) and the system, plus
// the external potential's force on every system bead.
//
// The per-item arithmetic lives here as plain FP64 C++ that compiles both for
// the device (kern_pressure.cu launches it) and for the host, so that the same
// code can be run over a configuration on a CPU and compared item by item.
//
// Work items:
//   pair item (site i, bead b): every bead b >= mol_start[phantom / 2], i.e.
//     the beads of the second wall's molecules and of the system, against
//     site i; site i of the second wall only meets system beads
//     (pressure.cc:419-455). LJ force (PairForce) and real-space Ewald z
//     force (PairForceZReal) go to accumulators 0-2 and 3-5: ion, polymer,
//     wall-wall (the molecule of b has one bead, more than one, or is a wall
//     molecule).
//   wall item (system bead b): half the external potential's force on the
//     wall (BeadForceOnWall) into accumulator 0 or 1 (pressure.cc:458-469).
//   k item (reciprocal vector k): the reference sums PairForceZRepl over
//     every (site, bead) pair, k_z e^{-k^2/4a}/k^2 sin(k.(r_site - r_bead))
//     over the k-set. Summed over a group of sites A and beads B that is
//     Im(S_A(k) conj(S_B(k))) with S_G(k) = sum_{g in G} q_g e^{i k.r_g}, so
//     each k needs the five group sums (first-wall sites, second-wall sites,
//     beads of second-wall molecules, ion beads, polymer beads) instead of
//     the site x bead double loop.
#pragma once

#include <math.h>

#if defined(__CUDACC__)
#define PLUM_HD __host__ __device__ __forceinline__
#else
#define PLUM_HD inline
#endif

namespace plum {

constexpr int kSlitMaxTypes = 8;
constexpr double kSlitPi = 3.14159265359;    // utilities/constants.h:20
constexpr double kSlit213 = 1.25992104989;   // 2^(1/3), utilities/constants.h
constexpr double kSlit216 = 1.12246204831;   // 2^(1/6), utilities/constants.h:62
constexpr double kSlitVeryLarge = 1e8;       // utilities/constants.h:15
constexpr double kSlitK93 = 2.59807621135;   // potential_truncated_lj_wall.cc (9-3 force)

struct SlitPressParams {
  int n_bead, n_mol, phantom, npbc, n_type;
  int use_pair, use_ewald, use_ext;
  int pair_kind;  // 0 truncated LJ, 1 hard spheres (no force)
  int ext_kind;   // 0 9-3 LJ wall, 1 hard wall, 2 square-well wall (no force)
  double box[3], ebox[3];
  // truncated LJ per type (sigma, epsilon), mixed per pair as the reference
  // does (potential_truncated_lj.cc:55-58); lj_cut < 0: WCA
  double lj_cut, lj_sig[kSlitMaxTypes], lj_eps[kSlitMaxTypes];
  // Ewald: Bjerrum length, alpha, real-space cut-off and image cells, the
  // Ewald box volume
  double lB, alpha, real_cut, evol;
  int real_cell[3];
  // 9-3 wall per type; graft 1 for "L" (grafted at z = 0), 2 for "R"
  double wall_cut, wall_sig[kSlitMaxTypes], wall_eps[kSlitMaxTypes];
  int graft[kSlitMaxTypes];
};

// Molecule of bead b: the largest m with mol_start[m] <= b.
PLUM_HD int slit_mol_of(const int* mol_start, int n_mol, int b) {
  int lo = 0, hi = n_mol - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (mol_start[mid] <= b)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

// Nearest-image component on a periodic axis (GetDistVector, misc.cc:43-56).
PLUM_HD double slit_wrap(double d, double L) { return d - L * round(d / L); }

// PotentialTruncatedLJ::PairForce (potential_truncated_lj.cc:87-122) at
// distance r between types ta and tb. Beyond a positive cut-off it is the
// cut-off's r^-6 term evaluated at r, as the reference writes it. The
// reference's own function tests an uninitialised local against -1 first
// (potential_truncated_lj.cc:95-100); this follows the evident intent, the
// overlap value only for r <= 0. Hard spheres exert none
// (potential_hard_sphere.cc:51-56).
PLUM_HD double slit_lj_force(const SlitPressParams& S, int ta, int tb, double r) {
  if (S.pair_kind == 1) return 0.0;
  const double sigma = (S.lj_sig[ta] + S.lj_sig[tb]) / 2;
  const double eps = sqrt(S.lj_eps[ta] * S.lj_eps[tb]);
  if (r <= 0) return kSlitVeryLarge;
  double x;
  if (S.lj_cut < 0) {
    if (!(r < kSlit216 * sigma)) return 0.0;
    x = sigma / r;
  } else {
    x = sigma / (r < S.lj_cut ? r : S.lj_cut);
  }
  const double x2 = x * x;
  const double r6 = x2 * x2 * x2;
  return 4 * eps * (r6 * r6 * 12 / r - r6 * 6 / r);
}

// PotentialEwaldCoul::PairForceZReal (potential_ewald_coul.cc:261-293): z
// force on a wall charge from a bead at (rx, ry, rz) = r_site - r_bead
// (nearest image on the periodic axes of the Ewald box), summed over the
// image cells within the real-space cut-off. qq = q_site q_bead.
PLUM_HD double slit_ew_real_z(const SlitPressParams& S, double rx, double ry, double rz,
                              double qq) {
  if (qq == 0) return 0.0;
  const double pre = S.lB * qq;
  const double pre2 = 2 * sqrt(S.alpha / kSlitPi);
  const double sa = sqrt(S.alpha), rc = S.real_cut;
  double f = 0.0;
  for (int a = -S.real_cell[0]; a <= S.real_cell[0]; a++) {
    const double x = rx + a * S.ebox[0];
    if (fabs(x) > rc) continue;  // no image of this shift is inside the cut-off
    for (int b = -S.real_cell[1]; b <= S.real_cell[1]; b++) {
      const double y = ry + b * S.ebox[1];
      if (fabs(y) > rc) continue;
      for (int c = -S.real_cell[2]; c <= S.real_cell[2]; c++) {
        const double z = rz + c * S.ebox[2];
        if (fabs(z) > rc) continue;
        const double d = sqrt(x * x + y * y + z * z);
        if (d > 0 && d <= rc)
          f += pre * ((pre2 * exp(-S.alpha * d * d)) + (erfc(sa * d) / d)) * z / (d * d);
      }
    }
  }
  return f;
}

// One 9-3 wall term of the force: k93 eps ((s/h)^6 6/h - (s/h)^3 3/h) with
// the distance h_c inside the powers.
PLUM_HD double slit_w93(double sigma, double eps, double hc, double h) {
  const double x = sigma / hc;
  const double r3 = x * x * x;
  return kSlitK93 * eps * (r3 * r3 * 6 / h - r3 * 3 / h);
}

// PotentialTruncatedLJWall::BeadForceOnWall (potential_truncated_lj_wall.cc:
// 136-214) for a bead of type ty at height z; the hard and square-well walls
// exert none (the base class's zero).
PLUM_HD double slit_wall_force(const SlitPressParams& S, double z, int ty) {
  if (S.ext_kind != 0) return 0.0;
  const double sigma = S.wall_sig[ty], eps = S.wall_eps[ty];
  if (eps == 0) return 0.0;
  const double lz = S.box[2], mc = S.wall_cut;
  const double R0 = 3 * kSlit213 * sigma, K = 1;
  const int g = S.graft[ty];
  if (z <= 0 || z >= lz) return kSlitVeryLarge;
  double f = 0.0;
  const double u = lz - z;
  if (mc < 0 && g == 0) {
    if (z < kSlit213 * sigma) f += slit_w93(sigma, eps, z, z);
    if (u < kSlit213 * sigma) f += slit_w93(sigma, eps, u, u);
  } else if (g == 1) {
    f += slit_w93(sigma, eps, z, z);
    f += -K * R0 * z / (1 - (z / R0) * (z / R0));
    if (u < kSlit213 * sigma) f += slit_w93(sigma, eps, u, u);
  } else if (g == 2) {
    f += slit_w93(sigma, eps, u, u);
    f += -K * R0 * u / (1 - (u / R0) * (u / R0));
    if (z < kSlit213 * sigma) f += slit_w93(sigma, eps, z, z);
  } else {
    f += slit_w93(sigma, eps, z < mc ? z : mc, z);
    if (u < mc)
      f += slit_w93(sigma, eps, u, u);
    else
      f += slit_w93(sigma, eps, mc, z);
  }
  return f;
}

// acc[base + kid] += v with constant indices only, so that a caller's
// accumulator array can stay in registers.
PLUM_HD void slit_add(double* acc, int base, int kid, double v) {
  if (kid == 0)
    acc[base] += v;
  else if (kid == 1)
    acc[base + 1] += v;
  else
    acc[base + 2] += v;
}

// First bead of the pair items and their count: sites x beads from the
// second wall's first bead on.
PLUM_HD long long slit_pair_items(const SlitPressParams& S, const int* mol_start) {
  if (S.phantom <= 0 || (!S.use_pair && !S.use_ewald)) return 0;
  return (long long)S.phantom * (S.n_bead - mol_start[S.phantom / 2]);
}

// Wall items: the beads of the system molecules (after the wall sites).
PLUM_HD long long slit_wall_items(const SlitPressParams& S, const int* mol_start) {
  if (!S.use_ext) return 0;
  return S.n_bead - mol_start[S.phantom];
}

// Pair item `item` (site i = item / nb, bead b0 + item % nb): adds its LJ and
// real-space z forces, weighted as pressure.cc:421-428 weights them, into
// acc[0..2] (LJ: ion, polymer, wall-wall) and acc[3..5] (Ewald real space).
// xyzq holds x, y, z, q per bead.
PLUM_HD void slit_pair_item(const SlitPressParams& S, const double* xyzq, const int* type,
                            const int* mol_start, long long item, double* acc) {
  const int ph = S.phantom;
  const int b0 = mol_start[ph / 2];
  const long long nb = S.n_bead - b0;
  const int i = (int)(item / nb);
  const int b = b0 + (int)(item - (long long)i * nb);
  const int j = slit_mol_of(mol_start, S.n_mol, b);
  if (i >= ph / 2 && j < ph) return;  // second wall with its own sites
  const double C = j >= ph ? (i < ph / 2 ? -0.5 : 0.5) : -1.0;
  const int kid = j >= ph ? (mol_start[j + 1] - mol_start[j] > 1 ? 1 : 0) : 2;
  const int w = mol_start[i];
  const double* pw = xyzq + 4 * (long long)w;
  const double* pb = xyzq + 4 * (long long)b;
  if (S.use_pair) {
    double r[3];
    for (int a = 0; a < 3; a++) {
      const double d = pw[a] - pb[a];
      r[a] = a < S.npbc ? slit_wrap(d, S.box[a]) : d;
    }
    const double rr = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
    slit_add(acc, 0, kid, C * (r[2] / rr) * slit_lj_force(S, type[b], type[w], rr));
  }
  if (S.use_ewald) {
    double r[3];
    for (int a = 0; a < 3; a++) {
      const double d = pw[a] - pb[a];
      r[a] = a < S.npbc ? slit_wrap(d, S.ebox[a]) : d;
    }
    slit_add(acc, 3, kid, C * slit_ew_real_z(S, r[0], r[1], r[2], pw[3] * pb[3]));
  }
}

// Wall item for system bead b: half its external force on the wall into
// acc[0] (ions) or acc[1] (polymer beads).
PLUM_HD void slit_wall_item(const SlitPressParams& S, const double* xyzq, const int* type,
                            const int* mol_start, int b, double* acc) {
  const int j = slit_mol_of(mol_start, S.n_mol, b);
  const int jid = mol_start[j + 1] - mol_start[j] > 1 ? 1 : 0;
  slit_add(acc, 0, jid, 0.5 * slit_wall_force(S, xyzq[4 * (long long)b + 2], type[b]));
}

// Group membership of bead b for the k items, a bit per group:
// 1 first-wall site, 2 second-wall site, 4 bead of a second-wall molecule,
// 8 ion bead, 16 polymer bead (system molecules of one / several beads).
PLUM_HD int slit_bead_groups(const SlitPressParams& S, const int* mol_start, int b) {
  const int ph = S.phantom;
  const int j = slit_mol_of(mol_start, S.n_mol, b);
  if (j >= ph) return mol_start[j + 1] - mol_start[j] > 1 ? 16 : 8;
  int g = 0;
  if (b == mol_start[j]) g |= j < ph / 2 ? 1 : 2;
  if (j >= ph / 2) g |= 4;
  return g;
}

// Reciprocal z forces of one k vector from its five group sums (re, im of
// S_G(k), G in the bit order above): out[0..2] += ion, polymer, wall-wall
// parts, each to be multiplied by lB 4 kPi / V * 2 (the half-space sum counts
// k and -k). kz: z component of k; w: e^{-k^2/4a}/k^2.
PLUM_HD void slit_k_terms(double kz, double w, const double* re, const double* im,
                          double* out) {
  // Im(S_a conj S_b) = sum_{a, b} q_a q_b sin(k.(r_a - r_b))
  const double w0_ion = im[0] * re[3] - re[0] * im[3];
  const double w1_ion = im[1] * re[3] - re[1] * im[3];
  const double w0_pol = im[0] * re[4] - re[0] * im[4];
  const double w1_pol = im[1] * re[4] - re[1] * im[4];
  const double w0_w2 = im[0] * re[2] - re[0] * im[2];
  const double kw = kz * w;
  out[0] += kw * (-0.5 * w0_ion + 0.5 * w1_ion);
  out[1] += kw * (-0.5 * w0_pol + 0.5 * w1_pol);
  out[2] += kw * (-1.0 * w0_w2);
}

PLUM_HD double slit_recip_prefactor(const SlitPressParams& S) {
  return S.lB * 4 * kSlitPi / S.evol * 2;
}

}  // namespace plum
