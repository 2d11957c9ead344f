#include "ewald_setup.h"

#include <cmath>

namespace plum {

namespace {
constexpr double kEwaldCut = 1e-7;        // utilities/constants.h:11
constexpr double kPi = 3.14159265359;     // utilities/constants.h:20
constexpr double kDiCorrection = 3;       // utilities/constants.h (dipole padding factor)
}  // namespace

bool ewald_setup(const Input& in, int max_kcell, EwaldSetup* out, std::string* err) {
  EwaldSetup& E = *out;
  for (int a = 0; a < 3; a++) E.ebox[a] = in.box[a];
  if (in.dipole) {
    const double min_padding = 150;
    if (E.ebox[2] * kDiCorrection > min_padding)
      E.ebox[2] = E.ebox[2] * kDiCorrection;
    else
      E.ebox[2] += min_padding;
  }
  E.vol = E.ebox[0] * E.ebox[1] * E.ebox[2];
  double rc = 1;
  while (0.5 * in.lB * 1 * 1 * std::erfc(std::sqrt(in.alpha) * rc) / rc > kEwaldCut) rc += 1;
  if (in.x_real_cutoff > 0) rc = in.x_real_cutoff;
  double kc2 = in.alpha;
  const double min_box_vol = std::pow(E.ebox[0], 3);
  while (in.lB * 1 * 1 / (2 * kPi * min_box_vol) * (4 * kPi * kPi) *
             std::exp(-kc2 / (4 * in.alpha)) / kc2 >
         kEwaldCut)
    kc2 += in.alpha;
  for (int a = 0; a < 3; a++) E.kcell[a] = (int)std::ceil(std::sqrt(kc2) * E.ebox[a] / (2 * kPi));
  if (in.x_kmax > 0) {
    for (int a = 0; a < 3; a++) E.kcell[a] = in.x_kmax;
    if (!in.x_have_kcut2) kc2 = INFINITY;
  }
  if (in.x_have_kcut2) kc2 = in.x_kcut2 > 0 ? in.x_kcut2 : INFINITY;
  for (int a = 0; a < 3; a++)
    if (E.kcell[a] > max_kcell) {
      *err = "k-space range |n| = " + std::to_string(E.kcell[a]) + " exceeds the supported " +
             std::to_string(max_kcell);
      return false;
    }
  for (int a = 0; a < 3; a++) E.real_cell[a] = (int)std::ceil(rc / E.ebox[a]);
  E.real_cut = rc;
  E.kc2 = kc2;
  E.kn.clear();
  E.kw.clear();
  for (int lx = -E.kcell[0]; lx <= E.kcell[0]; lx++)
    for (int ly = -E.kcell[1]; ly <= E.kcell[1]; ly++)
      for (int lz = -E.kcell[2]; lz <= E.kcell[2]; lz++) {
        const bool half = lx > 0 || (lx == 0 && ly > 0) || (lx == 0 && ly == 0 && lz > 0);
        if (!half) continue;
        const double kx = lx * 2 * kPi / E.ebox[0];
        const double ky = ly * 2 * kPi / E.ebox[1];
        const double kz = lz * 2 * kPi / E.ebox[2];
        const double k2 = kx * kx + ky * ky + kz * kz;
        if (!(k2 > 0 && k2 <= kc2)) continue;
        E.kn.push_back(lx);
        E.kn.push_back(ly);
        E.kn.push_back(lz);
        E.kw.push_back(std::exp(-k2 / (4 * in.alpha)) / k2);
      }
  return true;
}

}  // namespace plum
