// The Ewald set-up of run.in's parameters (PotentialEwaldCoul::ReadParameters,
// potential_ewald_coul.cc:38-115): the Ewald box (z padded for the dipole
// correction), the real-space cut-off and image cells, the k^2 cut-off and
// k cells, and the half-space k-set {k : 0 < k^2 <= kc^2} with the weights
// e^{-k^2/4a}/k^2. Plain host C++: the C ABI copies it into the device
// parameters, and it can be run and checked without a GPU.
#pragma once

#include <string>
#include <vector>

#include "input.h"

namespace plum {

struct EwaldSetup {
  double ebox[3] = {0, 0, 0};
  double vol = 0;        // Ewald box volume
  double real_cut = 0;   // real-space cut-off
  double kc2 = 0;        // k^2 cut-off (INFINITY when only k cells bound the set)
  int real_cell[3] = {0, 0, 0};
  int kcell[3] = {0, 0, 0};
  std::vector<int> kn;   // 3 integers (nx, ny, nz) per half-space vector
  std::vector<double> kw;
};

// Fills *out from in; false with *err set when a k cell count exceeds
// max_kcell (the device's phase tables hold |n| <= max_kcell per axis).
bool ewald_setup(const Input& in, int max_kcell, EwaldSetup* out, std::string* err);

}  // namespace plum
