// Readers for the reference's input files: run.in (positional "flag value"
// items), the coordinate file and the topology file.
//
// Grammar (the reference's readers, in order):
//   Simulation::Simulation       simulation.cc:30-50
//   ForceField::Initialize       force_field.cc:65-103 (+ GC block if used)
//   pair / Ewald / bond / rigid / external potential blocks
//                                force_field.cc:123-195 with
//                                potential_truncated_lj.cc:20-47,
//                                potential_ewald_coul.cc:29-37,
//                                potential_spring.cc:11-20,
//                                potential_truncated_lj_wall.cc:13-44,
//                                potential_hard_sphere.cc:20-36,
//                                potential_hard_wall.cc:15-33,
//                                potential_well_wall.cc:15-40
//   topology                     simulation.cc:610-646
//   coordinates                  simulation.cc:582-608
// Differences from the reference's readers, all on malformed input only: a
// missing item or "end" token is an error instead of an endless read at EOF
// (potential_truncated_lj.cc:31-35), and a molecule id >= n_mol is rejected
// (the reference lets mol_id == n_mol through, simulation.cc:594).
//
// A trailing block of `plum_*` items after the last potential block is read
// if present (the reference never reads that far): plum_ewald_real_cutoff,
// plum_ewald_kmax, plum_ewald_kcut2.
#pragma once

#include <map>
#include <string>
#include <vector>

namespace plum {

struct LJEntry {
  double sigma = 0.0, epsilon = 0.0;
};

struct Input {
  std::string dir, crd_name, top_name, run_name;
  long steps = 0, steps_eq = 0, sample_freq = 0, stat_out_freq = 0, traj_out_freq = 0;
  int npbc = 3;
  double beta = 1.0, move_size = 1.0;
  int calc_chem_pot = 0, phantom = 0, coion = 0, grafted = 0, grafted_counterion = 0;
  double move_prob[5] = {0, 0, 0, 0, 0};
  double vp_el_res = 0, vp_bead_size = 0;
  int use_pair = 0, use_ewald = 0, use_bond = 0, use_rigid = 0, use_angle = 0,
      use_dihed = 0, use_ext = 0, use_gc = 0;
  // grand canonical block
  double chem_pot = 0, deBroglie = 1;
  int gc_freq = 1, gc_chain_len = 0, cbmc_trials = 0;
  double gc_bead_charge = 0;
  std::string gc_symbol;
  // potentials
  double lj_cut = 0;
  std::map<std::string, LJEntry> lj;
  double lB = 0, dielectric = 0, alpha = 0;
  int dipole = 0;
  double k_bond = 0, r0 = 0, rigid = -1;
  double wall_cut = 0, wall_sigma = 0, wall_eps = 0;
  std::map<std::string, LJEntry> wall;
  // pair_kind 0 TruncatedLJ, 1 HardSphere (radius per symbol,
  // potential_hard_sphere.cc:20-36); ext_kind 0 TruncatedLJWall, 1 HardWall,
  // 2 WellWall (radius per symbol and the well, potential_hard_wall.cc:15-33,
  // potential_well_wall.cc:15-40)
  int pair_kind = 0, ext_kind = 0;
  std::map<std::string, double> hs_radius, wall_radius;
  double well_width = 0, well_depth = 0;
  // extension block
  double x_real_cutoff = -1;
  int x_kmax = -1;
  double x_kcut2 = -1;
  bool x_have_kcut2 = false;
  // topology
  int n_bead_decl = 0, n_mol = 0;
  double box[3] = {0, 0, 0};
  std::vector<std::vector<int>> bonds;  // {mol, i, j}
  // coordinates, grouped by molecule
  std::vector<int> mol_start;           // n_mol + 1
  std::vector<double> xyz, q;
  std::vector<int> type;                // index into type_names
  std::vector<std::string> type_names;  // first-appearance order
  std::vector<int> file_order;          // bead k came from crd row file_order[k]
};

// Reads dir/runin and the files it names. Returns false and sets *err on
// malformed input.
bool read_input(const std::string& dir, const std::string& runin, Input* in,
                std::string* err);
// Same, with the run.in content given as text (crd/top paths relative to dir).
bool read_input_text(const std::string& dir, const std::string& runin_text, Input* in,
                     std::string* err);

}  // namespace plum
