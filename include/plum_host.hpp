// C++ host classes with the reference's public surface, backed by the GB300
// engine (include/plum_gpu.h).
//
// A program written against the reference's Simulation / ForceField /
// Molecule / Bead (src/simulation/simulation.h:20-201,
// src/force_field/force_field.h:22-294, src/molecules/molecule.h:16-69,
// src/molecules/bead.h:14-87) switches by including this header and using
// namespace plum. Method names, argument meaning and draw order are the
// reference's; energies live on the GPU:
//
//   ForceField::EnergyDifference / FinalizeEnergies / Tot*Energy / InitializeEnergy
//       -> plum_delta_energy / plum_finalize / plum_energies / plum_total_energy
//   Simulation::TranslationalMove   host control flow, device energies
//   Simulation::Run                 the whole step loop on the device, with
//                                   rand_gen kept in step with the draws used
//
// Differences: bad input throws plum::InputError instead of exit(1);
// Simulation takes an explicit seed (the reference seeds from the clock,
// simulation.cc:133-136); grand-canonical runs step on the host (Step), each
// exchange growth step's trial energies in one device call.
#pragma once

#include <fstream>
#include <istream>
#include <random>
#include <stdexcept>
#include <string>
#include <vector>

#include "plum_gpu.h"

namespace plum {

struct InputError : std::runtime_error {
  using std::runtime_error::runtime_error;
};

class Bead {  // bead.h:14-87
 public:
  Bead();
  Bead(std::string symbol, int id, int c_id, double q, double x, double y, double z);
  double Charge() const { return q_; }
  void SetCharge(double q) { q_ = q; }
  int ID() const { return id_; }
  int ChainID() const { return c_id_; }
  void SetID(int id) { id_ = id; }
  void SetChainID(int c) { c_id_ = c; }
  std::string Symbol() const { return symbol_; }
  void SetSymbol(std::string s) { symbol_ = s; }
  int Type() const { return type_; }
  void SetType(int t) { type_ = t; }
  bool GetMoved() const { return moved_; }
  void SetMoved() { moved_ = true; }
  void UnsetMoved() { moved_ = false; }
  // flag 0: current position, 1: trial position; index 0..2 = x, y, z
  double GetCrd(int flag, int index) const;
  void SetCrd(int flag, int index, double value);
  void SetAllCrd(double pos[3]);
  void UpdateCurrentPos();
  void UpdateTrialPos();
  // minimum-image distance of the trial positions (bead.cc:162-176)
  double BBDist(const Bead& other, const double box_l[], int npbc) const;

 private:
  double current_[3], trial_[3];
  double q_ = 0;
  int id_ = -1, c_id_ = -1, type_ = 0;
  std::string symbol_ = "NONE";
  bool moved_ = false;
};

class Molecule {  // molecule.h:16-69
 public:
  std::vector<Bead> bds;
  std::vector<std::vector<int>> bonds;
  void AddBead(Bead b) { bds.push_back(b); }
  void AddBond(int i, int j) { bonds.push_back({i, j}); }
  int Size() const { return (int)bds.size(); }
  int NBond() const { return (int)bonds.size(); }
  // Monte Carlo moves (molecule.cc:103-312): write trial positions and set
  // the moved flags, consuming draws in the reference's order.
  void BeadTranslate(double move_size, double box_l[3], std::mt19937& rand_gen);
  void COMTranslate(double move_size, std::mt19937& rand_gen);
  void Pivot(double move_size, std::mt19937& rand_gen, double eq_bond_len, bool vary_bond);
  void Crankshaft(double move_size, std::mt19937& rand_gen);
  void RandomReptation(std::mt19937& rand_gen, double eq_bond_len, bool vary_bond);
};

class ForceField {  // force_field.h:22-294 (energy surface)
 public:
  ForceField() = default;
  ~ForceField();
  ForceField(const ForceField&) = delete;
  ForceField& operator=(const ForceField&) = delete;
  // Builds the device context from run.in text (crd/top relative to dir) and
  // fills mols with the system read from the coordinate file.
  void Initialize(const std::string& dir, const std::string& runin_text,
                  std::vector<Molecule>& mols, int form = PLUM_FORM_FP64, int device = 0);
  void InitializeEnergy(std::vector<Molecule>& mols);
  double EnergyDifference(std::vector<Molecule>& mols, int moved_mol);
  void FinalizeEnergies(std::vector<Molecule>& mols, bool accept, int moved_mol);
  double TotPairEnergy();
  double TotEwaldEnergy();
  double TotBondEnergy();
  double TotExtEnergy();
  bool UseGC() const { return run_.use_gc; }
  bool UsePairPot() const { return run_.use_pair; }
  bool UseEwaldPot() const { return run_.use_ewald; }
  bool UseBondPot() const { return run_.use_bond; }
  bool UseBondRigid() const { return run_.use_bond_rigid; }
  bool UseExtPot() const { return run_.use_ext; }
  int GCFrequency() const { return run_.gc_freq; }
  double RigidBondLen() const { return run_.rigid_bond; }
  double EqBondLen() const;
  plum_ctx* Context() const { return ctx_; }
  const plum_run_info& RunInfo() const { return run_; }
  const plum_info& Info() const { return info_; }

  // Grand-canonical exchange with configurational bias (cbmc.cc:5-442):
  // draws on the host in the reference's order, the trial-site energies of
  // each growth step in one batched device call (plum_cbmc_trials).
  // Insertion returns whether the grown chain was accepted (it is then
  // appended to mols, with its counterions for a charged species); deletion
  // returns the molecule to delete, or -1.
  bool CBMCFChainInsertion(std::vector<Molecule>& mols, std::mt19937& rand_gen);
  int CBMCFChainDeletion(std::vector<Molecule>& mols, std::mt19937& rand_gen);
  // cbmc.cc:444-531: Widom's average over 50 configurational-bias test
  // insertions of the exchanged species (consumes draws like the reference)
  double CalcChemicalPotentialF(std::vector<Molecule>& mols, std::mt19937& rand_gen);
  // Commits the molecules appended to mols / removes molecules on the device
  // (force_field.cc:1088-1105; the potentials' AdjustEnergyUponMolDeletion).
  void EnergyInitForAddedMolecule(std::vector<Molecule>& mols, int n_added);
  void AdjustEnergyUponMolDeletion(int first, int count);
  // pressure.cc:404-488: one evaluation of the wall-force pressure of a slit
  // system on the device (plum_pressure_slit), accumulated into p_tensor as
  // the reference accumulates it (the wall-wall terms on the first
  // evaluation only) and averaged over the evaluations.
  void CalcPressureForceLJELSlit(std::vector<Molecule>& mols);
  // pressure.cc:490-500: p_tensor[0..5] for systems with walls, else "nan"
  std::string GetPressure() const;
  // p_tensor[0..11]: 0-5 the averages GetPressure prints (LJ ions, polymers,
  // wall-wall; Ewald ions, polymers, wall-wall), 6-11 the accumulators
  double p_tensor[12] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
  double vp_z = 0;  // evaluations so far
  // gasdev's cached deviate (misc.cc:112-113), for checkpoints
  void GasdevState(int* iset, double* gset) const {
    *iset = gd_iset_;
    *gset = gd_gset_;
  }
  void SetGasdevState(int iset, double gset) {
    gd_iset_ = iset;
    gd_gset_ = gset;
  }
  double ChemPot() const { return gc_[0]; }
  int GCChainLen() const { return (int)gc_[3]; }
  double GCBeadCharge() const { return gc_[2]; }

 private:
  double CBMCFGenTrialBeads(const double* end, int current_len, std::mt19937& rand_gen,
                            int delete_id, const double* replace_first);
  double RandomBondLen(std::mt19937& rand_gen);  // potential_spring.cc:50-61
  double Gasdev(double mean, double sd, std::mt19937& rand_gen);  // misc.cc:111-134
  void GCCounts(const std::vector<Molecule>& mols, int* spc1, int* spc2) const;
  plum_ctx* ctx_ = nullptr;
  plum_run_info run_{};
  plum_info info_{};
  std::vector<int> mol_start_;
  double gc_[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};  // plum_gc_info
  std::vector<std::string> type_names_;
  // cbmc_chain (grown beads then their counterions), trial sites and weights
  std::vector<double> chain_, tb1_, tb2_, w_, u_;
  // gasdev's cached second deviate (the reference keeps it in statics)
  int gd_iset_ = 0;
  double gd_gset_ = 0;
};

class Simulation {  // simulation.h:20-201 (step loop and observables)
 public:
  // Reads run.in from `runin` (std::cin for the reference's usage
  // `plum < run.in`); crd/top paths are relative to dir.
  Simulation(std::istream& runin, const std::string& dir = ".", unsigned seed = 5489u,
             int form = PLUM_FORM_FP64, int device = 0);
  ~Simulation() { Finish(); }  // the reference's destructor writes (simulation.cc:202-211)
  void Run();                 // steps from run.in, on the device
  void RunSteps(long n);      // n steps on the device
  void TranslationalMove();   // one step, host control flow (simulation.cc:241-355)
  void GCMove();              // simulation.cc:357-404
  // One step of Simulation::Run's loop (simulation.cc:219-226): the draw,
  // then GCMove or TranslationalMove; last_move_type 5 / 6 for an insertion
  // / deletion attempt, last_accept when the molecule count changed.
  void Step();
  // simulation.cc:723-798: energies, density, rho(z), the wall-force
  // pressure of systems with walls every 10 samples, Widom's chemical
  // potential when run.in asks for it, Rg (x, y, z rounded to six significant
  // digits as the reference's string round trip does), end to end distance.
  // Without walls the reference evaluates CalcPressureVolScalingHSELSlit
  // there, whose results are never printed (GetPressure prints "nan"); it is
  // not evaluated here.
  void Sample();
  double RadiusOfGyration();  // simulation.cc:406-434
  double EndToEndDistance();  // simulation.cc:483-501
  void UpdateMolCounts();     // simulation.cc:1066-1094
  void SyncFromDevice();      // refresh host bead positions after device steps

  // The reference's output files (simulation.cc:120-131), written into dir:
  // <run_name>_stat.dat (its header now), _traj_p/_c/_a/_n.xyz,
  // _lastcrd.dat and .dat2, _lasttop.dat, _lastrhoZ.dat and .dat2, at the
  // steps where the reference writes them. Off until this is called.
  void EnableOutput(const std::string& dir = ".");
  void PrintStatHeader();  // simulation.cc:685-721
  void PrintStat();        // simulation.cc:800-867
  void PrintTraj();        // simulation.cc:869-933
  void PrintLastCrd();     // simulation.cc:935-979
  void PrintLastTop();     // simulation.cc:981-1027
  void PrintLastRhoZ();    // simulation.cc:1047-1064
  // The writes of the reference's destructor (simulation.cc:202-211), which
  // see step = steps + 1; closes the files.
  void Finish();
  // Exact restart (no reference counterpart): the step count, the
  // generator's state, the counters and running averages, and the device
  // context's snapshot (plum_ctx_save); for runs with grand-canonical
  // exchange also the molecule list, the exchange counters and gasdev's
  // cached deviate. ReadCheckpoint on a Simulation built from the same
  // inputs continues bit-identically: it first gives the context the
  // checkpoint's molecules (the molecules after the longest common prefix
  // are replaced, as an exchange appends and erases them).
  void WriteCheckpoint(const std::string& path);
  void ReadCheckpoint(const std::string& path);

  std::vector<Molecule> mols;
  ForceField force_field;
  std::mt19937 rand_gen;
  long step = 0;
  int accepted[5] = {0, 0, 0, 0, 0}, attempted[5] = {0, 0, 0, 0, 0};
  double pair_e_cumu = 0, ewald_e_cumu = 0, bond_e_cumu = 0, ext_e_cumu = 0, rg_tot_cumu = 0;
  double rg_x_cumu = 0, rg_y_cumu = 0, rg_z_cumu = 0, e_to_e_cumu = 0, density_cumu = 0;
  double chem_pot_cumu = 0;
  std::vector<double> density_z_cumu;  // [3 * bins] as CalcRhoZ accumulates it
  long ff_avg_counter = 0, mol_avg_counter = 0;
  int last_move_type = -1, last_accept = 0;
  long insertion_attempted = 0, insertion_accepted = 0;
  long deletion_attempted = 0, deletion_accepted = 0;

 private:
  plum_run_info run_{};
  double box_l[3];
  int npbc = 3;
  int n_mol = 0, n_chain = 0, n_chain_b = 0, n_cion = 0, n_aion = 0, n_nion = 0;
  int n_bead_ = 0;  // phantom + beads of the other molecules (UpdateMolCounts)
  bool out_on_ = false;
  std::string out_dir_, run_name_;
  std::ofstream info_out, traj_p_out, traj_c_out, traj_a_out, traj_n_out;
  std::ofstream crd_last_out[2], top_last_out, rho_last_out[2];
};

}  // namespace plum
