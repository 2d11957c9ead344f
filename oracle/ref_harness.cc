// Harness that links the UNMODIFIED reference sources (nuwapi/Plum src/) into
// oracle/_ref/libplumref.so and exposes a small C interface to the tests.
//
// Test infrastructure only (the reference checker): it is never part of the
// product and is loaded only by tests/ and by bench.py's CPU-baseline leg.
//
// What it adds around the reference:
//  * std::cin is pointed at a run.in file so that the reference's own
//    positional readers (simulation.cc:23-50, force_field.cc:64-195 and the
//    potentials' ReadParameters) parse it; std::cout goes to a log file.
//  * The reference seeds mt19937 from the wall clock (simulation.cc:133-136);
//    the harness reseeds `rand_gen` after construction so runs are repeatable.
//  * Private members are reached by compiling the reference headers with
//    `private` mapped to `public` in this translation unit only.
//  * Per-step bookkeeping (move type, accept flag, draws consumed) is read
//    from the reference's own counters (simulation.h:110-111) and from the
//    generator state, so the reference code path itself is unchanged.

#include <unistd.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <map>
#include <random>
#include <set>
#include <sstream>
#include <string>
#include <vector>

#define private public
#define protected public
#include "simulation/simulation.h"
#include "force_field/potential_ewald_coul.h"
#undef private
#undef protected

namespace {

struct Handle {
  Simulation* sim = nullptr;
  std::string dir;
  std::ofstream log;
};

struct CwdGuard {
  char old[4096];
  explicit CwdGuard(const std::string& d) {
    if (!getcwd(old, sizeof(old))) old[0] = 0;
    if (chdir(d.c_str()) != 0) perror("chdir");
  }
  ~CwdGuard() {
    if (old[0] && chdir(old) != 0) perror("chdir back");
  }
};

struct StreamSwap {
  std::streambuf* in_old;
  std::streambuf* out_old;
  StreamSwap(std::streambuf* in, std::streambuf* out)
      : in_old(std::cin.rdbuf(in)), out_old(std::cout.rdbuf(out)) {}
  ~StreamSwap() {
    std::cin.rdbuf(in_old);
    std::cout.rdbuf(out_old);
  }
};

long draws_between(std::mt19937 a, const std::mt19937& b, long cap) {
  long n = 0;
  while (!(a == b) && n < cap) {
    a();
    n++;
  }
  return a == b ? n : -1;
}

Bead& bead_at(Simulation* s, int mol, int b) { return s->mols[mol].bds[b]; }

}  // namespace

extern "C" {

// Builds a reference Simulation from `runin` (path relative to `dir`), with
// the working directory set to `dir`, then seeds its mt19937 with `seed`.
void* pr_create(const char* dir, const char* runin, unsigned seed) {
  Handle* h = new Handle();
  h->dir = dir;
  CwdGuard cg(h->dir);
  std::ifstream in(runin);
  if (!in) {
    delete h;
    return nullptr;
  }
  h->log.open("ref_harness.log");
  StreamSwap sw(in.rdbuf(), h->log.rdbuf());
  h->sim = new Simulation();
  h->sim->rand_gen.seed(seed);
  h->sim->step = 0;
  h->sim->UpdateMolCounts();
  return h;
}

void pr_destroy(void* hp) {
  Handle* h = (Handle*)hp;
  if (!h) return;
  {
    CwdGuard cg(h->dir);
    StreamSwap sw(std::cin.rdbuf(), h->log.rdbuf());
    delete h->sim;
  }
  delete h;
}

int pr_n_mol(void* hp) { return (int)((Handle*)hp)->sim->mols.size(); }

int pr_n_bead(void* hp) {
  Simulation* s = ((Handle*)hp)->sim;
  int n = 0;
  for (auto& m : s->mols) n += m.Size();
  return n;
}

int pr_mol_size(void* hp, int mol) { return ((Handle*)hp)->sim->mols[mol].Size(); }

// Running energy totals kept by the reference (force_field.cc:1201-1219):
// out = {pair, ewald, bond, ext}; unused terms are 0.
void pr_energies(void* hp, double* out) {
  Simulation* s = ((Handle*)hp)->sim;
  ForceField& f = s->force_field;
  out[0] = f.use_pair_pot ? f.TotPairEnergy() : 0.0;
  out[1] = f.use_ewald_pot ? f.TotEwaldEnergy() : 0.0;
  out[2] = f.use_bond_pot ? f.TotBondEnergy() : 0.0;
  out[3] = f.use_ext_pot ? f.TotExtEnergy() : 0.0;
}

// Current coordinates of every bead, molecule by molecule (n_bead x 3).
void pr_coords(void* hp, double* out) {
  Simulation* s = ((Handle*)hp)->sim;
  size_t k = 0;
  for (auto& m : s->mols)
    for (int b = 0; b < m.Size(); b++)
      for (int d = 0; d < 3; d++) out[k++] = m.bds[b].GetCrd(0, d);
}

// Ewald setup as derived by PotentialEwaldCoul::ReadParameters
// (potential_ewald_coul.cc:29-115):
// out = {real_cutoff, repl_cutoff, real_cell[0..2], repl_cell[0..2],
//        box_l[0..2] (Ewald box, padded for the dipole correction),
//        alpha, lB, box_vol, dipole_correction}
void pr_ewald_info(void* hp, double* out) {
  Simulation* s = ((Handle*)hp)->sim;
  PotentialEwaldCoul* e = (PotentialEwaldCoul*)s->force_field.ewald_pot;
  out[0] = e->real_cutoff;
  out[1] = e->repl_cutoff;
  for (int i = 0; i < 3; i++) out[2 + i] = e->real_cell[i];
  for (int i = 0; i < 3; i++) out[5 + i] = e->repl_cell[i];
  for (int i = 0; i < 3; i++) out[8 + i] = e->box_l[i];
  out[11] = e->alpha;
  out[12] = e->lB;
  out[13] = e->box_vol;
  out[14] = e->dipole_correction ? 1.0 : 0.0;
}

// Individual reference energy routines on beads (mol a, bead i) and
// (mol b, bead j), evaluated at the beads' trial coordinates (which equal the
// current ones between moves): out = {LJ PairEnergy, PairEnergyReal,
// PairEnergyRepl}.
void pr_pair_terms(void* hp, int ma, int ia, int mb, int ib, double* out) {
  Simulation* s = ((Handle*)hp)->sim;
  ForceField& f = s->force_field;
  Bead& a = bead_at(s, ma, ia);
  Bead& b = bead_at(s, mb, ib);
  out[0] = f.use_pair_pot ? f.pair_pot->PairEnergy(a, b, f.box_l, f.npbc) : 0.0;
  out[1] = f.use_ewald_pot ? f.ewald_pot->PairEnergyReal(a, b, f.npbc) : 0.0;
  out[2] = f.use_ewald_pot ? f.ewald_pot->PairEnergyRepl(a, b, f.npbc) : 0.0;
}

double pr_self_energy(void* hp, int m, int i) {
  Simulation* s = ((Handle*)hp)->sim;
  return s->force_field.ewald_pot->SelfEnergy(bead_at(s, m, i));
}

double pr_bond_energy(void* hp, int m) {
  Simulation* s = ((Handle*)hp)->sim;
  ForceField& f = s->force_field;
  return f.bond_pot->MoleculeEnergy(s->mols[m], f.box_l, f.npbc);
}

double pr_ext_energy(void* hp, int m, int i) {
  Simulation* s = ((Handle*)hp)->sim;
  ForceField& f = s->force_field;
  return f.ext_pot->BeadEnergy(bead_at(s, m, i), f.box_l);
}

double pr_dipole_energy(void* hp) {
  Simulation* s = ((Handle*)hp)->sim;
  return s->force_field.ewald_pot->DipoleE(s->mols);
}

// Totals recomputed from scratch by the reference's own EnergyInitialization
// routines (potential_pair.cc:55-100, potential_ewald.cc:176-231,
// potential_bond.cc:16-27, potential_external.cc:48-61). This resets the
// reference's running totals and maps to the recomputed values.
void pr_recompute(void* hp, double* out) {
  Handle* h = (Handle*)hp;
  Simulation* s = h->sim;
  ForceField& f = s->force_field;
  StreamSwap sw(std::cin.rdbuf(), h->log.rdbuf());
  out[0] = out[1] = out[2] = out[3] = 0.0;
  if (f.use_pair_pot) {
    f.pair_pot->EnergyInitialization(s->mols, f.box_l, f.npbc);
    out[0] = f.TotPairEnergy();
  }
  if (f.use_ewald_pot) {
    f.ewald_pot->EnergyInitialization(s->mols, f.npbc);
    out[1] = f.TotEwaldEnergy();
  }
  if (f.use_bond_pot) {
    f.bond_pot->EnergyInitialization(s->mols, f.box_l, f.npbc);
    out[2] = f.TotBondEnergy();
  }
  if (f.use_ext_pot) {
    f.ext_pot->EnergyInitialization(s->mols, f.box_l, f.npbc);
    out[3] = f.TotExtEnergy();
  }
}

// Energy difference of an arbitrary trial configuration of molecule `mol`
// through ForceField::EnergyDifference (force_field.cc:407-434), followed by
// a rejecting FinalizeEnergies so the reference's state is left unchanged.
// trial: mol_size x 3 coordinates; moved: mol_size flags.
// out = {dE_total, dE_pair, dE_ewald}.
void pr_delta_energy(void* hp, int mol, const double* trial, const int* moved,
                     double* out) {
  Simulation* s = ((Handle*)hp)->sim;
  ForceField& f = s->force_field;
  Molecule& m = s->mols[mol];
  for (int i = 0; i < m.Size(); i++) {
    for (int d = 0; d < 3; d++) m.bds[i].SetCrd(1, d, trial[3 * i + d]);
    if (moved[i]) m.bds[i].SetMoved();
  }
  double de = f.EnergyDifference(s->mols, mol);
  out[0] = de;
  out[1] = f.use_pair_pot ? f.pair_pot->dE : 0.0;
  out[2] = f.use_ewald_pot ? f.ewald_pot->dE : 0.0;
  f.FinalizeEnergies(s->mols, false, mol);
  for (int i = 0; i < m.Size(); i++) {
    m.bds[i].UpdateTrialPos();
    m.bds[i].UnsetMoved();
  }
}

// ForceField::CalcPressureForceLJELSlit (pressure.cc:400-488) on the current
// configuration; out12 = p_tensor[0..11] after the call.
void pr_pressure_force_slit(void* hp, double* out12) {
  Handle* h = (Handle*)hp;
  CwdGuard cg(h->dir);
  StreamSwap sw(std::cin.rdbuf(), h->log.rdbuf());
  h->sim->force_field.CalcPressureForceLJELSlit(h->sim->mols);
  for (int i = 0; i < 12; i++) out12[i] = h->sim->force_field.p_tensor[i];
}

// The pieces of the wall-force pressure, on the current configuration:
// PotentialExternal's BeadForceOnWall of one bead, and
// PotentialEwaldCoul::PairForceZReal / PairForceZRepl of the z force on bead
// (ma, ia) from bead (mb, ib): out2 = {real, reciprocal}.
double pr_wall_force(void* hp, int mol, int bead) {
  Simulation* s = ((Handle*)hp)->sim;
  return s->force_field.ext_pot->BeadForceOnWall(s->mols[mol].bds[bead], s->box_l);
}

void pr_ewald_force_z(void* hp, int ma, int ia, int mb, int ib, double* out2) {
  Simulation* s = ((Handle*)hp)->sim;
  Bead& a = s->mols[ma].bds[ia];
  Bead& b = s->mols[mb].bds[ib];
  out2[0] = s->force_field.ewald_pot->PairForceZReal(a, b, s->npbc);
  out2[1] = s->force_field.ewald_pot->PairForceZRepl(a, b, s->npbc);
}

// ForceField::CalcChemicalPotentialF (cbmc.cc:444-531) on the current
// configuration with the run's generator (it consumes draws).
double pr_chem_pot(void* hp) {
  Handle* h = (Handle*)hp;
  CwdGuard cg(h->dir);
  StreamSwap sw(std::cin.rdbuf(), h->log.rdbuf());
  Simulation* s = h->sim;
  s->force_field.UpdateMolCounts(s->mols);
  return s->force_field.CalcChemicalPotentialF(s->mols, s->rand_gen);
}

// The reference's own Simulation::Run (simulation.cc:216-239): every step
// with its sampling and output files (written into the handle's directory).
void pr_run_full(void* hp) {
  Handle* h = (Handle*)hp;
  CwdGuard cg(h->dir);
  StreamSwap sw(std::cin.rdbuf(), h->log.rdbuf());
  h->sim->Run();
}

// Runs `n` steps of the reference's Run loop body (simulation.cc:220-229)
// without the sampling/printing calls. Per step records the move type
// (0..4 translational, 5 insertion attempt, 6 deletion attempt), whether it
// was accepted, how many mt19937 draws it consumed, and the running total
// energy after the step. Returns the number of steps run.
int pr_run(void* hp, int n, int* move_type, int* accept, int* draws,
           double* etot) {
  Handle* h = (Handle*)hp;
  Simulation* s = h->sim;
  CwdGuard cg(h->dir);
  StreamSwap sw(std::cin.rdbuf(), h->log.rdbuf());
  int gc_freq = s->force_field.use_gc ? s->force_field.GCFrequency() : 1;
  for (int t = 0; t < n; t++) {
    int att[kNoMoveType], acc[kNoMoveType];
    std::memcpy(att, s->attempted, sizeof(att));
    std::memcpy(acc, s->accepted, sizeof(acc));
    int ins_att = s->insertion_attempted, del_att = s->deletion_attempted;
    size_t nmol0 = s->mols.size();
    std::mt19937 g0 = s->rand_gen;
    s->step++;
    int rand_num = s->rand_gen();
    if (s->force_field.UseGC() && (rand_num % gc_freq == 0)) {
      s->GCMove();
    } else {
      s->TranslationalMove();
    }
    int mt = -1, ac = 0;
    for (int k = 0; k < kNoMoveType; k++) {
      if (s->attempted[k] != att[k]) mt = k;
      if (s->accepted[k] != acc[k]) ac = 1;
    }
    if (s->insertion_attempted != ins_att) {
      mt = 5;
      ac = s->mols.size() != nmol0;
    }
    if (s->deletion_attempted != del_att) {
      mt = 6;
      ac = s->mols.size() != nmol0;
    }
    if (move_type) move_type[t] = mt;
    if (accept) accept[t] = ac;
    if (draws) draws[t] = (int)draws_between(g0, s->rand_gen, 10000000);
    if (etot) {
      double e[4];
      pr_energies(hp, e);
      etot[t] = e[0] + e[1] + e[2] + e[3];
    }
  }
  return n;
}

// Reference observables (simulation.cc:406-500): out = {Rg^2 averaged over
// chains, Rg_x^2, Rg_y^2, Rg_z^2, end-to-end^2}.
void pr_observables(void* hp, double* out) {
  Simulation* s = ((Handle*)hp)->sim;
  out[0] = s->RadiusOfGyration();
  std::istringstream iss(s->RadiusOfGyrationXYZ());
  iss >> out[1] >> out[2] >> out[3];
  out[4] = s->EndToEndDistance();
}

// One CalcRhoZ pass (simulation.cc:1029-1045) on a zeroed histogram.
// out: 3*n_bin values laid out [bin][species], species 0 chain, 1 q>=0 ion,
// 2 q<0 ion. Returns n_bin.
int pr_rhoz(void* hp, double* out, int cap) {
  Simulation* s = ((Handle*)hp)->sim;
  int nb = s->density_z_bin;
  for (int i = 0; i < 3 * nb; i++) s->density_z_cumu[i] = 0.0;
  s->CalcRhoZ();
  int n = 3 * nb < cap ? 3 * nb : cap;
  for (int i = 0; i < n; i++) out[i] = s->density_z_cumu[i];
  for (int i = 0; i < 3 * nb; i++) s->density_z_cumu[i] = 0.0;
  return nb;
}

// ForceField::BeadsEnergy (cbmc.cc:5-151) for a trial chain bead at b1 and,
// for a charged grand-canonical species, its trial counterion at b2, with the
// first current_len grown beads (and counterions) taken from chain /
// chain_ci (current_len x 3). delete_id = -1 for insertion. Bead symbols and
// charges are the species' own (force_field.cc:383-401).
double pr_beads_energy(void* hp, const double* b1, const double* b2, int current_len,
                       const double* chain, const double* chain_ci, int delete_id) {
  Simulation* s = ((Handle*)hp)->sim;
  ForceField& f = s->force_field;
  const int L = f.gc_chain_len;
  for (int i = 0; i < current_len; i++) {
    double p[3] = {chain[3 * i], chain[3 * i + 1], chain[3 * i + 2]};
    f.cbmc_chain[i].SetAllCrd(p);
    if (f.gc_bead_charge != 0) {
      double c[3] = {chain_ci[3 * i], chain_ci[3 * i + 1], chain_ci[3 * i + 2]};
      f.cbmc_chain[i + L].SetAllCrd(c);
    }
  }
  Bead x1(f.gc_bead_symbol, -1, -1, f.gc_chain_chg[0], b1[0], b1[1], b1[2]);
  Bead x2(f.gc_bead_symbol, -1, -1, -f.gc_chain_chg[0], 0, 0, 0);
  if (b2) {
    double c[3] = {b2[0], b2[1], b2[2]};
    x2.SetAllCrd(c);
  }
  return f.BeadsEnergy(x1, x2, s->mols, current_len, delete_id);
}

// The grand-canonical species: {chain length, bead charge, trials, gc_freq}.
void pr_gc_info(void* hp, double* out) {
  ForceField& f = ((Handle*)hp)->sim->force_field;
  out[0] = f.gc_chain_len;
  out[1] = f.gc_bead_charge;
  out[2] = f.cbmc_no_of_trials;
  out[3] = f.gc_freq;
}

// The reference's generator state as 624 words + position.
void pr_rng_words(void* hp, unsigned n, unsigned* out) {
  std::mt19937 g = ((Handle*)hp)->sim->rand_gen;
  for (unsigned i = 0; i < n; i++) out[i] = (unsigned)g();
}

}  // extern "C"
