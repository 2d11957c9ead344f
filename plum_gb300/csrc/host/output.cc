// The reference's output files, written by the host Simulation from the
// device state at the steps where the reference writes them
// (simulation.cc:120-131 opens them, 685-1064 writes them). The formatting
// is the reference's: the same ostream insertions and precisions, including
// the precision each stream keeps from its previous setprecision.
//
// The stat file's pressure columns are ForceField::GetPressure's: the
// wall-force pressure tensor for systems with walls, "nan" without. The
// reference's LJ columns there come from its PairForce, which reads an
// uninitialised local (potential_truncated_lj.cc:95-100); these follow the
// function's evident intent, so those three columns can differ from the
// reference's own files.
#include <cmath>
#include <cstdint>
#include <fstream>
#include <iomanip>
#include <sstream>
#include <stdexcept>
#include <vector>

#include "../../../include/plum_host.hpp"

namespace plum {

namespace {
constexpr double kRhoZ = 0.02;  // density_z_res (simulation.cc:113)
}

void Simulation::EnableOutput(const std::string& dir) {
  out_dir_ = dir.empty() ? "." : dir;
  run_name_ = run_.run_name;
  const std::string base = out_dir_ + "/" + run_name_;
  info_out.open(base + "_stat.dat");
  traj_p_out.open(base + "_traj_p.xyz");
  traj_c_out.open(base + "_traj_c.xyz");
  traj_a_out.open(base + "_traj_a.xyz");
  traj_n_out.open(base + "_traj_n.xyz");
  if (!info_out || !traj_p_out || !traj_c_out || !traj_a_out || !traj_n_out)
    throw InputError("cannot open the output files in " + out_dir_);
  out_on_ = true;
  PrintStatHeader();
}

void Simulation::PrintStatHeader() {
  info_out << "#Step";
  if (run_.use_pair) info_out << " " << "<PairEne>";
  if (run_.use_ewald) info_out << " " << "<EwaldEne>";
  if (run_.use_bond) info_out << " " << "<BondEne>";
  if (run_.use_ext) info_out << " " << "<ExtPotEne>";
  info_out << " " << "<TotalEnergy>";
  if (run_.use_gc) {
    info_out << " " << "NoOfMol";
    info_out << " " << "<Density>";
  }
  if (run_.use_ext)
    info_out << " " << "<Pzz_LJ_ion> <Pzz_LJ_pol> <Pzz_LJ_wal> <Pzz_EL_ion>"
             << " " << "<Pzz_EL_pol> <Pzz_EL_wal>";
  else
    info_out << " " << "<P>";
  if (run_.calc_chem_pot) info_out << " " << "mu";
  info_out << " " << "<|Rg|> <|Rgx|> <|Rgy|> <|Rgz|> <ete>";
  info_out << " " << "beadtrans comtrans pivot crankshaft reptate";
  if (run_.use_gc) info_out << " " << "insert delete";
  info_out << std::endl;
}

void Simulation::PrintStat() {
  if (!out_on_ || run_.stat_out_freq <= 0 || step % run_.stat_out_freq != 0) return;
  info_out << step;
  const double n = (double)ff_avg_counter;
  double tot_energy = 0;
  if (run_.use_pair) {
    info_out << " " << std::setprecision(7) << pair_e_cumu / n;
    tot_energy += pair_e_cumu / n;
  }
  if (run_.use_ewald) {
    info_out << " " << std::setprecision(7) << ewald_e_cumu / n;
    tot_energy += ewald_e_cumu / n;
  }
  if (run_.use_bond) {
    info_out << " " << std::setprecision(7) << bond_e_cumu / n;
    tot_energy += bond_e_cumu / n;
  }
  if (run_.use_ext) {
    info_out << " " << std::setprecision(7) << ext_e_cumu / n;
    tot_energy += ext_e_cumu / n;
  }
  info_out << " " << tot_energy;
  if (run_.use_gc)
    info_out << " " << (int)mols.size() << " " << std::setprecision(4) << density_cumu / n;
  info_out << " " << force_field.GetPressure();
  if (run_.calc_chem_pot) {
    if (chem_pot_cumu / n > 0)
      info_out << " " << -(1.0 / run_.beta) * std::log(chem_pot_cumu / n);
    else
      info_out << " INF";
  }
  const double m = (double)mol_avg_counter;
  info_out << " " << std::setprecision(4) << std::sqrt(rg_tot_cumu / m) << " "
           << std::setprecision(4) << std::sqrt(rg_x_cumu / m) << " " << std::setprecision(4)
           << std::sqrt(rg_y_cumu / m) << " " << std::setprecision(4) << std::sqrt(rg_z_cumu / m)
           << " " << std::setprecision(4) << std::sqrt(e_to_e_cumu / m);
  for (int k = 0; k < 5; k++) info_out << " " << accepted[k] / (double)attempted[k];
  if (run_.use_gc) {
    info_out << " " << insertion_accepted / (double)insertion_attempted;
    info_out << " " << deletion_accepted / (double)deletion_attempted;
  }
  info_out << std::endl;
}

namespace {

// Shift that brings a molecule's centre into the primary cell
// (simulation.cc:895-906): floor(centre / L) * L per axis.
void image_shift(const Molecule& m, const double* box, double* d) {
  double c[3] = {0, 0, 0};
  for (const Bead& b : m.bds)
    for (int a = 0; a < 3; a++) c[a] += b.GetCrd(0, a);
  for (int a = 0; a < 3; a++) {
    c[a] /= (double)m.Size();
    d[a] = std::floor(c[a] / box[a]) * box[a];
  }
}

}  // namespace

void Simulation::PrintTraj() {
  if (!out_on_ || !(step > run_.steps_eq && run_.traj_out_freq > 0 &&
                    step % run_.traj_out_freq == 0))
    return;
  if (run_.grafted + n_chain > 0) {
    traj_p_out << n_chain_b << std::endl;
    traj_p_out << "STEP: " << step << std::endl;
  }
  if (n_cion > 0) {
    traj_c_out << n_cion << std::endl;
    traj_c_out << "STEP: " << step << std::endl;
  }
  if (n_aion > 0) {
    traj_a_out << n_aion << std::endl;
    traj_a_out << "STEP: " << step << std::endl;
  }
  if (n_nion > 0) {
    traj_n_out << n_nion << std::endl;
    traj_n_out << "STEP: " << step << std::endl;
  }
  for (int i = run_.phantom; i < n_mol; i++) {
    double d[3];
    image_shift(mols[i], box_l, d);
    std::ofstream* out;
    if (mols[i].Size() > 1)
      out = &traj_p_out;
    else if (mols[i].bds[0].Charge() > 0)
      out = &traj_c_out;
    else if (mols[i].bds[0].Charge() < 0)
      out = &traj_a_out;
    else
      out = &traj_n_out;
    for (const Bead& b : mols[i].bds) {
      *out << b.Symbol() << " ";
      *out << b.GetCrd(0, 0) - d[0] << " ";
      *out << b.GetCrd(0, 1) - d[1] << " ";
      *out << b.GetCrd(0, 2) - d[2] << std::endl;
    }
  }
}

void Simulation::PrintLastCrd() {
  if (!out_on_ || !(step > run_.steps_eq && run_.stat_out_freq > 0 &&
                    step % run_.stat_out_freq == 0))
    return;
  const char* bck[2] = {"", "2"};
  for (int f = 0; f < 2; f++) {
    crd_last_out[f].open(out_dir_ + "/" + run_name_ + "_lastcrd.dat" + bck[f]);
    crd_last_out[f] << n_bead_ << std::endl;
    crd_last_out[f] << " " << std::endl;
    for (int i = 0; i < n_mol; i++) {
      double d[3];
      image_shift(mols[i], box_l, d);
      if (i < run_.phantom) d[0] = d[1] = d[2] = 0;
      for (const Bead& b : mols[i].bds) {
        crd_last_out[f] << i << " ";
        crd_last_out[f] << b.Symbol() << " ";
        crd_last_out[f] << std::setprecision(18) << b.GetCrd(0, 0) - d[0] << " ";
        crd_last_out[f] << std::setprecision(18) << b.GetCrd(0, 1) - d[1] << " ";
        crd_last_out[f] << std::setprecision(18) << b.GetCrd(0, 2) - d[2] << " ";
        crd_last_out[f] << std::setprecision(4) << b.Charge() << std::endl;
      }
    }
    crd_last_out[f].close();
  }
}

void Simulation::PrintLastTop() {
  if (!out_on_ || !(step > run_.steps_eq && run_.stat_out_freq > 0 &&
                    step % run_.stat_out_freq == 0))
    return;
  top_last_out.open(out_dir_ + "/" + run_name_ + "_lasttop.dat");
  top_last_out << "TotNoOfBeads: " << n_bead_ << std::endl;
  top_last_out << "TotNoOfMolec: " << n_mol << std::endl;
  top_last_out << "Box_Length_X: " << std::setprecision(18) << box_l[0] << std::endl;
  top_last_out << "Box_Length_Y: " << std::setprecision(18) << box_l[1] << std::endl;
  top_last_out << "Box_Length_Z: " << std::setprecision(18) << box_l[2] << std::endl;
  top_last_out << "bonds:" << std::endl;
  top_last_out << "-1" << std::endl;
  top_last_out << "angles:" << std::endl;
  top_last_out << "-1" << std::endl;
  top_last_out << "diheds" << std::endl;
  top_last_out << "-1" << std::endl;
  top_last_out.close();
}

void Simulation::PrintLastRhoZ() {
  if (!out_on_ || !(step > run_.steps_eq && run_.stat_out_freq > 0 &&
                    step % run_.stat_out_freq == 0))
    return;
  const char* bck[2] = {"", "2"};
  const int bins = (int)density_z_cumu.size() / 3;
  for (int f = 0; f < 2; f++) {
    rho_last_out[f].open(out_dir_ + "/" + run_name_ + "_lastrhoZ.dat" + bck[f]);
    for (int bin = 0; bin < bins; bin++) {
      const double pos = (bin + 0.5) * kRhoZ;
      rho_last_out[f] << pos << '\t' << density_z_cumu[3 * bin + 0] / (double)ff_avg_counter
                      << '\t' << density_z_cumu[3 * bin + 1] / (double)ff_avg_counter << '\t'
                      << density_z_cumu[3 * bin + 2] / (double)ff_avg_counter << std::endl;
    }
    rho_last_out[f].close();
  }
}

void Simulation::Finish() {
  if (!out_on_) return;
  // the reference's destructor runs after its step loop, with step one past
  // the last step
  const long keep = step;
  step = keep + 1;
  PrintLastCrd();
  PrintLastTop();
  step = keep;
  info_out.close();
  traj_p_out.close();
  traj_c_out.close();
  traj_a_out.close();
  traj_n_out.close();
  out_on_ = false;
}

namespace {

template <typename T>
void put(std::ostream& o, const T& v) {
  o.write(reinterpret_cast<const char*>(&v), sizeof(T));
}
template <typename T>
void get(std::istream& i, T& v) {
  i.read(reinterpret_cast<char*>(&v), sizeof(T));
}
constexpr uint32_t kCkptMagic = 0x3243504cu;  // "LPC2"

void put_str(std::ostream& o, const std::string& v) {
  put(o, (uint32_t)v.size());
  o.write(v.data(), (std::streamsize)v.size());
}
bool get_str(std::istream& i, std::string* v) {
  uint32_t n = 0;
  get(i, n);
  if (!i || n > 4096) return false;
  v->assign(n, ' ');
  i.read(&(*v)[0], (std::streamsize)n);
  return (bool)i;
}

// The molecule list of an exchange run: per molecule its beads (symbol, id,
// chain id, type, charge, position) and bonds.
void put_mols(std::ostream& o, const std::vector<Molecule>& mols) {
  put(o, (uint64_t)mols.size());
  for (const Molecule& m : mols) {
    put(o, (uint32_t)m.bds.size());
    for (const Bead& b : m.bds) {
      put_str(o, b.Symbol());
      const int iv[3] = {b.ID(), b.ChainID(), b.Type()};
      const double dv[4] = {b.Charge(), b.GetCrd(0, 0), b.GetCrd(0, 1), b.GetCrd(0, 2)};
      for (int v : iv) put(o, v);
      for (double v : dv) put(o, v);
    }
    put(o, (uint32_t)m.bonds.size());
    for (const auto& bd : m.bonds) {
      put(o, (int32_t)bd[0]);
      put(o, (int32_t)bd[1]);
    }
  }
}

bool get_mols(std::istream& i, std::vector<Molecule>* mols) {
  uint64_t n = 0;
  get(i, n);
  if (!i || n > (1u << 26)) return false;
  mols->assign(n, Molecule());
  for (Molecule& m : *mols) {
    uint32_t nb = 0;
    get(i, nb);
    if (!i || nb > (1u << 26)) return false;
    for (uint32_t k = 0; k < nb; k++) {
      std::string sym;
      if (!get_str(i, &sym)) return false;
      int iv[3];
      double dv[4];
      for (int& v : iv) get(i, v);
      for (double& v : dv) get(i, v);
      Bead b(sym, iv[0], iv[1], dv[0], dv[1], dv[2], dv[3]);
      b.SetType(iv[2]);
      m.AddBead(b);
    }
    uint32_t nbond = 0;
    get(i, nbond);
    if (!i || nbond > (1u << 26)) return false;
    for (uint32_t k = 0; k < nbond; k++) {
      int32_t a = 0, c = 0;
      get(i, a);
      get(i, c);
      m.AddBond(a, c);
    }
  }
  return (bool)i;
}

// Same beads (type and charge) in the same order: the structure a context
// holds for a molecule; positions are the snapshot's.
bool same_structure(const Molecule& a, const Molecule& b) {
  if (a.Size() != b.Size()) return false;
  for (int k = 0; k < a.Size(); k++)
    if (a.bds[k].Type() != b.bds[k].Type() || a.bds[k].Charge() != b.bds[k].Charge())
      return false;
  return true;
}

}  // namespace

void Simulation::WriteCheckpoint(const std::string& path) {
  std::ofstream o(path, std::ios::binary);
  if (!o) throw InputError("cannot write " + path);
  std::ostringstream g;
  g << rand_gen;
  const std::string gs = g.str();
  put(o, kCkptMagic);
  put(o, step);
  put(o, (uint64_t)gs.size());
  o.write(gs.data(), (std::streamsize)gs.size());
  for (int k = 0; k < 5; k++) {
    put(o, accepted[k]);
    put(o, attempted[k]);
  }
  const double sums[10] = {pair_e_cumu, ewald_e_cumu, bond_e_cumu, ext_e_cumu, rg_tot_cumu,
                           rg_x_cumu,   rg_y_cumu,    rg_z_cumu,   e_to_e_cumu, density_cumu};
  for (double v : sums) put(o, v);
  put(o, ff_avg_counter);
  put(o, mol_avg_counter);
  put(o, (uint64_t)density_z_cumu.size());
  o.write(reinterpret_cast<const char*>(density_z_cumu.data()),
          (std::streamsize)(sizeof(double) * density_z_cumu.size()));
  put(o, chem_pot_cumu);
  put(o, force_field.vp_z);
  for (double v : force_field.p_tensor) put(o, v);
  put(o, (int32_t)force_field.UseGC());
  if (force_field.UseGC()) {
    const long gc[4] = {insertion_attempted, insertion_accepted, deletion_attempted,
                        deletion_accepted};
    for (long v : gc) put(o, v);
    int iset = 0;
    double gset = 0;
    force_field.GasdevState(&iset, &gset);
    put(o, iset);
    put(o, gset);
    SyncFromDevice();
    put_mols(o, mols);
  }
  const long n = plum_ctx_snapshot_size(force_field.Context());
  std::vector<char> snap((size_t)n);
  if (plum_ctx_save(force_field.Context(), snap.data(), n))
    throw std::runtime_error(std::string("plum_ctx_save: ") + plum_last_error());
  put(o, (uint64_t)n);
  o.write(snap.data(), n);
  if (!o) throw InputError("cannot write " + path);
}

void Simulation::ReadCheckpoint(const std::string& path) {
  std::ifstream i(path, std::ios::binary);
  uint32_t magic = 0;
  get(i, magic);
  if (!i || magic != kCkptMagic) throw InputError(path + " is not a checkpoint");
  get(i, step);
  uint64_t len = 0;
  get(i, len);
  std::string gs(len, ' ');
  i.read(&gs[0], (std::streamsize)len);
  std::istringstream g(gs);
  g >> rand_gen;
  for (int k = 0; k < 5; k++) {
    get(i, accepted[k]);
    get(i, attempted[k]);
  }
  double sums[10];
  for (double& v : sums) get(i, v);
  pair_e_cumu = sums[0];
  ewald_e_cumu = sums[1];
  bond_e_cumu = sums[2];
  ext_e_cumu = sums[3];
  rg_tot_cumu = sums[4];
  rg_x_cumu = sums[5];
  rg_y_cumu = sums[6];
  rg_z_cumu = sums[7];
  e_to_e_cumu = sums[8];
  density_cumu = sums[9];
  get(i, ff_avg_counter);
  get(i, mol_avg_counter);
  get(i, len);
  if (len != density_z_cumu.size()) throw InputError(path + " belongs to another box");
  i.read(reinterpret_cast<char*>(density_z_cumu.data()), (std::streamsize)(sizeof(double) * len));
  get(i, chem_pot_cumu);
  get(i, force_field.vp_z);
  for (double& v : force_field.p_tensor) get(i, v);
  int32_t gc_run = 0;
  get(i, gc_run);
  if (!i || gc_run != (int32_t)force_field.UseGC())
    throw InputError(path + " belongs to another kind of run");
  if (gc_run) {
    long gc[4];
    for (long& v : gc) get(i, v);
    insertion_attempted = gc[0];
    insertion_accepted = gc[1];
    deletion_attempted = gc[2];
    deletion_accepted = gc[3];
    int iset = 0;
    double gset = 0;
    get(i, iset);
    get(i, gset);
    force_field.SetGasdevState(iset, gset);
    std::vector<Molecule> saved;
    if (!get_mols(i, &saved)) throw InputError(path + " is truncated");
    // give the context the checkpoint's molecules: keep the common prefix,
    // append the checkpoint's tail, then erase the old tail (as GCMove
    // appends and erases), so the context never holds zero molecules
    size_t keep = 0;
    while (keep < mols.size() && keep < saved.size() && same_structure(mols[keep], saved[keep]))
      keep++;
    const int old_n = (int)mols.size();
    const int n_add = (int)(saved.size() - keep);
    for (size_t m = keep; m < saved.size(); m++) mols.push_back(saved[m]);
    if (n_add > 0) force_field.EnergyInitForAddedMolecule(mols, n_add);
    if (old_n > (int)keep) {
      force_field.AdjustEnergyUponMolDeletion((int)keep, old_n - (int)keep);
      mols.erase(mols.begin() + keep, mols.begin() + old_n);
    }
    for (size_t m = 0; m < keep; m++) mols[m] = saved[m];
  }
  get(i, len);
  std::vector<char> snap(len);
  i.read(snap.data(), (std::streamsize)len);
  if (!i) throw InputError(path + " is truncated");
  if (plum_ctx_load(force_field.Context(), snap.data(), (long)len))
    throw InputError(std::string("plum_ctx_load: ") + plum_last_error());
  SyncFromDevice();
  UpdateMolCounts();
}

}  // namespace plum
