// Host classes with the reference's public surface (include/plum_host.hpp).
// Control flow and draw order follow the reference file by file; energies are
// computed on the device through the C ABI.
#include "../../../include/plum_host.hpp"
#include "../../../include/plum_host_capi.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <iterator>
#include <sstream>

namespace plum {

namespace {
constexpr double kMax = 4294967295.0;  // std::mt19937::max()
constexpr double kVeryLargeEnergy = 1e8;

void check(int rc) {
  if (rc != PLUM_OK) throw InputError(plum_last_error());
}

// randSphere (misc.cc:95-109)
void rand_sphere(double* vec, std::mt19937& g) {
  double rs = 2, r1 = 0, r2 = 0;
  while (rs > 1) {
    r1 = 1 - 2 * ((double)g() / kMax);
    r2 = 1 - 2 * ((double)g() / kMax);
    rs = r1 * r1 + r2 * r2;
  }
  double ranh = 2 * std::sqrt(1 - rs);
  vec[0] = r1 * ranh;
  vec[1] = r2 * ranh;
  vec[2] = (1 - 2 * rs);
}
}  // namespace

// ------------------------------------------------------------------ Bead
Bead::Bead() {
  for (int i = 0; i < 3; i++) current_[i] = trial_[i] = 0;
}

Bead::Bead(std::string symbol, int id, int c_id, double q, double x, double y, double z)
    : q_(q), id_(id), c_id_(c_id), symbol_(symbol) {
  trial_[0] = current_[0] = x;
  trial_[1] = current_[1] = y;
  trial_[2] = current_[2] = z;
}

double Bead::GetCrd(int flag, int index) const {
  if (flag == 0) return current_[index];
  if (flag == 1) return trial_[index];
  throw InputError("Bead::GetCrd: invalid flag");
}

void Bead::SetCrd(int flag, int index, double value) {
  if (flag == 0)
    current_[index] = value;
  else if (flag == 1)
    trial_[index] = value;
}

void Bead::SetAllCrd(double pos[3]) {
  for (int i = 0; i < 3; i++) current_[i] = trial_[i] = pos[i];
}

void Bead::UpdateCurrentPos() { std::memcpy(current_, trial_, sizeof(current_)); }
void Bead::UpdateTrialPos() { std::memcpy(trial_, current_, sizeof(trial_)); }

double Bead::BBDist(const Bead& o, const double box_l[], int npbc) const {
  double dist = 0;
  for (int i = 0; i < 3; i++) {
    double d = trial_[i] - o.trial_[i];
    if (i < npbc) {
      d -= box_l[i] * std::round(d / box_l[i]);
      if (std::fabs(d) > 0.5 * box_l[i]) d = box_l[i] - std::fabs(d);
    }
    dist += d * d;
  }
  return std::sqrt(dist);
}

// -------------------------------------------------------------- Molecule
void Molecule::BeadTranslate(double move_size, double box_l[3], std::mt19937& g) {
  (void)box_l;
  double vec[3];
  rand_sphere(vec, g);
  double len = std::sqrt(vec[0] * vec[0] + vec[1] * vec[1] + vec[2] * vec[2]);
  if (len > 0) len = 3 * move_size / len;  // ion step of 3 move sizes (molecule.cc:108-113)
  bds[0].SetMoved();
  for (int i = 0; i < 3; i++) bds[0].SetCrd(1, i, bds[0].GetCrd(0, i) + len * vec[i]);
}

void Molecule::COMTranslate(double move_size, std::mt19937& g) {
  double vec[3];
  for (int i = 0; i < 3; i++) vec[i] = 0.5 * move_size * (double)g() / kMax;
  for (int i = 0; i < 3; i++)
    if (g() % 2 == 0) vec[i] = -vec[i];
  for (auto& b : bds) {
    for (int j = 0; j < 3; j++) b.SetCrd(1, j, b.GetCrd(0, j) + vec[j]);
    b.SetMoved();
  }
}

void Molecule::Pivot(double move_size, std::mt19937& g, double eq, bool vary) {
  const int len = Size();
  int pivot = (int)std::floor(len * (double)g() / kMax);
  if (pivot == len) pivot--;
  const double s = move_size * (double)g() / kMax;
  // Each bead is displaced by s * randSphere, put back at a bond length from
  // its (already moved) neighbour toward the pivot, and the rest of that side
  // follows by the same translation.
  for (int dir = 0; dir < 2; dir++) {
    const int step = dir == 0 ? 1 : -1;
    for (int i = pivot + step; i >= 0 && i < len; i += step) {
      double vec[3];
      rand_sphere(vec, g);
      const Bead& prev = bds[i - step];
      double d[3];
      for (int a = 0; a < 3; a++) d[a] = (bds[i].GetCrd(1, a) + s * vec[a]) - prev.GetCrd(1, a);
      double bl = eq;
      if (vary) bl += (eq / 5.0) * ((double)g() / kMax - 0.5);
      const double norm = bl / std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
      double m[3];
      for (int a = 0; a < 3; a++) m[a] = (norm * d[a] + prev.GetCrd(1, a)) - bds[i].GetCrd(1, a);
      for (int j = i; j >= 0 && j < len; j += step)
        for (int a = 0; a < 3; a++) bds[j].SetCrd(1, a, bds[j].GetCrd(1, a) + m[a]);
    }
  }
  for (auto& b : bds) b.SetMoved();
}

void Molecule::Crankshaft(double move_size, std::mt19937& g) {
  const int len = Size();
  int first = (int)std::floor((len - 2) * (double)g() / kMax);
  int last = (int)std::floor((len - first) * (double)g() / kMax) + first;
  if (last > len - 1) last = len - 1;  // the reference reads past the chain here
  double ax[3];
  for (int i = 0; i < 3; i++) ax[i] = bds[last].GetCrd(0, i) - bds[first].GetCrd(0, i);
  double z = ax[0] * ax[0] + ax[1] * ax[1] + ax[2] * ax[2];
  if (z > 0)
    for (int i = 0; i < 3; i++) ax[i] /= std::sqrt(z);
  const double pi = 3.14159265358979323846;
  const double angle = move_size * ((double)g() / kMax * 2 * pi - pi);
  // Rodrigues rotation about the first->last axis.
  const double sn = std::sin(angle), cs = std::cos(angle);
  double R[3][3];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) R[i][j] = (1.0 - cs) * ax[i] * ax[j] + (i == j ? cs : 0.0);
  R[0][1] -= sn * ax[2];
  R[1][0] += sn * ax[2];
  R[0][2] += sn * ax[1];
  R[2][0] -= sn * ax[1];
  R[1][2] -= sn * ax[0];
  R[2][1] += sn * ax[0];
  for (int i = first + 1; i < last; i++) {
    bds[i].SetMoved();
    double v[3];
    for (int k = 0; k < 3; k++) v[k] = bds[i].GetCrd(0, k) - bds[first].GetCrd(0, k);
    for (int k = 0; k < 3; k++)
      bds[i].SetCrd(1, k, (R[k][0] * v[0] + R[k][1] * v[1]) + R[k][2] * v[2] +
                              bds[first].GetCrd(0, k));
  }
}

void Molecule::RandomReptation(std::mt19937& g, double eq, bool vary) {
  if (eq < 0) throw InputError("reptation needs a rigid bond length");
  double bl = eq;
  if (vary) bl += (eq / 5.0) * ((double)g() / kMax - 0.5);
  const int len = Size();
  int dir = 1, begin = 0, end = len - 1;
  if (g() % 2 == 0) {
    dir = -1;
    begin = len - 1;
    end = 0;
  }
  for (int i = begin; i != end; i += dir)
    for (int j = 0; j < 3; j++) bds[i].SetCrd(1, j, bds[i + dir].GetCrd(0, j));
  double vec[3];
  rand_sphere(vec, g);
  const double vl = std::sqrt(vec[0] * vec[0] + vec[1] * vec[1] + vec[2] * vec[2]);
  for (int i = 0; i < 3; i++) bds[end].SetCrd(1, i, bds[end].GetCrd(0, i) + bl * vec[i] / vl);
  for (auto& b : bds) b.SetMoved();
}

// ------------------------------------------------------------ ForceField
ForceField::~ForceField() {
  if (ctx_) plum_ctx_destroy(ctx_);
}

void ForceField::Initialize(const std::string& dir, const std::string& runin_text,
                            std::vector<Molecule>& mols, int form, int device) {
  if (ctx_) plum_ctx_destroy(ctx_);
  ctx_ = nullptr;
  check(plum_ctx_create_text(dir.c_str(), runin_text.c_str(), form, device, &ctx_));
  check(plum_ctx_info(ctx_, &info_));
  check(plum_run_params(ctx_, &run_));
  const int nb = info_.n_bead, nm = info_.n_mol;
  mol_start_.assign(nm + 1, 0);
  std::vector<double> q(nb), xyz(3 * (size_t)nb);
  std::vector<int> type(nb);
  check(plum_get_topology(ctx_, mol_start_.data(), q.data(), type.data()));
  check(plum_get_positions(ctx_, xyz.data()));
  std::vector<std::string> names(info_.n_type);
  for (int t = 0; t < info_.n_type; t++) {
    char buf[64];
    check(plum_type_name(ctx_, t, buf, sizeof buf));
    names[t] = buf;
  }
  type_names_ = names;
  if (run_.use_gc) check(plum_gc_info(ctx_, gc_));
  mols.assign(nm, Molecule());
  int id = 0;
  for (int m = 0; m < nm; m++)
    for (int i = mol_start_[m]; i < mol_start_[m + 1]; i++) {
      Bead b(names[type[i]], id++, m, q[i], xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
      b.SetType(type[i]);
      mols[m].AddBead(b);
    }
}

void ForceField::InitializeEnergy(std::vector<Molecule>& mols) {
  (void)mols;
  double out[8];
  check(plum_total_energy(ctx_, out));
}

double ForceField::EnergyDifference(std::vector<Molecule>& mols, int mol) {
  const Molecule& M = mols[mol];
  std::vector<double> trial(3 * (size_t)M.Size());
  std::vector<int> moved(M.Size());
  for (int i = 0; i < M.Size(); i++) {
    for (int a = 0; a < 3; a++) trial[3 * i + a] = M.bds[i].GetCrd(1, a);
    moved[i] = M.bds[i].GetMoved();
  }
  double out[5];
  check(plum_delta_energy(ctx_, mol, trial.data(), moved.data(), out));
  return out[0];
}

void ForceField::FinalizeEnergies(std::vector<Molecule>& mols, bool accept, int mol) {
  (void)mols;
  (void)mol;
  check(plum_finalize(ctx_, accept ? 1 : 0));
}

static double term(plum_ctx* c, int k) {
  double e[4];
  check(plum_energies(c, e));
  return e[k];
}
double ForceField::TotPairEnergy() { return term(ctx_, 0); }
double ForceField::TotEwaldEnergy() { return term(ctx_, 1); }
double ForceField::TotBondEnergy() { return term(ctx_, 2); }
double ForceField::TotExtEnergy() { return term(ctx_, 3); }

// ------------------------------------------------- grand-canonical exchange
double ForceField::Gasdev(double mean, double sd, std::mt19937& g) {
  if (gd_iset_ == 0) {
    double v1, v2, rsq;
    do {
      v1 = 2.0 * ((double)g() / kMax) - 1.0;
      v2 = 2.0 * ((double)g() / kMax) - 1.0;
      rsq = v1 * v1 + v2 * v2;
    } while (rsq >= 1.0 || rsq == 0.0);
    const double fac = std::sqrt(-2.0 * std::log(rsq) / rsq);
    gd_gset_ = v1 * fac;
    gd_iset_ = 1;
    return v2 * fac * sd + mean;
  }
  gd_iset_ = 0;
  return gd_gset_ * sd + mean;
}

double ForceField::RandomBondLen(std::mt19937& g) {
  const double k = gc_[6], r0 = gc_[7];
  const double sigma = std::sqrt(1 / (run_.beta * k));
  const double a = (r0 + 3 * sigma) * (r0 + 3 * sigma);
  double len = 0;
  bool ready = false;
  while (!ready) {
    len = Gasdev(r0, sigma, g);
    ready = ((double)g() / kMax < (len * len / a));
  }
  return len;
}

void ForceField::GCCounts(const std::vector<Molecule>& mols, int* spc1, int* spc2) const {
  // ForceField::UpdateMolCounts (force_field.cc:1258-1277): neutral single
  // beads count with the cations
  int nc = 0, ncat = 0, nan = 0;
  for (int m = run_.phantom; m < (int)mols.size(); m++) {
    if (mols[m].Size() > 1)
      nc++;
    else if (mols[m].bds[0].Charge() >= 0)
      ncat++;
    else
      nan++;
  }
  nc -= run_.grafted;
  const double qb = gc_[2];
  if (GCChainLen() > 1)
    *spc1 = nc;
  else if (qb >= 0)
    *spc1 = ncat - run_.coion;
  else
    *spc1 = nan - run_.coion;
  *spc2 = qb == 0 ? 0 : (qb > 0 ? nan : ncat);
}

// CBMCFGenTrialBeads (cbmc.cc:161-212): every trial's draws (bond length,
// direction, the counterion's position) in the reference's order, then all
// trials' energies in one device call. replace_first (deletion) stands for
// trial 0 in the energies, as cbmc.cc:386-388 overwrites its weight.
double ForceField::CBMCFGenTrialBeads(const double* end, int cl, std::mt19937& g, int delete_id,
                                      const double* replace_first) {
  const int T = (int)gc_[4], L = GCChainLen();
  const bool charged = gc_[2] != 0;
  tb1_.assign(3 * (size_t)T, 0.0);
  tb2_.assign(3 * (size_t)T, 0.0);
  w_.assign(T, 0.0);
  u_.assign(T, 0.0);
  for (int i = 0; i < T; i++) {
    double bl = 0;
    if (run_.use_bond)
      bl = RandomBondLen(g);
    else if (run_.use_bond_rigid)
      bl = run_.rigid_bond;
    double v[3];
    rand_sphere(v, g);
    for (int a = 0; a < 3; a++) tb1_[3 * i + a] = v[a] * bl + end[a];
    if (charged)
      for (int a = 0; a < 3; a++) tb2_[3 * i + a] = (double)g() / kMax * info_.box[a];
  }
  if (replace_first)
    for (int a = 0; a < 3; a++) {
      tb1_[a] = replace_first[a];
      tb2_[a] = replace_first[3 + a];
    }
  check(plum_cbmc_trials(ctx_, T, tb1_.data(), charged ? tb2_.data() : nullptr, cl,
                         cl > 0 ? chain_.data() : nullptr,
                         (charged && cl > 0) ? chain_.data() + 3 * L : nullptr, delete_id,
                         u_.data()));
  double Wi = 0;
  for (int i = 0; i < T; i++) {
    w_[i] = std::exp(-run_.beta * u_[i]);
    Wi += w_[i];
  }
  return Wi;
}

bool ForceField::CBMCFChainInsertion(std::vector<Molecule>& mols, std::mt19937& g) {
  const int L = GCChainLen(), T = (int)gc_[4];
  const double qb = gc_[2];
  const bool charged = qb != 0;
  chain_.assign(6 * (size_t)L, 0.0);
  double weight = 1.0;
  const int i_index = charged ? L : 0, initial = charged ? 2 : 1;
  for (int i = 0; i < initial; i++)
    for (int a = 0; a < 3; a++) chain_[3 * (i * L) + a] = (double)g() / kMax * info_.box[a];
  double u0 = 0;
  check(plum_cbmc_trials(ctx_, 1, chain_.data(), charged ? chain_.data() + 3 * i_index : nullptr,
                         0, nullptr, nullptr, -1, &u0));
  weight *= std::exp(-run_.beta * u0);
  if (weight <= 0) return false;
  for (int i = 1; i < L; i++) {
    const double Wi = CBMCFGenTrialBeads(&chain_[3 * (i - 1)], i, g, -1, nullptr);
    weight *= Wi / T;
    if (weight <= 0) return false;
    const double rn = (double)g() / kMax * Wi;
    int cb = 0;
    double cum = w_[0];
    while (cum < rn && cb < T - 1) cum += w_[++cb];
    for (int a = 0; a < 3; a++) chain_[3 * i + a] = tb1_[3 * cb + a];
    if (charged)
      for (int a = 0; a < 3; a++) chain_[3 * (i + L) + a] = tb2_[3 * cb + a];
  }
  int spc1, spc2;
  GCCounts(mols, &spc1, &spc2);
  const int spc2_add = charged ? L : 0;
  double factorial = 1;
  for (int i = spc1 + 1; i <= spc1 + 1; i++) factorial *= i;
  for (int i = spc2 + 1; i <= spc2 + spc2_add; i++) factorial *= i;
  const double vol = info_.box[0] * info_.box[1] * info_.box[2], deb = gc_[1];
  double vol_over_lam = 1;
  vol_over_lam *= std::pow(vol / (deb / std::pow((double)L, 1.5)), 1);
  vol_over_lam *= std::pow(vol / (deb / std::pow(1.0, 1.5)), spc2_add);
  const double C = vol_over_lam * (1.0 / factorial);
  const double rn = (double)g() / kMax;
  if (!(rn < (std::exp(run_.beta * gc_[0]) * weight) * C)) return false;
  const std::string& sym = type_names_[(int)gc_[8]];
  Molecule chain;
  for (int i = 0; i < L; i++) {
    Bead b(sym, -1, (int)mols.size(), qb, chain_[3 * i], chain_[3 * i + 1], chain_[3 * i + 2]);
    b.SetType((int)gc_[8]);
    chain.AddBead(b);
  }
  for (int i = 0; i + 1 < L; i++) chain.AddBond(i, i + 1);
  mols.push_back(chain);
  if (charged)
    for (int i = 0; i < L; i++) {
      Molecule ion;
      Bead b(sym, -1, (int)mols.size(), -qb, chain_[3 * (i + L)], chain_[3 * (i + L) + 1],
             chain_[3 * (i + L) + 2]);
      b.SetType((int)gc_[8]);
      ion.AddBead(b);
      mols.push_back(ion);
    }
  return true;
}

double ForceField::CalcChemicalPotentialF(std::vector<Molecule>& mols, std::mt19937& g) {
  if (!UseGC()) throw InputError("the chemical potential needs the grand-canonical block");
  const int L = GCChainLen(), T = (int)gc_[4], n_ins = 50;  // mu_tot_ins (force_field.cc:236)
  const double qb = gc_[2];
  const bool charged = qb != 0;
  int spc1, spc2;
  GCCounts(mols, &spc1, &spc2);
  const int spc2_add = charged ? L : 0;
  double factorial = 1;
  for (int i = spc1 + 1; i <= spc1 + 1; i++) factorial *= i;
  for (int i = spc2 + 1; i <= spc2 + spc2_add; i++) factorial *= i;
  // the reference's volume here is divided by 15.625 (cbmc.cc:465-466)
  const double vol = info_.box[0] * info_.box[1] * info_.box[2], deb = gc_[1];
  double vol_over_lam = 1;
  vol_over_lam *= std::pow(vol / 15.625 / (deb / std::pow((double)L, 1.5)), 1);
  vol_over_lam *= std::pow(vol / 15.625 / (deb / std::pow(1.0, 1.5)), spc2_add);
  const double C = vol_over_lam * (1.0 / factorial);
  chain_.assign(6 * (size_t)L, 0.0);
  double total = 0;
  for (int n = 0; n < n_ins; n++) {
    double weight = 1.0;
    const int i_index = charged ? L : 0, initial = charged ? 2 : 1;
    for (int i = 0; i < initial; i++)
      for (int a = 0; a < 3; a++) chain_[3 * (i * L) + a] = (double)g() / kMax * info_.box[a];
    double u0 = 0;
    check(plum_cbmc_trials(ctx_, 1, chain_.data(), charged ? chain_.data() + 3 * i_index : nullptr,
                           0, nullptr, nullptr, -1, &u0));
    if (u0 == kVeryLargeEnergy)
      weight *= 0;
    else
      weight *= std::exp(-run_.beta * u0);
    for (int i = 1; i < L; i++) {
      // the trial beads are drawn before the weight is tested (cbmc.cc:495-497)
      const double Wi = CBMCFGenTrialBeads(&chain_[3 * (i - 1)], i, g, -1, nullptr);
      weight *= Wi / T;
      if (weight <= 0) break;
      const double rn = (double)g() / kMax * Wi;
      int cb = 0;
      double cum = w_[0];
      while (cum < rn && cb < T - 1) cum += w_[++cb];
      for (int a = 0; a < 3; a++) chain_[3 * i + a] = tb1_[3 * cb + a];
      if (charged)
        for (int a = 0; a < 3; a++) chain_[3 * (i + L) + a] = tb2_[3 * cb + a];
    }
    total += weight * C;
  }
  return total / (double)n_ins;
}

void ForceField::CalcPressureForceLJELSlit(std::vector<Molecule>& /*mols*/) {
  double d[6];
  check(plum_pressure_slit(ctx_, d));
  vp_z += 1;
  double* p = p_tensor;
  p[6] += d[0];
  p[7] += d[1];
  p[9] += d[3];
  p[10] += d[4];
  // the walls are fixed: their mutual force counts once (pressure.cc:438, 451)
  if (vp_z == 1) {
    p[8] += d[2];
    p[11] += d[5];
  }
  const double area = info_.box[0] * info_.box[1];
  if (vp_z == 1) {
    p[2] = p[8] / area;
    p[5] = p[11] / area;
  }
  p[0] = p[6] / (vp_z * area);
  p[1] = p[7] / (vp_z * area);
  p[3] = p[9] / (vp_z * area);
  p[4] = p[10] / (vp_z * area);
}

std::string ForceField::GetPressure() const {
  std::ostringstream foo;
  if (run_.use_ext)
    foo << p_tensor[0] << " " << p_tensor[1] << " " << p_tensor[2] << " " << p_tensor[3] << " "
        << p_tensor[4] << " " << p_tensor[5];
  else
    foo << "nan";
  return foo.str();
}

int ForceField::CBMCFChainDeletion(std::vector<Molecule>& mols, std::mt19937& g) {
  const int L = GCChainLen();
  const double qb = gc_[2];
  const bool charged = qb != 0;
  int spc1, spc2;
  GCCounts(mols, &spc1, &spc2);
  int did = (int)std::floor((double)g() / kMax * spc1);
  if (did >= spc1) did = spc1 - 1;
  // nothing of the species to delete (the reference would index outside it)
  if (did < 0) return -1;
  did = run_.phantom + run_.coion + run_.grafted + run_.grafted_counterion +
        (charged ? did * (1 + L) : did);
  const int second = charged ? did + 1 : did;
  if (second >= (int)mols.size() || mols[did].Size() < L) return -1;
  chain_.assign(6 * (size_t)L, 0.0);
  for (int a = 0; a < 3; a++) {
    chain_[a] = mols[did].bds[0].GetCrd(0, a);
    if (charged) chain_[3 * L + a] = mols[second].bds[0].GetCrd(0, a);
  }
  double u0 = 0;
  check(plum_cbmc_trials(ctx_, 1, chain_.data(), charged ? chain_.data() + 3 * L : nullptr, 0,
                         nullptr, nullptr, did, &u0));
  double weight = std::exp(-run_.beta * u0);
  for (int i = 1; i < L; i++) {
    for (int a = 0; a < 3; a++) {
      chain_[3 * i + a] = mols[did].bds[i].GetCrd(0, a);
      if (charged) chain_[3 * (i + L) + a] = mols[did + i + 1].bds[0].GetCrd(0, a);
    }
    double rep[6];
    for (int a = 0; a < 3; a++) {
      rep[a] = chain_[3 * i + a];
      rep[3 + a] = charged ? chain_[3 * (i + L) + a] : chain_[3 * i + a];
    }
    const double Wi = CBMCFGenTrialBeads(&chain_[3 * (i - 1)], i, g, did, rep);
    weight *= Wi / (int)gc_[4];
  }
  const int spc2_del = charged ? L : 0;
  double factorial = 1;
  for (int i = spc1; i > spc1 - 1; i--) factorial *= i;
  for (int i = spc2; i > spc2 - spc2_del; i--) factorial *= i;
  const double vol = info_.box[0] * info_.box[1] * info_.box[2], deb = gc_[1];
  double lam_over_vol = 1;
  lam_over_vol *= std::pow((deb / std::pow((double)L, 1.5)) / vol, 1);
  lam_over_vol *= std::pow((deb / std::pow(1.0, 1.5)) / vol, spc2_del);
  const double C = lam_over_vol * factorial;
  const double rn = (double)g() / kMax;
  if (rn < C / (std::exp(run_.beta * gc_[0]) * weight)) return did;
  return -1;
}

void ForceField::EnergyInitForAddedMolecule(std::vector<Molecule>& mols, int n_added) {
  std::vector<int> sizes;
  std::vector<double> xyz, q;
  std::vector<int> type;
  for (int m = (int)mols.size() - n_added; m < (int)mols.size(); m++) {
    sizes.push_back(mols[m].Size());
    for (const Bead& b : mols[m].bds) {
      for (int a = 0; a < 3; a++) xyz.push_back(b.GetCrd(0, a));
      q.push_back(b.Charge());
      type.push_back(b.Type());
    }
  }
  check(plum_append_molecules(ctx_, n_added, sizes.data(), xyz.data(), q.data(), type.data()));
  for (int sz : sizes) mol_start_.push_back(mol_start_.back() + sz);
  check(plum_ctx_info(ctx_, &info_));
}

void ForceField::AdjustEnergyUponMolDeletion(int first, int count) {
  check(plum_erase_molecules(ctx_, first, count));
  const int nb = mol_start_[first + count] - mol_start_[first];
  mol_start_.erase(mol_start_.begin() + first + 1, mol_start_.begin() + first + count + 1);
  for (size_t m = first + 1; m < mol_start_.size(); m++) mol_start_[m] -= nb;
  check(plum_ctx_info(ctx_, &info_));
}

double ForceField::EqBondLen() const {
  if (!run_.use_bond) throw InputError("Illegal request of bond length");
  return run_.eq_bond;
}

// ------------------------------------------------------------ Simulation
Simulation::Simulation(std::istream& runin, const std::string& dir, unsigned seed, int form,
                       int device) {
  std::string text((std::istreambuf_iterator<char>(runin)), std::istreambuf_iterator<char>());
  force_field.Initialize(dir, text, mols, form, device);
  run_ = force_field.RunInfo();
  const plum_info& info = force_field.Info();
  for (int a = 0; a < 3; a++) box_l[a] = info.box[a];
  npbc = info.npbc;
  rand_gen.seed(seed);
  // rho(z) accumulator: ceil(Lz / 0.02) bins x {chain, q >= 0 ion, q < 0 ion}
  // (simulation.cc:112-117)
  density_z_cumu.assign(3 * (size_t)std::ceil(box_l[2] / 0.02), 0.0);
  UpdateMolCounts();
}

void Simulation::UpdateMolCounts() {
  n_mol = (int)mols.size();
  n_chain = n_chain_b = n_cion = n_aion = n_nion = 0;
  n_bead_ = run_.phantom;  // each phantom molecule counted as one bead
  for (int i = run_.phantom; i < n_mol; i++) {
    n_bead_ += mols[i].Size();
    if (mols[i].Size() > 1) {
      n_chain++;
      n_chain_b += mols[i].Size();
    } else if (mols[i].bds[0].Charge() > 0)
      n_cion++;
    else if (mols[i].bds[0].Charge() < 0)
      n_aion++;
    else
      n_nion++;
  }
  n_chain -= run_.grafted;
}

void Simulation::TranslationalMove() {
  last_move_type = -1;
  last_accept = 0;
  if (n_mol - run_.phantom <= 0) return;
  const int n_ch = run_.grafted + n_chain, n_io = n_cion + n_aion + n_nion;
  int chain_id = -1, ion_id = -1, mol_id = -1;
  int which_chain = (int)std::floor((double)rand_gen() / kMax * n_ch);
  int which_ion = (int)std::floor((double)rand_gen() / kMax * n_io);
  if (which_chain == n_ch) which_chain--;
  if (which_ion == n_io) which_ion--;
  int cc = -1, ic = -1;
  for (int i = run_.phantom; i < n_mol; i++) {
    if (mols[i].Size() > 1)
      cc++;
    else
      ic++;
    if (cc == which_chain) {
      chain_id = i;
      which_chain = -2;
    }
    if (ic == which_ion) {
      ion_id = i;
      which_ion = -2;
    }
  }
  int move_type = 0;
  const double u = (double)rand_gen() / kMax;
  double cur = run_.move_prob[0];
  while (cur < u && move_type < 4) cur += run_.move_prob[++move_type];
  if (cur < u) move_type++;
  if (move_type > 4) move_type = 4;
  if (move_type == 0 && n_io > 0) {
    mol_id = ion_id;
    mols[mol_id].BeadTranslate(run_.move_size, box_l, rand_gen);
  } else if (n_ch > 0) {
    mol_id = chain_id;
    double bond_len = 0;
    bool vary = false;
    if (force_field.UseBondRigid()) bond_len = force_field.RigidBondLen();
    if (force_field.UseBondPot()) {
      bond_len = force_field.EqBondLen();
      vary = true;
    }
    switch (move_type) {
      case 1: mols[mol_id].COMTranslate(run_.move_size, rand_gen); break;
      case 2: mols[mol_id].Pivot(run_.move_size, rand_gen, bond_len, vary); break;
      case 3: mols[mol_id].Crankshaft(run_.move_size, rand_gen); break;
      case 4: mols[mol_id].RandomReptation(rand_gen, bond_len, vary); break;
    }
  }
  if (!((move_type == 0 && n_io > 0) || (move_type > 0 && n_ch > 0))) return;
  attempted[move_type]++;
  const double dE = force_field.EnergyDifference(mols, mol_id);
  bool accept = false;
  if (!(dE >= kVeryLargeEnergy)) accept = (double)rand_gen() / kMax < std::exp(-run_.beta * dE);
  force_field.FinalizeEnergies(mols, accept, mol_id);
  for (auto& b : mols[mol_id].bds) {
    if (accept)
      b.UpdateCurrentPos();
    else
      b.UpdateTrialPos();
    b.UnsetMoved();
  }
  if (accept) accepted[move_type]++;
  last_move_type = move_type;
  last_accept = accept;
}

void Simulation::GCMove() {
  const bool insert = rand_gen() % 2;
  last_move_type = insert ? 5 : 6;
  last_accept = 0;
  if (insert) {
    if (step > run_.steps_eq) insertion_attempted++;
    const int before = (int)mols.size();
    if (force_field.CBMCFChainInsertion(mols, rand_gen)) {
      if (step > run_.steps_eq) insertion_accepted++;
      force_field.EnergyInitForAddedMolecule(mols, (int)mols.size() - before);
      last_accept = 1;
    }
  } else {
    if (step > run_.steps_eq) deletion_attempted++;
    int deleted = -1;
    if (n_mol - run_.phantom - run_.coion > 0) deleted = force_field.CBMCFChainDeletion(mols, rand_gen);
    if (deleted >= run_.phantom + run_.coion) {
      if (step > run_.steps_eq) deletion_accepted++;
      int ions = 0;
      for (const Bead& b : mols[deleted].bds) ions += (int)std::round(std::fabs(b.Charge()));
      force_field.AdjustEnergyUponMolDeletion(deleted, 1 + ions);
      mols.erase(mols.begin() + deleted, mols.begin() + deleted + 1 + ions);
      last_accept = 1;
    }
  }
  UpdateMolCounts();
}

void Simulation::Step() {
  step++;
  // simulation.cc:221-226: int rand_num = rand_gen(); exchange when
  // rand_num % gc_freq == 0, with the reference's signed remainder
  const int32_t rand_num = (int32_t)rand_gen();
  if (force_field.UseGC() && force_field.GCFrequency() > 0 &&
      rand_num % force_field.GCFrequency() == 0)
    GCMove();
  else
    TranslationalMove();
}

void Simulation::RunSteps(long n) {
  if (force_field.UseGC()) {
    // exchanges need host control flow; every step runs here
    for (long i = 0; i < n; i++) Step();
    return;
  }
  int max_len = 1;
  for (auto& m : mols) max_len = std::max(max_len, m.Size());
  while (n > 0) {
    const int chunk = (int)std::min<long>(n, 4096);
    // The device consumes the same mt19937 words rand_gen would produce; the
    // generator is then advanced by exactly the words used. Budget: a pivot
    // takes 2 + len (2 r + 1) draws with r rejected pairs (mean 1.27).
    std::mt19937 g0 = rand_gen;
    const long words = (long)chunk * (16 + 6L * max_len) + 65536L;
    std::vector<uint32_t> stream(words);
    for (long i = 0; i < words; i++) stream[i] = rand_gen();
    long used = 0;
    std::vector<int> mt(chunk), ac(chunk);
    check(plum_run_moves(force_field.Context(), stream.data(), words, chunk, mt.data(),
                         ac.data(), nullptr, &used));
    rand_gen = g0;
    rand_gen.discard((unsigned long long)used);
    // attempted / accepted per move type (simulation.cc:319, 341)
    for (int i = 0; i < chunk; i++)
      if (mt[i] >= 0 && mt[i] < 5) {
        attempted[mt[i]]++;
        if (ac[i]) accepted[mt[i]]++;
      }
    step += chunk;
    n -= chunk;
  }
  SyncFromDevice();
}

void Simulation::Run() {
  UpdateMolCounts();
  for (long s = 0; s < run_.steps;) {
    // run on the device up to the next step where the reference samples or
    // writes (its loop checks every step, simulation.cc:219-237)
    long n = run_.steps - s;
    auto upto = [&](long f) {
      if (f > 0) n = std::min(n, f - (step % f));
    };
    upto(run_.sample_freq);
    if (out_on_) {
      upto(run_.stat_out_freq);
      upto(run_.traj_out_freq);
    }
    RunSteps(n);
    s += n;
    Sample();
    PrintStat();
    PrintTraj();
    PrintLastCrd();
    PrintLastTop();
    PrintLastRhoZ();
  }
}

void Simulation::SyncFromDevice() {
  const int nb = force_field.Info().n_bead;
  std::vector<double> xyz(3 * (size_t)nb);
  check(plum_get_positions(force_field.Context(), xyz.data()));
  int k = 0;
  for (auto& m : mols)
    for (auto& b : m.bds) {
      double p[3] = {xyz[3 * k], xyz[3 * k + 1], xyz[3 * k + 2]};
      b.SetAllCrd(p);
      k++;
    }
}

void Simulation::Sample() {
  if (!(step > run_.steps_eq && run_.sample_freq > 0 && step % run_.sample_freq == 0)) return;
  ff_avg_counter++;
  double e[4];
  check(plum_energies(force_field.Context(), e));
  if (run_.use_pair) pair_e_cumu += e[0];
  if (run_.use_ewald) ewald_e_cumu += e[1];
  if (run_.use_bond) bond_e_cumu += e[2];
  if (run_.use_ext) ext_e_cumu += e[3];
  density_cumu += (double)mols.size() / (box_l[0] * box_l[1] * box_l[2]);
  // CalcRhoZ (simulation.cc:1029-1045): one sample added to the accumulator
  int bins = 0;
  check(plum_rhoz(force_field.Context(), nullptr, 0, &bins));
  std::vector<double> rz(3 * (size_t)bins);
  check(plum_rhoz(force_field.Context(), rz.data(), (int)rz.size(), nullptr));
  for (size_t k = 0; k < rz.size() && k < density_z_cumu.size(); k++) density_z_cumu[k] += rz[k];
  // pressure every 10 samples (simulation.cc:756-761)
  if (run_.use_ext && step % (run_.sample_freq * 10) == 0)
    force_field.CalcPressureForceLJELSlit(mols);
  if (run_.calc_chem_pot) chem_pot_cumu += force_field.CalcChemicalPotentialF(mols, rand_gen);
  if (mols.empty()) return;
  mol_avg_counter++;
  double o[5];
  check(plum_observables(force_field.Context(), o));
  rg_tot_cumu += o[0];
  // RadiusOfGyrationXYZ returns its three values through an ostringstream
  // with the default six significant digits (simulation.cc:476-478), and
  // Sample reads them back from that string
  std::ostringstream foo;
  foo << o[1] << " " << o[2] << " " << o[3];
  std::istringstream iss(foo.str());
  double x = 0, y = 0, z = 0;
  iss >> x >> y >> z;
  rg_x_cumu += x;
  rg_y_cumu += y;
  rg_z_cumu += z;
  e_to_e_cumu += o[4];
}

double Simulation::RadiusOfGyration() {
  double o[5];
  check(plum_observables(force_field.Context(), o));
  return o[0];
}

double Simulation::EndToEndDistance() {
  double o[5];
  check(plum_observables(force_field.Context(), o));
  return o[4];
}

}  // namespace plum

// ---------------------------------------------------------------- C driver
// Drives the host classes from a C caller (used by the tests and the CLI).
extern "C" {

struct plum_sim {
  plum::Simulation* s;
};

int plum_sim_create(const char* dir, const char* runin_text, unsigned seed, int form,
                    plum_sim** out) {
  try {
    std::istringstream is(runin_text);
    *out = new plum_sim{new plum::Simulation(is, dir, seed, form, 0)};
    return PLUM_OK;
  } catch (const std::exception& e) {
    *out = nullptr;
    return PLUM_ERR_INPUT;
  }
}

int plum_sim_destroy(plum_sim* s) {
  if (s) {
    delete s->s;
    delete s;
  }
  return PLUM_OK;
}

int plum_sim_translational_moves(plum_sim* s, int n, int* move_type, int* accept) {
  try {
    for (int i = 0; i < n; i++) {
      (void)s->s->rand_gen();  // simulation.cc:221, the grand-canonical check draw
      s->s->TranslationalMove();
      s->s->step++;
      if (move_type) move_type[i] = s->s->last_move_type;
      if (accept) accept[i] = s->s->last_accept;
    }
    return PLUM_OK;
  } catch (const std::exception&) {
    return PLUM_ERR_STATE;
  }
}

int plum_sim_steps(plum_sim* s, int n, int* move_type, int* accept) {
  try {
    for (int i = 0; i < n; i++) {
      s->s->Step();
      if (move_type) move_type[i] = s->s->last_move_type;
      if (accept) accept[i] = s->s->last_accept;
    }
    return PLUM_OK;
  } catch (const std::exception&) {
    return PLUM_ERR_STATE;
  }
}

int plum_sim_n_bead(plum_sim* s) {
  int n = 0;
  for (auto& m : s->s->mols) n += m.Size();
  return n;
}

int plum_sim_enable_output(plum_sim* s, const char* dir) {
  try {
    s->s->EnableOutput(dir ? dir : ".");
    return PLUM_OK;
  } catch (const std::exception&) {
    return PLUM_ERR_INPUT;
  }
}

int plum_sim_write_checkpoint(plum_sim* s, const char* path) {
  try {
    s->s->WriteCheckpoint(path ? path : "");
    return PLUM_OK;
  } catch (const std::exception&) {
    return PLUM_ERR_INPUT;
  }
}

int plum_sim_read_checkpoint(plum_sim* s, const char* path) {
  try {
    s->s->ReadCheckpoint(path ? path : "");
    return PLUM_OK;
  } catch (const std::exception&) {
    return PLUM_ERR_INPUT;
  }
}

int plum_sim_chem_pot(plum_sim* s, double* out) {
  try {
    *out = s->s->force_field.CalcChemicalPotentialF(s->s->mols, s->s->rand_gen);
    return PLUM_OK;
  } catch (const std::exception&) {
    return PLUM_ERR_INPUT;
  }
}

int plum_sim_pressure(plum_sim* s, int eval, double* out13) {
  try {
    if (eval) s->s->force_field.CalcPressureForceLJELSlit(s->s->mols);
    for (int k = 0; k < 12; k++) out13[k] = s->s->force_field.p_tensor[k];
    out13[12] = s->s->force_field.vp_z;
    return PLUM_OK;
  } catch (const std::exception&) {
    return PLUM_ERR_INPUT;
  }
}

int plum_sim_run(plum_sim* s) {
  try {
    s->s->Run();
    return PLUM_OK;
  } catch (const std::exception&) {
    return PLUM_ERR_STATE;
  }
}

int plum_sim_finish(plum_sim* s) {
  try {
    s->s->Finish();
    return PLUM_OK;
  } catch (const std::exception&) {
    return PLUM_ERR_STATE;
  }
}

int plum_sim_run_steps(plum_sim* s, long n) {
  try {
    s->s->RunSteps(n);
    return PLUM_OK;
  } catch (const std::exception&) {
    return PLUM_ERR_STATE;
  }
}

// host-side positions (current), n_bead*3
int plum_sim_positions(plum_sim* s, double* xyz) {
  int k = 0;
  for (auto& m : s->s->mols)
    for (auto& b : m.bds)
      for (int a = 0; a < 3; a++) xyz[k++] = b.GetCrd(0, a);
  return PLUM_OK;
}

int plum_sim_energies(plum_sim* s, double* out) {
  out[0] = s->s->force_field.TotPairEnergy();
  out[1] = s->s->force_field.TotEwaldEnergy();
  out[2] = s->s->force_field.UseBondPot() ? s->s->force_field.TotBondEnergy() : 0.0;
  out[3] = s->s->force_field.UseExtPot() ? s->s->force_field.TotExtEnergy() : 0.0;
  return PLUM_OK;
}

}  // extern "C"
