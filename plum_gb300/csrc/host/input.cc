#include "input.h"

#include <fstream>
#include <sstream>

namespace plum {
namespace {

struct Reader {
  std::istream& is;
  std::string* err;
  bool bad = false;
  const char* file;

  bool fail(const std::string& what) {
    if (!bad) *err = std::string(file) + ": input ended or malformed while reading " + what;
    bad = true;
    return false;
  }
  // One "flag value" item (the flag token is ignored, as in the reference).
  template <class T>
  bool item(T* v, const char* what) {
    std::string flag;
    if (bad || !(is >> flag) || !(is >> *v)) return fail(what);
    return true;
  }
  bool word(std::string* v, const char* what) {
    if (bad || !(is >> *v)) return fail(what);
    return true;
  }
};

// {flag symbol; flag sigma; flag epsilon}... until the symbol "end".
// {symbol radius}... end
bool read_radii(Reader& r, std::map<std::string, double>* t) {
  for (int guard = 0; guard < 1000000; guard++) {
    std::string sym;
    if (!r.item(&sym, "bead type symbol")) return false;
    if (sym == "end") return true;
    double v = 0;
    if (!r.item(&v, "radius")) return false;
    (*t)[sym] = v;
  }
  return r.fail("a radius table without an 'end' token");
}

bool read_table(Reader& r, std::map<std::string, LJEntry>* t) {
  for (int guard = 0; guard < 1000000; guard++) {
    std::string sym;
    if (!r.item(&sym, "bead type symbol")) return false;
    if (sym == "end") return true;
    LJEntry e;
    if (!r.item(&e.sigma, "sigma") || !r.item(&e.epsilon, "epsilon")) return false;
    (*t)[sym] = e;
  }
  return r.fail("a parameter table without an 'end' token");
}

std::string path_in(const std::string& dir, const std::string& name) {
  if (!name.empty() && name[0] == '/') return name;
  return dir.empty() ? name : dir + "/" + name;
}

}  // namespace

static bool read_stream(const std::string& dir, std::istream& f, Input* in, std::string* err);

bool read_input(const std::string& dir, const std::string& runin, Input* in,
                std::string* err) {
  std::ifstream f(path_in(dir, runin));
  if (!f) {
    *err = "cannot open " + path_in(dir, runin);
    return false;
  }
  return read_stream(dir, f, in, err);
}

bool read_input_text(const std::string& dir, const std::string& text, Input* in,
                     std::string* err) {
  std::istringstream f(text);
  return read_stream(dir, f, in, err);
}

static bool read_stream(const std::string& dir, std::istream& f, Input* in, std::string* err) {
  in->dir = dir;
  Reader r{f, err, false, "run.in"};
  int calc = 0;
  r.item(&in->crd_name, "coordinate file name");
  r.item(&in->top_name, "topology file name");
  r.item(&in->run_name, "run name");
  r.item(&in->steps, "steps");
  r.item(&in->steps_eq, "equilibration steps");
  r.item(&in->sample_freq, "sample frequency");
  r.item(&in->stat_out_freq, "stat frequency");
  r.item(&in->traj_out_freq, "trajectory frequency");
  r.item(&in->npbc, "PBC dimensions");
  r.item(&in->beta, "beta");
  r.item(&in->move_size, "move size");
  r.item(&calc, "calc_chem_pot");
  in->calc_chem_pot = calc;
  r.item(&in->phantom, "surface sites");
  r.item(&in->coion, "coions");
  r.item(&in->grafted, "grafted chains");
  r.item(&in->grafted_counterion, "grafted counterions");
  for (int i = 0; i < 5; i++) r.item(&in->move_prob[i], "move probability");
  r.item(&in->vp_el_res, "virial bin resolution");
  r.item(&in->vp_bead_size, "virial bead size");
  r.item(&in->use_pair, "use_pair");
  r.item(&in->use_ewald, "use_ewald");
  r.item(&in->use_bond, "use_bond");
  r.item(&in->use_rigid, "use_bond_rigid");
  r.item(&in->use_angle, "use_angle");
  r.item(&in->use_dihed, "use_dihed");
  r.item(&in->use_ext, "use_ext");
  r.item(&in->use_gc, "use_gc");
  if (in->use_gc) {
    r.item(&in->chem_pot, "chemical potential");
    r.item(&in->deBroglie, "de Broglie prefactor");
    r.item(&in->gc_freq, "GC frequency");
    r.item(&in->gc_chain_len, "GC chain length");
    r.item(&in->gc_bead_charge, "GC bead charge");
    r.item(&in->gc_symbol, "GC bead symbol");
    r.item(&in->cbmc_trials, "CBMC trials");
  }
  std::string name;
  if (in->use_pair && !r.bad) {
    r.item(&name, "pair potential name");
    if (!r.bad && name == "HardSphere") {
      in->pair_kind = 1;
      read_radii(r, &in->hs_radius);
    } else {
      if (!r.bad && name != "TruncatedLJ") {
        *err = "unsupported pair potential " + name;
        return false;
      }
      r.item(&in->lj_cut, "LJ cutoff");
      read_table(r, &in->lj);
    }
  }
  if (in->use_ewald && !r.bad) {
    r.item(&name, "Ewald potential name");
    if (!r.bad && name != "Coul") {
      *err = "unsupported Ewald potential " + name;
      return false;
    }
    r.item(&in->lB, "Bjerrum length");
    r.item(&in->dielectric, "dielectric constant");
    r.item(&in->alpha, "Ewald alpha");
    r.item(&in->dipole, "dipole correction");
  }
  if (in->use_bond && !r.bad) {
    r.item(&name, "bond potential name");
    if (!r.bad && name != "Spring") {
      *err = "unsupported bond potential " + name;
      return false;
    }
    r.item(&in->k_bond, "spring constant");
    r.item(&in->r0, "spring length");
  }
  if (in->use_rigid && !r.bad) r.item(&in->rigid, "rigid bond length");
  if (in->use_ext && !r.bad) {
    r.item(&name, "external potential name");
    if (!r.bad && name == "HardWall") {
      in->ext_kind = 1;
      read_radii(r, &in->wall_radius);
    } else if (!r.bad && name == "WellWall") {
      in->ext_kind = 2;
      r.item(&in->well_width, "well width");
      r.item(&in->well_depth, "well depth");
      read_radii(r, &in->wall_radius);
    } else {
      if (!r.bad && name != "TruncatedLJWall") {
        *err = "unsupported external potential " + name;
        return false;
      }
      r.item(&in->wall_cut, "wall cutoff");
      r.item(&in->wall_sigma, "wall sigma");
      r.item(&in->wall_eps, "wall epsilon");
      read_table(r, &in->wall);
    }
  }
  if (r.bad) return false;
  for (;;) {
    std::string key, val;
    if (!(f >> key) || !(f >> val)) break;
    if (key == "plum_ewald_real_cutoff") in->x_real_cutoff = std::stod(val);
    if (key == "plum_ewald_kmax") in->x_kmax = std::stoi(val);
    if (key == "plum_ewald_kcut2") {
      in->x_kcut2 = std::stod(val);
      in->x_have_kcut2 = true;
    }
  }

  // Topology (simulation.cc:610-646).
  std::ifstream t(path_in(dir, in->top_name));
  if (!t) {
    *err = "cannot open topology file " + path_in(dir, in->top_name);
    return false;
  }
  Reader rt{t, err, false, "topology"};
  rt.item(&in->n_bead_decl, "bead count");
  rt.item(&in->n_mol, "molecule count");
  for (int a = 0; a < 3; a++) rt.item(&in->box[a], "box length");
  int mol = 0;
  std::string flag;
  rt.item(&mol, "bond list");
  for (int guard = 0; !rt.bad && mol != -1 && guard < 100000000; guard++) {
    int i, j;
    if (!(t >> i >> j)) {
      rt.fail("bond list");
      break;
    }
    in->bonds.push_back({mol, i, j});
    if (!(t >> mol)) rt.fail("bond list");
  }
  if (rt.bad) return false;
  if (in->n_mol <= 0 || in->box[0] <= 0 || in->box[1] <= 0 || in->box[2] <= 0) {
    *err = "topology: molecule count and box lengths must be positive";
    return false;
  }

  // Coordinates (simulation.cc:582-608): two header lines, then rows.
  std::ifstream c(path_in(dir, in->crd_name));
  if (!c) {
    *err = "cannot open coordinate file " + path_in(dir, in->crd_name);
    return false;
  }
  std::string line;
  std::getline(c, line);
  std::getline(c, line);
  std::vector<int> mids;
  std::vector<double> xyz, q;
  std::vector<int> ty;
  std::map<std::string, int> tid;
  int mid;
  std::string sym;
  double x, y, z, ch;
  while (c >> mid >> sym >> x >> y >> z >> ch) {
    if (mid < 0 || mid >= in->n_mol) {
      *err = "coordinates: molecule ID " + std::to_string(mid) + " is out of bounds";
      return false;
    }
    auto it = tid.find(sym);
    int tix;
    if (it == tid.end()) {
      tix = (int)in->type_names.size();
      tid[sym] = tix;
      in->type_names.push_back(sym);
    } else {
      tix = it->second;
    }
    mids.push_back(mid);
    xyz.push_back(x), xyz.push_back(y), xyz.push_back(z);
    q.push_back(ch);
    ty.push_back(tix);
  }
  const int nb = (int)mids.size();
  in->mol_start.assign(in->n_mol + 1, 0);
  for (int i = 0; i < nb; i++) in->mol_start[mids[i] + 1]++;
  for (int m = 0; m < in->n_mol; m++) {
    if (in->mol_start[m + 1] == 0) {
      *err = "coordinates: molecule " + std::to_string(m) + " has no beads";
      return false;
    }
    in->mol_start[m + 1] += in->mol_start[m];
  }
  std::vector<int> fill(in->n_mol, 0);
  in->xyz.assign(3 * (size_t)nb, 0.0);
  in->q.assign(nb, 0.0);
  in->type.assign(nb, 0);
  in->file_order.assign(nb, 0);
  for (int i = 0; i < nb; i++) {
    int k = in->mol_start[mids[i]] + fill[mids[i]]++;
    for (int a = 0; a < 3; a++) in->xyz[3 * k + a] = xyz[3 * i + a];
    in->q[k] = q[i];
    in->type[k] = ty[i];
    in->file_order[k] = i;
  }
  return true;
}

}  // namespace plum
