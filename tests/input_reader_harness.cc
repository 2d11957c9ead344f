// Test harness: reads a case directory with the library's run.in /
// coordinate / topology readers (plum_gb300/csrc/host/input.cc, the host code
// the C ABI builds its device context from) and with the oracle's, and
// compares what both hold: counts, box, switches, potential parameters per
// bead, charges, coordinates and molecule boundaries; then the library's
// Ewald set-up (host/ewald_setup.cc) against the oracle's: Ewald box,
// cut-offs, image and k cells, and the k-set with its weights, exactly.
//
//   input_reader_harness <case dir> [library]
//
// Prints "ok <n_bead> <n_mol> <k vectors checked>" and exits 0 when everything agrees, else
// prints the first difference and exits 1. With "library" only the library's
// reader runs (for malformed inputs, which the reference may read forever).
#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

#include "../oracle/plum_oracle.h"
#include "../plum_gb300/csrc/host/ewald_setup.h"
#include "../plum_gb300/csrc/host/input.h"

static int bad(const char* what, double a, double b) {
  std::printf("differs: %s library %.17g oracle %.17g\n", what, a, b);
  return 1;
}

int main(int argc, char** argv) {
  if (argc < 2) return 2;
  plum::Input in;
  std::string err;
  if (!plum::read_input(argv[1], "run.in", &in, &err)) {
    std::printf("library reader: %s\n", err.c_str());
    return 1;
  }
  if (argc > 2 && std::string(argv[2]) == "library") {
    std::printf("ok %d %d\n", (int)in.q.size(), in.n_mol);
    return 0;
  }
  char oerr[512];
  po_set_fast_init(1);  // the energy totals are not compared here
  po_ctx* c = po_create(argv[1], "run.in", 1, oerr, sizeof oerr);
  if (!c) {
    std::printf("oracle reader: %s\n", oerr);
    return 1;
  }
  const int nb = (int)in.q.size();
  if (nb != po_n_bead(c)) return bad("n_bead", nb, po_n_bead(c));
  if (in.n_mol != po_n_mol(c)) return bad("n_mol", in.n_mol, po_n_mol(c));
  double sc[26];
  po_slit_inputs(c, sc, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr);
  const int n_type = (int)sc[22];
  std::vector<double> per(5 * (size_t)n_type + 5), q(nb), xyz(3 * (size_t)nb);
  std::vector<int> type(nb), ms(in.n_mol + 1);
  po_slit_inputs(c, nullptr, per.data(), type.data(), q.data(), ms.data(), nullptr, nullptr);
  po_coords(c, xyz.data());
  for (int a = 0; a < 3; a++)
    if (in.box[a] != sc[a]) return bad("box", in.box[a], sc[a]);
  const double sw[][2] = {{(double)in.npbc, sc[6]},      {(double)in.phantom, sc[7]},
                          {(double)in.use_pair, sc[8]},  {(double)in.use_ewald, sc[9]},
                          {(double)in.use_ext, sc[10]},  {(double)in.pair_kind, sc[11]},
                          {(double)in.ext_kind, sc[12]}, {in.lj_cut, sc[13]},
                          {in.lB, sc[14]},               {in.alpha, sc[15]},
                          {in.wall_cut, sc[21]}};
  const char* names[] = {"npbc", "phantom", "use_pair", "use_ewald", "use_ext", "pair_kind",
                         "ext_kind", "lj_cut", "lB", "alpha", "wall_cut"};
  for (int k = 0; k < 11; k++)
    if (sw[k][0] != sw[k][1]) return bad(names[k], sw[k][0], sw[k][1]);
  for (int m = 0; m <= in.n_mol; m++)
    if (in.mol_start[m] != ms[m]) return bad("mol_start", in.mol_start[m], ms[m]);
  for (int b = 0; b < nb; b++) {
    if (in.q[b] != q[b]) return bad("charge", in.q[b], q[b]);
    for (int a = 0; a < 3; a++)
      if (in.xyz[3 * b + a] != xyz[3 * b + a]) return bad("coordinate", in.xyz[3 * b + a], xyz[3 * b + a]);
    const std::string& sym = in.type_names[in.type[b]];
    const double* o = per.data() + 5 * type[b];
    auto il = in.lj.find(sym);
    const double ls = il != in.lj.end() ? il->second.sigma : 0.0;
    const double le = il != in.lj.end() ? il->second.epsilon : 0.0;
    auto iw = in.wall.find(sym);
    const double ws = iw != in.wall.end() ? iw->second.sigma : 0.0;
    const double we = iw != in.wall.end() ? iw->second.epsilon : 0.0;
    const double g = sym == "L" ? 1 : (sym == "R" ? 2 : 0);
    if (in.pair_kind == 0 && ls != o[0]) return bad("lj sigma", ls, o[0]);
    if (in.pair_kind == 0 && le != o[1]) return bad("lj epsilon", le, o[1]);
    if (in.use_ext && in.ext_kind == 0 && ws != o[2]) return bad("wall sigma", ws, o[2]);
    if (in.use_ext && in.ext_kind == 0 && we != o[3]) return bad("wall epsilon", we, o[3]);
    if (g != o[4]) return bad("graft", g, o[4]);
  }
  int n_k_checked = 0;
  if (in.use_ewald) {
    plum::EwaldSetup E;
    if (!plum::ewald_setup(in, 1 << 20, &E, &err)) {
      std::printf("library Ewald set-up: %s\n", err.c_str());
      return 1;
    }
    double ei[15];
    po_ewald_info(c, ei);
    if (E.real_cut != ei[0]) return bad("real_cut", E.real_cut, ei[0]);
    if (E.kc2 != ei[1]) return bad("kc2", E.kc2, ei[1]);
    for (int a = 0; a < 3; a++) {
      if (E.real_cell[a] != ei[2 + a]) return bad("real_cell", E.real_cell[a], ei[2 + a]);
      if (E.kcell[a] != ei[5 + a]) return bad("k cells", E.kcell[a], ei[5 + a]);
      if (E.ebox[a] != ei[8 + a]) return bad("Ewald box", E.ebox[a], ei[8 + a]);
    }
    if (E.vol != ei[13]) return bad("Ewald volume", E.vol, ei[13]);
    const int n_k = po_n_kvec(c);
    if ((int)E.kw.size() != n_k) return bad("n_k", (double)E.kw.size(), n_k);
    std::vector<double> kv(3 * (size_t)n_k + 3), kw(n_k + 1);
    po_slit_inputs(c, nullptr, nullptr, nullptr, nullptr, nullptr, kv.data(), kw.data());
    for (int k = 0; k < n_k; k++) {
      for (int a = 0; a < 3; a++) {
        const double kk = E.kn[3 * k + a] * 2 * 3.14159265359 / E.ebox[a];
        if (kk != kv[3 * k + a]) return bad("k vector", kk, kv[3 * k + a]);
      }
      if (E.kw[k] != kw[k]) return bad("k weight", E.kw[k], kw[k]);
    }
    n_k_checked = n_k;
  }
  std::printf("ok %d %d %d\n", nb, in.n_mol, n_k_checked);
  po_destroy(c);
  return 0;
}
