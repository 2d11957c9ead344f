// Test harness: runs the device's per-item wall-force pressure arithmetic
// (plum_gb300/csrc/slit_pressure.h, compiled here for the host) over the
// oracle's configuration and prints it beside the oracle's
// po_pressure_force_slit, for two evaluations (after n1 steps and after n2
// more).
//
//   slit_pressure_harness <case dir> <seed> <n1> <n2>
//
// Output, one line per evaluation: 6 sums of this code (p_tensor[6..11]
// increments), 6 sums of |term| (the scale of each sum), 6 increments of the
// oracle's accumulators.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "../oracle/plum_oracle.h"
#include "../plum_gb300/csrc/slit_pressure.h"

using namespace plum;

static void eval(po_ctx* c, double* mine, double* scale) {
  double sc[26];
  po_slit_inputs(c, sc, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr);
  const int n_type = (int)sc[22], n_k = (int)sc[23], n_bead = (int)sc[24], n_mol = (int)sc[25];
  if (n_type > kSlitMaxTypes) {
    std::fprintf(stderr, "too many types\n");
    std::exit(2);
  }
  std::vector<double> per(5 * n_type), q(n_bead), kv(3 * (size_t)n_k + 3), kw(n_k + 1);
  std::vector<int> type(n_bead), ms(n_mol + 1);
  std::vector<double> xyz(3 * (size_t)n_bead), xyzq(4 * (size_t)n_bead);
  po_slit_inputs(c, nullptr, per.data(), type.data(), q.data(), ms.data(), kv.data(), kw.data());
  po_coords(c, xyz.data());
  for (int b = 0; b < n_bead; b++) {
    for (int a = 0; a < 3; a++) xyzq[4 * b + a] = xyz[3 * b + a];
    xyzq[4 * b + 3] = q[b];
  }
  SlitPressParams S{};
  S.n_bead = n_bead;
  S.n_mol = n_mol;
  S.phantom = (int)sc[7];
  S.npbc = (int)sc[6];
  S.n_type = n_type;
  S.use_pair = (int)sc[8];
  S.use_ewald = (int)sc[9];
  S.use_ext = (int)sc[10];
  S.pair_kind = (int)sc[11];
  S.ext_kind = (int)sc[12];
  for (int a = 0; a < 3; a++) {
    S.box[a] = sc[a];
    S.ebox[a] = sc[3 + a];
    S.real_cell[a] = (int)sc[17 + a];
  }
  S.lj_cut = sc[13];
  S.lB = sc[14];
  S.alpha = sc[15];
  S.real_cut = sc[16];
  S.evol = sc[20];
  S.wall_cut = sc[21];
  for (int t = 0; t < n_type; t++) {
    S.lj_sig[t] = per[5 * t];
    S.lj_eps[t] = per[5 * t + 1];
    S.wall_sig[t] = per[5 * t + 2];
    S.wall_eps[t] = per[5 * t + 3];
    S.graft[t] = (int)per[5 * t + 4];
  }
  for (int k = 0; k < 6; k++) mine[k] = scale[k] = 0;
  const long long np = slit_pair_items(S, ms.data());
  const long long nw = slit_wall_items(S, ms.data());
  for (long long it = 0; it < np; it++) {
    double a[6] = {0, 0, 0, 0, 0, 0};
    slit_pair_item(S, xyzq.data(), type.data(), ms.data(), it, a);
    for (int k = 0; k < 6; k++) {
      mine[k] += a[k];
      scale[k] += std::fabs(a[k]);
    }
  }
  const int w0 = ms[S.phantom];
  for (long long it = 0; it < nw; it++) {
    double a[2] = {0, 0};
    slit_wall_item(S, xyzq.data(), type.data(), ms.data(), w0 + (int)it, a);
    for (int k = 0; k < 2; k++) {
      mine[k] += a[k];
      scale[k] += std::fabs(a[k]);
    }
  }
  if (S.use_ewald && S.phantom > 0) {
    const double pre = slit_recip_prefactor(S);
    std::vector<int> g(n_bead);
    for (int b = 0; b < n_bead; b++) g[b] = slit_bead_groups(S, ms.data(), b);
    for (int k = 0; k < n_k; k++) {
      double re[5] = {0, 0, 0, 0, 0}, im[5] = {0, 0, 0, 0, 0};
      for (int b = 0; b < n_bead; b++) {
        double ph = 0;
        for (int a = 0; a < 3; a++) ph += kv[3 * k + a] * xyzq[4 * b + a];
        for (int u = 0; u < 5; u++)
          if (g[b] >> u & 1) {
            re[u] += q[b] * std::cos(ph);
            im[u] += q[b] * std::sin(ph);
          }
      }
      double o[3] = {0, 0, 0};
      slit_k_terms(kv[3 * k + 2], kw[k], re, im, o);
      for (int u = 0; u < 3; u++) {
        mine[3 + u] += pre * o[u];
        scale[3 + u] += std::fabs(pre * o[u]);
      }
    }
  }
}

int main(int argc, char** argv) {
  if (argc < 5) {
    std::fprintf(stderr, "usage: %s dir seed n1 n2\n", argv[0]);
    return 2;
  }
  char err[512];
  po_ctx* c = po_create(argv[1], "run.in", (uint32_t)std::atoi(argv[2]), err, sizeof err);
  if (!c) {
    std::fprintf(stderr, "%s\n", err);
    return 1;
  }
  double before[12] = {0}, after[12];
  for (int pass = 0; pass < 2; pass++) {
    const int n = std::atoi(argv[3 + pass]);
    std::vector<int> mt(n + 1), ac(n + 1), dr(n + 1);
    std::vector<double> et(n + 1);
    if (n > 0) po_run(c, n, mt.data(), ac.data(), dr.data(), et.data());
    double mine[6], scale[6];
    eval(c, mine, scale);
    po_pressure_force_slit(c, after);
    for (int k = 0; k < 6; k++) std::printf("%.17g ", mine[k]);
    for (int k = 0; k < 6; k++) std::printf("%.17g ", scale[k]);
    for (int k = 0; k < 6; k++) std::printf("%.17g ", after[6 + k] - before[6 + k]);
    std::printf("\n");
    for (int k = 0; k < 12; k++) before[k] = after[k];
  }
  po_destroy(c);
  return 0;
}
