// C ABI of the engine (include/plum_gpu.h): context creation from the
// reference's input files, device buffers, and the host-side orchestration of
// the kernels in kern_energy.cu and kern_moves.cu.
#include <cmath>
#include <cstdio>
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/plum_gpu.h"
#include "engine.h"
#include "slit_pressure.h"
#include "host/ewald_setup.h"
#include "host/input.h"
#include "mlp.h"
#include "surrogate.h"

using namespace plum;

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

}  // namespace

namespace plum {
int fail_msg(int code, const std::string& msg) { return fail(code, msg); }
}  // namespace plum

namespace {

#define CK(call)                                                                 \
  do {                                                                           \
    cudaError_t e_ = (call);                                                     \
    if (e_ != cudaSuccess)                                                       \
      return fail(PLUM_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

constexpr double k216 = 1.12246204831;  // utilities/constants.h:62

}  // namespace

struct plum_ctx {
  Input in;
  DevParams P;
  DevBuffers B;
  int form = PLUM_FORM_FP64;
  int device = 0;
  cudaStream_t s = nullptr;
  std::vector<double4_32a> h_pos;  // host mirror of the current positions
  bool h_pos_valid = true;
  // scratch
  double* d_tot_part = nullptr;
  int n_tot_part = 0;
  double2* d_sk_part = nullptr;
  float4* d_htab = nullptr;      // FP32 h(u) table (precision form)
  double* d_htab64 = nullptr;    // FP64 h(u) table  // [kSkGroupsTotal][n_k] partial S(k) of a recompute
  double* d_out = nullptr;     // small result block
  double* d_obs_per = nullptr;  // [n_mol * 5] per-molecule Rg / Ree sums
  double* d_press = nullptr;    // wall-force pressure partials and sums
  int press_cap = 0;
  unsigned* d_rhoz = nullptr;   // [3 * rhoz_bins] rho(z) counts
  int rhoz_bins = 0;
  // surrogate training data: descriptor accumulator and device copies of
  // P and B for the descriptor kernel
  unsigned* desc_acc = nullptr;
  unsigned* desc_fine = nullptr;
  DevParams* d_rp1 = nullptr;
  DevBuffers* d_rb1 = nullptr;
  double* h_out = nullptr;     // pinned
  uint32_t* d_stream = nullptr;
  long long stream_cap = 0;
  uint32_t* d_mt = nullptr;    // device mt19937 state (625 words)
  long long gen_len = 0;       // valid words in d_stream for plum_run
  int* d_log_type = nullptr;
  int* d_log_acc = nullptr;
  double* d_log_e = nullptr;
  double* d_log_de = nullptr;
  int log_cap = 0;
  bool host_pending = false;
  int max_len = 1;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  double last_ms = 0.0;
  long last_kernels = 0;
  long recompute_every = 0;    // full FP64 recompute cadence of plum_run (0: never)
  long since_recompute = 0;
  // configurational-bias scratch
  double4_32a* cb_b = nullptr;   // [2 * cap] trial beads and counterions
  double4_32a* cb_c = nullptr;   // [2 * cap] grown chain and counterions
  double2* cb_so = nullptr;
  double* cb_part = nullptr;
  double* cb_u = nullptr;
  int cb_cap = 0;
  double* cb_part32 = nullptr;   // slots of the precision form's trial kernel
  long long cb_part32_cap = 0;
  int* cb_ticket = nullptr;      // its last-block counter (zero between launches)
  double drift[4] = {0, 0, 0, 0};  // running minus recomputed at the last reset
  double drift_max = 0.0;
  // CUDA graph of one batch of moves (kernels read the pending move from
  // device state, so one capture replays for every batch of the same size)
  cudaGraphExec_t gexec = nullptr;
  int g_moves = 0;
  DevBuffers g_B;
  bool g_warm = false;
  // per-kernel timing (plum_time_kernels): while set, the step loop runs as
  // plain launches with events around each energy-change (kind 0) and
  // serial (kind 1) launch
  bool kt_on = false;
  std::vector<cudaEvent_t> kt_ev;
  std::vector<int> kt_kind;
};

namespace {

// PotentialEwaldCoul::ReadParameters (potential_ewald_coul.cc:38-115):
// padded z for the dipole correction, real-space cut-off and cells, k^2
// cut-off and cells; then the half-space k-set {k : 0 < k^2 <= kc^2}.
int setup_ewald(plum_ctx* c, std::vector<short4>* kn, std::vector<double>* kw) {
  Input& in = c->in;
  DevParams& P = c->P;
  EwaldSetup E;
  std::string err;
  if (!ewald_setup(in, kMaxKmax, &E, &err)) return fail(PLUM_ERR_INPUT, err);
  const double vol = E.vol;
  for (int a = 0; a < 3; a++) {
    P.ebox[a] = E.ebox[a];
    P.inv_ebox[a] = 1.0 / E.ebox[a];
    P.real_cell[a] = E.real_cell[a];
    P.kmax[a] = E.kcell[a];
    P.kunit[a] = 2 * kPiRef / E.ebox[a];
  }
  P.kper = 0;
  for (int a = 0; a < 3; a++) {
    P.koff[a] = P.kper;
    P.kper += E.kcell[a] + 1;
  }
  const int row = (int)(P.kper * sizeof(double2));
  P.kchunk_delta = std::max(1, std::min(16, kKTableBytes / (2 * row)));
  P.kchunk_sk = std::max(1, std::min(32, kKTableBytes / row));
  const double rc = E.real_cut;
  P.real_cut = rc;
  P.single_image = rc <= 0.5 * E.ebox[0] && rc <= 0.5 * E.ebox[1] && rc <= 0.5 * E.ebox[2];
  P.lB = in.lB;
  P.sqrt_alpha = std::sqrt(in.alpha);
  P.alpha = in.alpha;
  P.kpref = in.lB / (kPiRef * vol) * (4 * kPiRef * kPiRef);
  P.self_coef = -in.lB * std::sqrt(in.alpha / kPiRef);
  P.dip_coef = in.lB * 2 * kPiRef / (vol / 1.0);
  P.dipole = in.dipole;
  kn->clear();
  kw->clear();
  for (size_t k = 0; k < E.kw.size(); k++) {
    kn->push_back(make_short4((short)E.kn[3 * k], (short)E.kn[3 * k + 1], (short)E.kn[3 * k + 2], 0));
    kw->push_back(E.kw[k]);
  }
  P.n_k = (int)kn->size();
  c->in.x_kcut2 = E.kc2;  // effective k^2 cut-off, reported by plum_ctx_info
  return PLUM_OK;
}

template <class T>
int dalloc(T** p, size_t n) {
  if (n == 0) n = 1;
  cudaError_t e = cudaMalloc((void**)p, n * sizeof(T));
  if (e != cudaSuccess) return fail(PLUM_ERR_CUDA, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  return PLUM_OK;
}

// Final fixed-order reductions of the from-scratch energy into out[8] and the
// running state. With drift != null the running totals it replaces are
// compared first: drift[0..3] = running - recomputed per term, drift[4] =
// the largest |total drift| seen (kept across calls), drift[5] += 1.
__global__ void k_assemble_total(const DevParams P, const DevBuffers B, const double* tot_part,
                                 int n_part, const double* misc, double* out, double* drift) {
  __shared__ double red[8];
  double lj = 0.0, re = 0.0, ek = 0.0;
  for (int i = threadIdx.x; i < n_part; i += blockDim.x) {
    lj += tot_part[2 * i];
    re += tot_part[2 * i + 1];
  }
  if (P.use_ewald)
    for (int k = threadIdx.x; k < P.n_k; k += blockDim.x) {
      double2 s = B.sk[k];
      ek += B.kw[k] * (s.x * s.x + s.y * s.y);
    }
  double v[3] = {lj, re, ek};
  double t[3];
  for (int q = 0; q < 3; q++) {
    double x = v[q];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = x;
    __syncthreads();
    double s = 0.0;
    for (int w = 0; w < (int)blockDim.x / 32; w++) s += red[w];
    t[q] = s;
  }
  if (threadIdx.x == 0) {
    DevState* st = B.state;
    double e_pair = P.use_pair ? t[0] : 0.0;
    double real = P.use_ewald ? t[1] + misc[3] : 0.0;
    double recip = P.use_ewald ? P.kpref * t[2] : 0.0;
    double self = P.use_ewald ? misc[2] : 0.0;
    double dip = (P.use_ewald && P.dipole) ? P.dip_coef * misc[4] * misc[4] : 0.0;
    if (drift) {
      const double fresh[4] = {e_pair, real + recip + self + dip, P.use_bond ? misc[0] : 0.0,
                               P.use_ext ? misc[1] : 0.0};
      const double run[4] = {st->e_pair, st->e_ewald, st->e_bond, st->e_ext};
      double tot = 0.0;
      for (int q = 0; q < 4; q++) {
        drift[q] = run[q] - fresh[q];
        tot += drift[q];
      }
      drift[4] = fmax(drift[4], fabs(tot));
      drift[5] += 1.0;
    }
    st->e_pair = e_pair;
    st->e_ewald = real + recip + self + dip;
    st->e_bond = P.use_bond ? misc[0] : 0.0;
    st->e_ext = P.use_ext ? misc[1] : 0.0;
    st->mz = misc[4];
    st->dipl_cur = dip;
    st->sk_pending = 0;  // S(k) was rebuilt from the committed positions
    out[0] = st->e_pair;
    out[1] = st->e_ewald;
    out[2] = st->e_bond;
    out[3] = st->e_ext;
    out[4] = real;
    out[5] = recip;
    out[6] = self;
    out[7] = dip;
  }
}

// The from-scratch FP64 energy of context c enqueued on stream s (no host
// synchronisation): pair and real-space sums, S(k), bonds/walls/self terms,
// then the assembly into the running state (and drift, when given) and, in
// the precision form, the fixed-point mirror. Returns the kernels launched.
int enqueue_total(plum_ctx* c, cudaStream_t s, double* drift) {
  const DevParams& P = c->P;
  int k = 0;
  if (P.use_pair || P.use_ewald) {
    launch_total64(P, c->B, c->d_tot_part, c->n_tot_part, s);
    k++;
  } else {
    cudaMemsetAsync(c->d_tot_part, 0, sizeof(double) * 2 * c->n_tot_part, s);
  }
  if (P.use_ewald && P.n_k > 0) {
    launch_sk_full64(P, c->B, c->d_sk_part, s);
    k += 2;
  }
  launch_misc_total64(P, c->B, c->d_out + 16, s);
  k_assemble_total<<<1, 256, 0, s>>>(P, c->B, c->d_tot_part, c->n_tot_part, c->d_out + 16,
                                     c->d_out, drift);
  k += 2;
  if (c->form == PLUM_FORM_FP32) {
    launch_fix_all(P, c->B, s);
    k++;
  }
  if (c->B.fpos64) {
    launch_fix64_all(P, c->B, s);
    k++;
  }
  return k;
}

int total_energy(plum_ctx* c, double* out8) {
  cudaSetDevice(c->device);
  enqueue_total(c, c->s, nullptr);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(c->h_out, c->d_out, sizeof(double) * 8, cudaMemcpyDeviceToHost, c->s));
  CK(cudaStreamSynchronize(c->s));
  if (out8) std::memcpy(out8, c->h_out, sizeof(double) * 8);
  return PLUM_OK;
}

int read_state(plum_ctx* c, DevState* st) {
  CK(cudaMemcpyAsync(st, c->B.state, sizeof(DevState), cudaMemcpyDeviceToHost, c->s));
  CK(cudaStreamSynchronize(c->s));
  return PLUM_OK;
}

int refresh_host_pos(plum_ctx* c) {
  if (c->h_pos_valid) return PLUM_OK;
  CK(cudaMemcpyAsync(c->h_pos.data(), c->B.pos, sizeof(double4_32a) * c->P.n_bead,
                     cudaMemcpyDeviceToHost, c->s));
  CK(cudaStreamSynchronize(c->s));
  c->h_pos_valid = true;
  return PLUM_OK;
}

int ensure_logs(plum_ctx* c, int n) {
  if (n <= c->log_cap) return PLUM_OK;
  cudaFree(c->d_log_type);
  cudaFree(c->d_log_acc);
  cudaFree(c->d_log_e);
  cudaFree(c->d_log_de);
  if (dalloc(&c->d_log_type, n) || dalloc(&c->d_log_acc, n) || dalloc(&c->d_log_e, n) ||
      dalloc(&c->d_log_de, n))
    return PLUM_ERR_CUDA;
  c->log_cap = n;
  return PLUM_OK;
}

int ensure_stream(plum_ctx* c, long long n) {
  if (n <= c->stream_cap) return PLUM_OK;
  cudaFree(c->d_stream);
  c->d_stream = nullptr;
  if (dalloc(&c->d_stream, (size_t)n)) return PLUM_ERR_CUDA;
  c->stream_cap = n;
  c->gen_len = 0;
  return PLUM_OK;
}

// The energy-difference kernel of the context's form.
void launch_delta(const plum_ctx* c, const DevBuffers& B) {
  if (c->form == PLUM_FORM_FP32)
    launch_delta_pairs32(c->P, B, c->s);
  else
    launch_delta_pairs64(c->P, B, c->s);
}

// Records an event on the context's stream for per-kernel timing.
void kt_mark(plum_ctx* c, int kind) {
  cudaEvent_t e;
  if (cudaEventCreate(&e) != cudaSuccess) return;
  cudaEventRecord(e, c->s);
  c->kt_ev.push_back(e);
  c->kt_kind.push_back(kind);
}

void enqueue_loop(plum_ctx* c, int n_moves, const DevBuffers& B) {
  // with a training log, each generated chain move's descriptor is taken
  // before its energy change
  const bool desc = B.log_desc != nullptr;
  launch_serial64(c->P, B, kModeGen, c->s);
  if (desc) launch_desc_batch(c->d_rp1, c->d_rb1, 1, B.desc_acc, c->P.form, 0, c->s);
  for (int i = 0; i < n_moves; i++) {
    if (c->kt_on) kt_mark(c, 0);
    launch_delta(c, B);
    if (c->kt_on) kt_mark(c, 1);
    int mode = kModeFinish | kModeDecide | (i + 1 < n_moves ? kModeGen : 0);
    launch_serial64(c->P, B, mode, c->s);
    if (c->kt_on) kt_mark(c, 2);
    if (desc && i + 1 < n_moves)
      launch_desc_batch(c->d_rp1, c->d_rb1, 1, B.desc_acc, c->P.form, 0, c->s);
  }
}

// The device MC loop: gen, then (pairs, finish+decide+gen) per step. Batches
// of a repeated size run as one CUDA graph, captured on the second use (the
// first runs as plain launches so lazy kernel set-up happens outside a
// capture); the kernels read the pending move from device state, so one
// capture replays for every batch.
int device_loop(plum_ctx* c, int n_moves, DevBuffers B) {
  const long k = 1 + 2L * n_moves + (B.log_desc ? n_moves : 0);
  if (B.log_desc) CK(cudaMemcpyAsync(c->d_rb1, &B, sizeof(B), cudaMemcpyHostToDevice, c->s));
  if (c->kt_on) {
    enqueue_loop(c, n_moves, B);
    CK(cudaGetLastError());
    c->last_kernels += k;
    return PLUM_OK;
  }
  const bool same = c->gexec && c->g_moves == n_moves && !std::memcmp(&c->g_B, &B, sizeof(B));
  if (same) {
    CK(cudaGraphLaunch(c->gexec, c->s));
    c->last_kernels += k;
    return PLUM_OK;
  }
  if (c->g_warm && n_moves >= 8) {
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(c->s, cudaStreamCaptureModeThreadLocal));
    enqueue_loop(c, n_moves, B);
    CK(cudaStreamEndCapture(c->s, &g));
    if (c->gexec) cudaGraphExecDestroy(c->gexec);
    c->gexec = nullptr;
    cudaError_t e = cudaGraphInstantiate(&c->gexec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return fail(PLUM_ERR_CUDA, cudaGetErrorString(e));
    c->g_moves = n_moves;
    c->g_B = B;
    CK(cudaGraphLaunch(c->gexec, c->s));
    c->last_kernels += k;
    return PLUM_OK;
  }
  c->g_warm = true;
  enqueue_loop(c, n_moves, B);
  CK(cudaGetLastError());
  c->last_kernels += k;
  return PLUM_OK;
}

}  // namespace

// FMA throughput probe: every thread runs 8 independent FMA chains, so the
// pipe, not latency, limits it.
template <typename T>
__global__ void k_fma_probe(T* out, int iters, T a, T b) {
  T x[8];
  for (int i = 0; i < 8; i++) x[i] = (T)(threadIdx.x + i) * (T)1e-3;
  for (int it = 0; it < iters; it++)
#pragma unroll
    for (int i = 0; i < 8; i++) x[i] = x[i] * a + b;
  T s = 0;
  for (int i = 0; i < 8; i++) s += x[i];
  if (s == (T)-1.2345) out[0] = s;  // keeps the chains live
}

extern "C" {

const char* plum_last_error(void) { return g_err.c_str(); }

static int create_ctx(plum_ctx* c, int form, int device, plum_ctx** out);

int plum_ctx_create(const char* dir, const char* runin, int form, int device,
                    plum_ctx** out) {
  if (!out || !dir || !runin) return fail(PLUM_ERR_INPUT, "null argument");
  *out = nullptr;
  plum_ctx* c = new plum_ctx();
  std::string err;
  if (!read_input(dir, runin, &c->in, &err)) {
    delete c;
    return fail(PLUM_ERR_INPUT, err);
  }
  return create_ctx(c, form, device, out);
}

int plum_ctx_create_text(const char* dir, const char* runin_text, int form, int device,
                         plum_ctx** out) {
  if (!out || !dir || !runin_text) return fail(PLUM_ERR_INPUT, "null argument");
  *out = nullptr;
  plum_ctx* c = new plum_ctx();
  std::string err;
  if (!read_input_text(dir, runin_text, &c->in, &err)) {
    delete c;
    return fail(PLUM_ERR_INPUT, err);
  }
  return create_ctx(c, form, device, out);
}

static int create_ctx(plum_ctx* c, int form, int device, plum_ctx** out) {
  if (form != PLUM_FORM_FP64 && form != PLUM_FORM_FP32) {
    delete c;
    return fail(PLUM_ERR_INPUT, "unknown form");
  }
  c->form = form;
  c->device = device;
  if (c->in.use_gc) {
    // the grand-canonical species' symbol joins the type table (the
    // reference creates its beads with that symbol, force_field.cc:383-401)
    auto& tn = c->in.type_names;
    if (std::find(tn.begin(), tn.end(), c->in.gc_symbol) == tn.end()) tn.push_back(c->in.gc_symbol);
  }
  Input& in = c->in;
  // The reference's own input checks (simulation.cc:142-191, force_field.cc:205-209).
  std::string bad;
  double ptot = 0;
  for (int i = 0; i < 5; i++) ptot += in.move_prob[i];
  if (in.beta <= 0) bad = "beta must be positive";
  else if (in.npbc < 2 || in.npbc > 3) bad = "PBC dimensions must be 2 or 3";
  else if (std::fabs(ptot - 1.0) > 1e-4) bad = "MC move probabilities do not sum up to 1.0";
  else if (in.move_prob[4] > 0 && !in.use_rigid)
    bad = "the reptation move requires the rigid bond setting";
  else if (in.calc_chem_pot && in.use_gc)
    bad = "chemical potential cannot be calculated when GCMC is used";
  else if (in.vp_bead_size < 0) bad = "virial bead size must not be negative";
  else if ((int)in.type_names.size() > kMaxTypes)
    bad = "more than " + std::to_string(kMaxTypes) + " bead types";
  if (!bad.empty()) {
    delete c;
    return fail(PLUM_ERR_INPUT, bad);
  }
  DevParams& P = c->P;
  std::memset(&P, 0, sizeof(P));
  const int nb = (int)in.q.size();
  P.n_bead = nb;
  P.n_mol = in.n_mol;
  P.n_type = (int)in.type_names.size();
  P.npbc = in.npbc;
  P.phantom = in.phantom;
  P.grafted = in.grafted;
  for (int a = 0; a < 3; a++) {
    P.box[a] = in.box[a];
    P.inv_box[a] = 1.0 / in.box[a];
    P.ebox[a] = in.box[a];
    P.inv_ebox[a] = 1.0 / in.box[a];
  }
  P.use_pair = in.use_pair;
  P.use_ewald = in.use_ewald;
  P.use_bond = in.use_bond;
  P.use_rigid = in.use_rigid;
  P.use_ext = in.use_ext;
  P.beta = in.beta;
  P.move_size = in.move_size;
  for (int i = 0; i < 5; i++) P.move_prob[i] = in.move_prob[i];
  // simulation.cc:286-296
  P.bond_len = 0;
  P.vary_bond = 0;
  if (in.use_rigid) P.bond_len = in.rigid;
  if (in.use_bond) {
    P.bond_len = in.r0;
    P.vary_bond = 1;
  }
  P.k_bond = in.k_bond;
  P.r0 = in.r0;
  // LJ mixing and shifts (potential_truncated_lj.cc:55-81).
  for (int i = 0; i < P.n_type; i++)
    for (int j = 0; j < P.n_type; j++) {
      LJEntry a, b;
      auto ia = in.lj.find(in.type_names[i]);
      auto ib = in.lj.find(in.type_names[j]);
      if (ia != in.lj.end()) a = ia->second;
      if (ib != in.lj.end()) b = ib->second;
      double sigma = (a.sigma + b.sigma) / 2;
      double eps = std::sqrt((a.epsilon * b.epsilon));
      int k = i * P.n_type + j;
      P.lj_sig2[k] = sigma * sigma;
      P.lj_eps4[k] = 4 * eps;
      if (in.lj_cut < 0) {
        double r6r = std::pow((1.0 / k216), 6);
        P.lj_eref[k] = 4 * eps * (r6r * r6r - r6r);
        P.lj_rc2[k] = (k216 * sigma) * (k216 * sigma);
      } else {
        double r6r = std::pow((sigma / in.lj_cut), 6);
        P.lj_eref[k] = 4 * eps * (r6r * r6r - r6r);
        P.lj_rc2[k] = in.lj_cut * in.lj_cut;
      }
    }
  // hard spheres: radius sums; symbols absent from the table have radius 0
  // (std::map::operator[] in potential_hard_sphere.cc:42)
  P.pair_kind = in.pair_kind;
  if (in.pair_kind == 1)
    for (int i = 0; i < P.n_type; i++)
      for (int j = 0; j < P.n_type; j++) {
        auto ia = in.hs_radius.find(in.type_names[i]);
        auto ib = in.hs_radius.find(in.type_names[j]);
        const double s = (ia != in.hs_radius.end() ? ia->second : 0.0) +
                         (ib != in.hs_radius.end() ? ib->second : 0.0);
        const int k = i * P.n_type + j;
        P.hs_sum[k] = s;
        // pre-test bound: every r <= s passes r2 < lj_rc2
        P.lj_rc2[k] = s * s * (1.0 + 1e-5) + 1e-30;
        P.lj_sig2[k] = P.lj_eps4[k] = P.lj_eref[k] = 0.0;
      }
  P.wall_cut = in.wall_cut;
  P.ext_kind = in.ext_kind;
  P.well_width = in.well_width;
  P.well_depth = in.well_depth;
  for (int i = 0; i < P.n_type; i++) {
    auto it = in.wall.find(in.type_names[i]);
    P.wall_sig[i] = it != in.wall.end() ? it->second.sigma : 0.0;
    P.wall_eps[i] = it != in.wall.end() ? it->second.epsilon : 0.0;
    P.graft[i] = in.type_names[i] == "L" ? 1 : (in.type_names[i] == "R" ? 2 : 0);
    auto ir = in.wall_radius.find(in.type_names[i]);
    P.wall_rad[i] = ir != in.wall_radius.end() ? ir->second : 0.0;
  }
  std::vector<int> chains, ions;
  for (int m = in.phantom; m < in.n_mol; m++) {
    int sz = in.mol_start[m + 1] - in.mol_start[m];
    (sz > 1 ? chains : ions).push_back(m);
    c->max_len = std::max(c->max_len, sz);
  }
  P.n_chain_total = (int)chains.size();
  P.n_ion_total = (int)ions.size();
  std::vector<short4> kn;
  std::vector<double> kw;
  if (form == PLUM_FORM_FP32 && in.npbc == 3 && in.dipole) {
    delete c;
    return fail(PLUM_ERR_INPUT, "the precision form needs npbc = 2 when the dipole correction is on");
  }
  if (in.use_ewald) {
    int rc = setup_ewald(c, &kn, &kw);
    if (rc) {
      delete c;
      return rc;
    }
  }
  // Precision-form constants: fixed point in units of the Ewald box.
  P.form = form;
  for (int a = 0; a < 3; a++) {
    P.f_scale[a] = (float)(P.ebox[a] / 4294967296.0);
    P.same_wrap = (a == 0 ? 1 : P.same_wrap) &&
                  (a >= P.npbc || (P.box[a] == P.ebox[a] && P.inv_box[a] == P.inv_ebox[a]));
    P.inv_fix[a] = 4294967296.0 / P.ebox[a];
    P.f_box[a] = (float)P.ebox[a];
  }
  // the largest LJ (or hard-sphere bound) cut-off over the type pairs in
  // use: a uniform pre-test before the per-pair table lookup; > 0, so a
  // coincident pair (r2 = 0, the overlap value) always reaches lj64
  P.lj_max2 = 1e-300;
  for (int k = 0; k < P.n_type * P.n_type; k++) P.lj_max2 = std::max(P.lj_max2, P.lj_rc2[k]);
  for (int k = 0; k < kMaxT2; k++) {
    P.f_lj_sig2[k] = (float)P.lj_sig2[k];
    P.f_lj_eps4[k] = (float)P.lj_eps4[k];
    P.f_lj_rc2[k] = (float)P.lj_rc2[k];
    P.f_lj_eref[k] = (float)P.lj_eref[k];
    P.f_hs_sum[k] = (float)P.hs_sum[k];
  }
  P.f_real_cut = (float)P.real_cut;
  P.f_sqrt_alpha = (float)P.sqrt_alpha;
  P.f_lB = (float)P.lB;
  c->recompute_every = form == PLUM_FORM_FP32 ? 10000 : 0;
  // Device state.
  if (cudaSetDevice(device) != cudaSuccess) {
    delete c;
    return fail(PLUM_ERR_CUDA, "cannot select CUDA device " + std::to_string(device));
  }
  if (cudaStreamCreateWithFlags(&c->s, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&c->ev0) != cudaSuccess || cudaEventCreate(&c->ev1) != cudaSuccess) {
    plum_ctx_destroy(c);
    return fail(PLUM_ERR_CUDA, "cannot create the context's stream and events");
  }
  DevBuffers& B = c->B;
  std::memset(&B, 0, sizeof(B));
  int rc = 0;
  rc |= dalloc(&B.pos, nb);
  rc |= dalloc(&B.trial, nb);
  rc |= dalloc(&B.type, nb);
  rc |= dalloc(&B.mol_start, in.n_mol + 1);
  rc |= dalloc(&B.chain_ids, chains.size());
  rc |= dalloc(&B.ion_ids, ions.size());
  rc |= dalloc(&B.kn, kn.size());
  rc |= dalloc(&B.kw, kw.size());
  rc |= dalloc(&B.sk, kn.size());
  rc |= dalloc(&B.dsk, 2 * kn.size());
  rc |= dalloc(&B.done_count, 1);
  rc |= dalloc(&B.partial, 4 * (size_t)std::max(pair_grid(), pair_grid32()));
  rc |= dalloc(&B.fpos, nb);
  rc |= dalloc(&B.fq, nb);
  rc |= dalloc(&B.ftrial, c->max_len);
  {
    int groups = (c->max_len + std::max(1, P.kchunk_delta) - 1) / std::max(1, P.kchunk_delta);
    rc |= dalloc(&B.dsk_part, (size_t)groups * std::max(1, P.n_k));
    rc |= dalloc(&B.dsk_part32, (size_t)groups * std::max(1, P.n_k));
    rc |= dalloc(&B.ktile_count, ktile_count(P));
    rc |= dalloc(&B.kpartial, ktile_count(P));
  }
  rc |= dalloc(&B.bond_mol, in.n_mol);
  rc |= dalloc(&B.state, 1);
  c->n_tot_part = total_partials_count(P);
  rc |= dalloc(&c->d_tot_part, 2 * (size_t)c->n_tot_part);
  rc |= dalloc(&c->d_sk_part, (size_t)sk_full_groups(P) * std::max(1, P.n_k));
  rc |= dalloc(&c->d_out, 64);
  rc |= dalloc(&c->d_obs_per, 5 * (size_t)std::max(1, in.n_mol));
  c->rhoz_bins = (int)std::ceil(in.box[2] / kRhoZRes);
  rc |= dalloc(&c->d_rhoz, 3 * (size_t)std::max(1, c->rhoz_bins));
  rc |= dalloc(&c->d_mt, 625);
  // the FP64 real-space term from the h(u) table (every form: the plain
  // form's moves, the from-scratch energies, the FP64 trial energies)
  P.htab64 = nullptr;
  if (P.use_ewald) {
    rc |= dalloc(&c->d_htab64, (size_t)kH64Bins * kH64Stride);
    if (!rc) {
      std::vector<double> h((size_t)kH64Bins * kH64Stride);
      build_h64_table(h.data());
      cudaMemcpy(c->d_htab64, h.data(), sizeof(double) * h.size(), cudaMemcpyHostToDevice);
      P.htab64 = c->d_htab64;
    }
  }
  // the plain form's 64-bit position mirror for its fixed-point pair loop
  if (form == PLUM_FORM_FP64 && fix_pairs(P)) rc |= dalloc(&c->B.fpos64, nb);
  // the precision form's real-space term from the h(u) table where the
  // cut-off lies inside it (alpha r_c^2 < 2^kH32EHi)
  P.htab = nullptr;
  if (form == PLUM_FORM_FP32 && P.use_ewald &&
      P.sqrt_alpha * P.sqrt_alpha * P.real_cut * P.real_cut < std::ldexp(1.0, kH32EHi)) {
    rc |= dalloc(&c->d_htab, kH32Bins);
    if (!rc) {
      std::vector<float4> h(kH32Bins);
      build_h32_table(h.data());
      cudaMemcpy(c->d_htab, h.data(), sizeof(float4) * kH32Bins, cudaMemcpyHostToDevice);
      P.htab = c->d_htab;
    }
  }
  if (rc) {
    plum_ctx_destroy(c);
    return PLUM_ERR_CUDA;
  }
  if (cudaMallocHost(&c->h_out, 64 * sizeof(double)) != cudaSuccess) {
    c->h_out = nullptr;
    plum_ctx_destroy(c);
    return fail(PLUM_ERR_CUDA, "cannot allocate pinned host memory");
  }
  c->h_pos.resize(nb);
  for (int i = 0; i < nb; i++)
    c->h_pos[i] = make_double4_32a(in.xyz[3 * i], in.xyz[3 * i + 1], in.xyz[3 * i + 2], in.q[i]);
  cudaMemcpy(B.pos, c->h_pos.data(), sizeof(double4_32a) * nb, cudaMemcpyHostToDevice);
  cudaMemcpy(B.trial, c->h_pos.data(), sizeof(double4_32a) * nb, cudaMemcpyHostToDevice);
  cudaMemcpy(B.type, in.type.data(), sizeof(int) * nb, cudaMemcpyHostToDevice);
  cudaMemcpy(B.mol_start, in.mol_start.data(), sizeof(int) * (in.n_mol + 1),
             cudaMemcpyHostToDevice);
  if (!chains.empty())
    cudaMemcpy(B.chain_ids, chains.data(), sizeof(int) * chains.size(), cudaMemcpyHostToDevice);
  if (!ions.empty())
    cudaMemcpy(B.ion_ids, ions.data(), sizeof(int) * ions.size(), cudaMemcpyHostToDevice);
  if (!kn.empty()) {
    cudaMemcpy(B.kn, kn.data(), sizeof(short4) * kn.size(), cudaMemcpyHostToDevice);
    cudaMemcpy(B.kw, kw.data(), sizeof(double) * kw.size(), cudaMemcpyHostToDevice);
  }
  cudaMemset(B.state, 0, sizeof(DevState));
  cudaMemset(B.ktile_count, 0, sizeof(int) * std::max(1, ktile_count(P)));
  cudaMemset(B.done_count, 0, sizeof(int));
  cudaError_t e = cudaDeviceSynchronize();
  if (e != cudaSuccess) {
    plum_ctx_destroy(c);
    return fail(PLUM_ERR_CUDA, cudaGetErrorString(e));
  }
  rc = plum_seed(c, 5489u);
  if (!rc) rc = total_energy(c, nullptr);
  if (rc) {
    plum_ctx_destroy(c);
    return rc;
  }
  *out = c;
  return PLUM_OK;
}

int plum_ctx_destroy(plum_ctx* c) {
  if (!c) return PLUM_OK;
  cudaSetDevice(c->device);
  if (c->s) cudaStreamSynchronize(c->s);
  void* ptrs[] = {c->B.pos,      c->B.trial,   c->B.type,  c->B.mol_start, c->B.chain_ids,
                  c->B.ion_ids,  c->B.kn,      c->B.kw,    c->B.sk,        c->B.dsk,
                  c->B.partial,  c->B.bond_mol, c->B.state, c->d_tot_part,  c->d_out,
                  c->B.dsk_part, c->B.ktile_count, c->B.kpartial, c->B.fpos, c->B.done_count,
                  c->B.fq,       c->B.ftrial,  c->B.dsk_part32, c->cb_b, c->cb_c, c->cb_so,
                  c->cb_part,    c->cb_u,      c->d_obs_per, c->d_rhoz, c->desc_acc,
                  c->d_rp1,      c->d_rb1,     c->desc_fine, c->cb_part32, c->cb_ticket,
                  c->d_stream,   c->d_mt,      c->d_log_type, c->d_log_acc, c->d_log_e,
                  c->d_press,    c->d_sk_part, c->d_log_de, c->d_htab, c->d_htab64,
                  c->B.fpos64};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (c->h_out) cudaFreeHost(c->h_out);
  if (c->ev0) cudaEventDestroy(c->ev0);
  if (c->ev1) cudaEventDestroy(c->ev1);
  for (cudaEvent_t e : c->kt_ev) cudaEventDestroy(e);
  if (c->gexec) cudaGraphExecDestroy(c->gexec);
  if (c->s) cudaStreamDestroy(c->s);
  delete c;
  return PLUM_OK;
}

int plum_ctx_info(const plum_ctx* c, plum_info* o) {
  if (!c || !o) return fail(PLUM_ERR_INPUT, "null argument");
  std::memset(o, 0, sizeof(*o));
  o->n_bead = c->P.n_bead;
  o->n_mol = c->P.n_mol;
  o->n_type = c->P.n_type;
  o->n_kvec = c->P.n_k;
  o->npbc = c->P.npbc;
  o->form = c->form;
  for (int a = 0; a < 3; a++) {
    o->box[a] = c->P.box[a];
    o->ewald_box[a] = c->P.ebox[a];
    o->real_cell[a] = c->P.real_cell[a];
    o->k_cell[a] = c->P.kmax[a];
  }
  o->real_cutoff = c->P.real_cut;
  o->kcut2 = c->in.x_kcut2;
  o->alpha = c->in.alpha;
  o->lB = c->in.lB;
  return PLUM_OK;
}

int plum_total_energy(plum_ctx* c, double* out) {
  if (!c) return fail(PLUM_ERR_INPUT, "null context");
  if (c->host_pending) return fail(PLUM_ERR_STATE, "a trial move is pending");
  return total_energy(c, out);
}

int plum_energies(const plum_ctx* cc, double* out) {
  plum_ctx* c = const_cast<plum_ctx*>(cc);
  if (!c || !out) return fail(PLUM_ERR_INPUT, "null argument");
  cudaSetDevice(c->device);
  DevState st;
  int rc = read_state(c, &st);
  if (rc) return rc;
  out[0] = st.e_pair, out[1] = st.e_ewald, out[2] = st.e_bond, out[3] = st.e_ext;
  return PLUM_OK;
}

int plum_delta_energy(plum_ctx* c, int mol, const double* trial, const int* moved,
                      double* out) {
  if (!c || !trial || !moved || !out) return fail(PLUM_ERR_INPUT, "null argument");
  if (mol < 0 || mol >= c->P.n_mol) return fail(PLUM_ERR_INPUT, "molecule index out of range");
  if (c->host_pending) return fail(PLUM_ERR_STATE, "a trial move is already pending");
  cudaSetDevice(c->device);
  int rc = refresh_host_pos(c);
  if (rc) return rc;
  const int b0 = c->in.mol_start[mol], b1 = c->in.mol_start[mol + 1];
  int lo = -1, hi = -1;
  for (int i = b0; i < b1; i++)
    if (moved[i - b0]) {
      if (lo < 0) lo = i;
      hi = i + 1;
    }
  if (lo < 0) lo = hi = b0;
  // Beads inside [lo, hi) that are not flagged keep their current position,
  // so their terms cancel exactly.
  std::vector<double4_32a> span(hi - lo);
  for (int i = lo; i < hi; i++) {
    double4_32a p = c->h_pos[i];
    if (moved[i - b0]) {
      p.x = trial[3 * (i - b0)];
      p.y = trial[3 * (i - b0) + 1];
      p.z = trial[3 * (i - b0) + 2];
    }
    span[i - lo] = p;
  }
  if (hi > lo)
    CK(cudaMemcpyAsync(c->B.trial + lo, span.data(), sizeof(double4_32a) * (hi - lo),
                       cudaMemcpyHostToDevice, c->s));
  launch_set_move(c->B, mol, lo, hi, c->s);
  if (c->form == PLUM_FORM_FP32) launch_fix_trial(c->P, c->B, c->s);
  launch_delta(c, c->B);
  launch_serial64(c->P, c->B, kModeFinish, c->s);
  CK(cudaGetLastError());
  DevState st;
  rc = read_state(c, &st);
  if (rc) return rc;
  if (st.error) return fail(st.error, "device reported an error in the energy difference");
  out[0] = st.de, out[1] = st.de_pair, out[2] = st.de_ewald, out[3] = st.de_bond,
  out[4] = st.de_ext;
  c->host_pending = true;
  return PLUM_OK;
}

namespace {
int ensure_desc(plum_ctx* c) {
  if (c->desc_acc) return PLUM_OK;
  int rc = dalloc(&c->desc_acc, mlp::kIn) | dalloc(&c->desc_fine, mlp::kFineAll) |
           dalloc(&c->d_rp1, 1) | dalloc(&c->d_rb1, 1);
  if (rc) return PLUM_ERR_CUDA;
  CK(cudaMemcpyAsync(c->d_rp1, &c->P, sizeof(DevParams), cudaMemcpyHostToDevice, c->s));
  return PLUM_OK;
}
}  // namespace

namespace {
// Re-creates the bead-count-dependent device buffers from the host copy of
// the system (in.q, in.type, in.mol_start and h_pos) after molecules were
// added or removed, then recomputes every energy term and S(k) from scratch.
int rebuild_system(plum_ctx* c) {
  Input& in = c->in;
  DevParams& P = c->P;
  DevBuffers& B = c->B;
  const int nb = (int)in.q.size();
  CK(cudaStreamSynchronize(c->s));
  std::vector<int> chains, ions;
  c->max_len = 1;
  for (int m = in.phantom; m < in.n_mol; m++) {
    const int sz = in.mol_start[m + 1] - in.mol_start[m];
    (sz > 1 ? chains : ions).push_back(m);
    c->max_len = std::max(c->max_len, sz);
  }
  P.n_bead = nb;
  P.n_mol = in.n_mol;
  P.n_chain_total = (int)chains.size();
  P.n_ion_total = (int)ions.size();
  const bool mirror64 = B.fpos64 != nullptr;
  void* old[] = {B.pos,      B.trial,      B.type,     B.mol_start, B.chain_ids, B.ion_ids,
                 B.fpos,     B.fq,         B.ftrial,   B.dsk_part,  B.dsk_part32, B.bond_mol,
                 c->d_tot_part, c->d_obs_per, c->cb_b, c->cb_c,    c->cb_part,  c->cb_u,
                 B.fpos64};
  for (void* q : old)
    if (q) cudaFree(q);
  B.pos = B.trial = nullptr;
  B.fpos64 = nullptr;
  B.type = B.mol_start = B.chain_ids = B.ion_ids = nullptr;
  B.fpos = B.ftrial = nullptr;
  B.fq = nullptr;
  B.dsk_part = nullptr;
  B.dsk_part32 = nullptr;
  B.bond_mol = nullptr;
  c->d_tot_part = c->d_obs_per = nullptr;
  c->cb_b = c->cb_c = nullptr;
  c->cb_part = c->cb_u = nullptr;
  c->cb_cap = 0;
  int rc = dalloc(&B.pos, nb) | dalloc(&B.trial, nb) | dalloc(&B.type, nb) |
           dalloc(&B.mol_start, in.n_mol + 1) | dalloc(&B.chain_ids, chains.size()) |
           dalloc(&B.ion_ids, ions.size()) | dalloc(&B.fpos, nb) | dalloc(&B.fq, nb) |
           dalloc(&B.ftrial, c->max_len) | dalloc(&B.bond_mol, in.n_mol);
  if (mirror64) rc |= dalloc(&B.fpos64, nb);
  const int groups = (c->max_len + std::max(1, P.kchunk_delta) - 1) / std::max(1, P.kchunk_delta);
  rc |= dalloc(&B.dsk_part, (size_t)groups * std::max(1, P.n_k));
  rc |= dalloc(&B.dsk_part32, (size_t)groups * std::max(1, P.n_k));
  c->n_tot_part = total_partials_count(P);
  rc |= dalloc(&c->d_tot_part, 2 * (size_t)c->n_tot_part);
  rc |= dalloc(&c->d_obs_per, 5 * (size_t)std::max(1, in.n_mol));
  if (rc) return PLUM_ERR_CUDA;
  CK(cudaMemcpyAsync(B.pos, c->h_pos.data(), sizeof(double4_32a) * nb, cudaMemcpyHostToDevice,
                     c->s));
  CK(cudaMemcpyAsync(B.trial, c->h_pos.data(), sizeof(double4_32a) * nb, cudaMemcpyHostToDevice,
                     c->s));
  CK(cudaMemcpyAsync(B.type, in.type.data(), sizeof(int) * nb, cudaMemcpyHostToDevice, c->s));
  CK(cudaMemcpyAsync(B.mol_start, in.mol_start.data(), sizeof(int) * (in.n_mol + 1),
                     cudaMemcpyHostToDevice, c->s));
  if (!chains.empty())
    CK(cudaMemcpyAsync(B.chain_ids, chains.data(), sizeof(int) * chains.size(),
                       cudaMemcpyHostToDevice, c->s));
  if (!ions.empty())
    CK(cudaMemcpyAsync(B.ion_ids, ions.data(), sizeof(int) * ions.size(), cudaMemcpyHostToDevice,
                       c->s));
  if (c->d_rp1) CK(cudaMemcpyAsync(c->d_rp1, &P, sizeof(P), cudaMemcpyHostToDevice, c->s));
  DevState st;
  rc = read_state(c, &st);
  if (rc) return rc;
  st.pending = 0;
  st.sk_pending = 0;
  CK(cudaMemcpyAsync(B.state, &st, sizeof(st), cudaMemcpyHostToDevice, c->s));
  if (c->gexec) cudaGraphExecDestroy(c->gexec);
  c->gexec = nullptr;
  c->g_moves = 0;
  c->g_warm = false;
  c->host_pending = false;
  c->h_pos_valid = true;
  in.xyz.resize(3 * (size_t)nb);
  for (int i = 0; i < nb; i++) {
    in.xyz[3 * i] = c->h_pos[i].x;
    in.xyz[3 * i + 1] = c->h_pos[i].y;
    in.xyz[3 * i + 2] = c->h_pos[i].z;
  }
  return total_energy(c, nullptr);
}
}  // namespace

int plum_gc_info(const plum_ctx* c, double* out) {
  if (!c || !out) return fail(PLUM_ERR_INPUT, "null argument");
  const Input& in = c->in;
  if (!in.use_gc) return fail(PLUM_ERR_INPUT, "run.in has no grand-canonical species");
  const auto& tn = in.type_names;
  out[0] = in.chem_pot;
  out[1] = in.deBroglie;
  out[2] = in.gc_bead_charge;
  out[3] = in.gc_chain_len;
  out[4] = in.cbmc_trials;
  out[5] = in.gc_freq;
  out[6] = in.k_bond;
  out[7] = in.r0;
  out[8] = (double)(std::find(tn.begin(), tn.end(), in.gc_symbol) - tn.begin());
  return PLUM_OK;
}

int plum_append_molecules(plum_ctx* c, int n_mols, const int* sizes, const double* xyz,
                          const double* q, const int* type) {
  if (!c || n_mols <= 0 || !sizes || !xyz || !q || !type)
    return fail(PLUM_ERR_INPUT, "bad argument");
  if (c->host_pending) return fail(PLUM_ERR_STATE, "a trial move is pending");
  long total = 0;
  for (int m = 0; m < n_mols; m++) {
    if (sizes[m] <= 0) return fail(PLUM_ERR_INPUT, "empty molecule");
    total += sizes[m];
  }
  for (long k = 0; k < total; k++)
    if (type[k] < 0 || type[k] >= c->P.n_type || !std::isfinite(xyz[3 * k]) ||
        !std::isfinite(xyz[3 * k + 1]) || !std::isfinite(xyz[3 * k + 2]))
      return fail(PLUM_ERR_INPUT, "bad bead type or position");
  cudaSetDevice(c->device);
  int rc = refresh_host_pos(c);
  if (rc) return rc;
  Input& in = c->in;
  for (long k = 0; k < total; k++) {
    in.q.push_back(q[k]);
    in.type.push_back(type[k]);
    c->h_pos.push_back(make_double4_32a(xyz[3 * k], xyz[3 * k + 1], xyz[3 * k + 2], q[k]));
  }
  for (int m = 0; m < n_mols; m++) in.mol_start.push_back(in.mol_start.back() + sizes[m]);
  in.n_mol += n_mols;
  return rebuild_system(c);
}

int plum_erase_molecules(plum_ctx* c, int first, int count) {
  if (!c || first < 0 || count <= 0 || first + count > c->in.n_mol)
    return fail(PLUM_ERR_INPUT, "molecule range out of bounds");
  if (c->host_pending) return fail(PLUM_ERR_STATE, "a trial move is pending");
  cudaSetDevice(c->device);
  int rc = refresh_host_pos(c);
  if (rc) return rc;
  Input& in = c->in;
  const int b0 = in.mol_start[first], b1 = in.mol_start[first + count], nb = b1 - b0;
  in.q.erase(in.q.begin() + b0, in.q.begin() + b1);
  in.type.erase(in.type.begin() + b0, in.type.begin() + b1);
  c->h_pos.erase(c->h_pos.begin() + b0, c->h_pos.begin() + b1);
  in.mol_start.erase(in.mol_start.begin() + first + 1, in.mol_start.begin() + first + count + 1);
  for (int m = first + 1; m <= in.n_mol - count; m++) in.mol_start[m] -= nb;
  in.n_mol -= count;
  return rebuild_system(c);
}

int plum_move_descriptor(plum_ctx* c, double* out) {
  if (!c || !out) return fail(PLUM_ERR_INPUT, "null argument");
  if (!c->host_pending) return fail(PLUM_ERR_STATE, "no pending trial move");
  cudaSetDevice(c->device);
  int rc = ensure_desc(c);
  if (rc) return rc;
  DevBuffers B = c->B;
  B.desc_acc = c->desc_acc;
  B.desc_fine = c->desc_fine;
  const int one = 1, zero = 0;
  CK(cudaMemcpyAsync(c->d_rb1, &B, sizeof(B), cudaMemcpyHostToDevice, c->s));
  CK(cudaMemsetAsync(c->desc_fine, 0, sizeof(unsigned) * mlp::kFineAll, c->s));
  CK(cudaMemcpyAsync(&c->B.state->da_active, &one, sizeof(int), cudaMemcpyHostToDevice, c->s));
  launch_desc_batch(c->d_rp1, c->d_rb1, 1, c->desc_acc, c->P.form, 0, c->s);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(&c->B.state->da_active, &zero, sizeof(int), cudaMemcpyHostToDevice, c->s));
  unsigned h[mlp::kIn];
  CK(cudaMemcpyAsync(h, c->desc_acc, sizeof(h), cudaMemcpyDeviceToHost, c->s));
  CK(cudaStreamSynchronize(c->s));
  for (int k = 0; k < mlp::kIn; k++) out[k] = h[k] * (double)mlp::kDescUnit;
  return PLUM_OK;
}

int plum_finalize(plum_ctx* c, int accept) {
  if (!c) return fail(PLUM_ERR_INPUT, "null context");
  if (!c->host_pending) return fail(PLUM_ERR_STATE, "no pending trial move");
  cudaSetDevice(c->device);
  int acc = accept ? 1 : 0;
  CK(cudaMemcpyAsync(&c->B.state->last_accept, &acc, sizeof(int), cudaMemcpyHostToDevice, c->s));
  launch_serial64(c->P, c->B, kModeCommit, c->s);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(c->s));
  c->host_pending = false;
  if (accept) c->h_pos_valid = false;
  return PLUM_OK;
}

int plum_run_moves(plum_ctx* c, const uint32_t* stream, long n_stream, int n_moves,
                   int* move_type, int* accept, double* etot, long* draws_used) {
  return plum_run_moves_de(c, stream, n_stream, n_moves, move_type, accept, etot, nullptr,
                           draws_used);
}

int plum_run_moves_de(plum_ctx* c, const uint32_t* stream, long n_stream, int n_moves,
                      int* move_type, int* accept, double* etot, double* de,
                      long* draws_used) {
  if (!c || (!stream && n_stream > 0) || n_moves < 0)
    return fail(PLUM_ERR_INPUT, "bad argument");
  if (c->host_pending) return fail(PLUM_ERR_STATE, "a trial move is pending");
  if (c->in.use_gc) return fail(PLUM_ERR_INPUT, "grand-canonical steps are not run by this loop");
  if (n_moves == 0) return PLUM_OK;
  cudaSetDevice(c->device);
  int rc = ensure_stream(c, n_stream);
  if (!rc) rc = ensure_logs(c, n_moves);
  if (rc) return rc;
  CK(cudaMemcpyAsync(c->d_stream, stream, sizeof(uint32_t) * n_stream, cudaMemcpyHostToDevice,
                     c->s));
  c->gen_len = 0;  // the device generator's buffer is overwritten
  DevState st;
  rc = read_state(c, &st);
  if (rc) return rc;
  st.stream_pos = 0;
  st.stream_len = n_stream;
  st.step = 0;
  st.step_open = 0;
  st.error = 0;
  st.pending = 0;
  CK(cudaMemcpyAsync(c->B.state, &st, sizeof(DevState), cudaMemcpyHostToDevice, c->s));
  DevBuffers B = c->B;
  B.stream = c->d_stream;
  B.log_type = c->d_log_type;
  B.log_accept = c->d_log_acc;
  B.log_etot = c->d_log_e;
  B.log_step_de = de ? c->d_log_de : nullptr;
  c->last_kernels = 0;
  CK(cudaEventRecord(c->ev0, c->s));
  rc = device_loop(c, n_moves, B);
  if (rc) return rc;
  CK(cudaEventRecord(c->ev1, c->s));
  CK(cudaStreamSynchronize(c->s));
  float ms = 0;
  cudaEventElapsedTime(&ms, c->ev0, c->ev1);
  c->last_ms = ms;
  rc = read_state(c, &st);
  if (rc) return rc;
  c->h_pos_valid = false;
  if (move_type)
    CK(cudaMemcpy(move_type, c->d_log_type, sizeof(int) * n_moves, cudaMemcpyDeviceToHost));
  if (accept)
    CK(cudaMemcpy(accept, c->d_log_acc, sizeof(int) * n_moves, cudaMemcpyDeviceToHost));
  if (etot) CK(cudaMemcpy(etot, c->d_log_e, sizeof(double) * n_moves, cudaMemcpyDeviceToHost));
  if (de) CK(cudaMemcpy(de, c->d_log_de, sizeof(double) * n_moves, cudaMemcpyDeviceToHost));
  if (draws_used) *draws_used = (long)st.stream_pos;
  if (st.error == PLUM_ERR_STREAM_DEV)
    return fail(PLUM_ERR_STREAM, "the recorded random stream ran out");
  if (st.error) return fail(st.error, "device reported an error during the moves");
  return PLUM_OK;
}

int plum_seed(plum_ctx* c, uint32_t seed) {
  if (!c) return fail(PLUM_ERR_INPUT, "null context");
  // std::mt19937::seed: mt[0] = s, mt[i] = 1812433253 (mt[i-1] ^ (mt[i-1] >> 30)) + i.
  uint32_t mt[625];
  mt[0] = seed;
  for (int i = 1; i < 624; i++) mt[i] = 1812433253u * (mt[i - 1] ^ (mt[i - 1] >> 30)) + (uint32_t)i;
  mt[624] = 624;
  cudaSetDevice(c->device);
  CK(cudaMemcpyAsync(c->d_mt, mt, sizeof(mt), cudaMemcpyHostToDevice, c->s));
  CK(cudaStreamSynchronize(c->s));
  c->gen_len = 0;
  return PLUM_OK;
}

int plum_run(plum_ctx* c, int n_moves, int* accepted_out) {
  if (!c || n_moves < 0) return fail(PLUM_ERR_INPUT, "bad argument");
  if (c->host_pending) return fail(PLUM_ERR_STATE, "a trial move is pending");
  if (c->in.use_gc) return fail(PLUM_ERR_INPUT, "grand-canonical steps are not run by this loop");
  cudaSetDevice(c->device);
  // Draw budget per step: 5 fixed draws + the move's own; a pivot consumes
  // 2 + len (2 r + 1) with r rejected pairs per randSphere (mean 1.27).
  const int batch = 256;
  const long long per_move = 16 + 12LL * c->max_len;
  const long long need = per_move * batch;
  const long long cap = std::max<long long>(4 * need, 1 << 22);
  int rc = ensure_stream(c, cap);
  if (rc) return rc;
  DevState st;
  rc = read_state(c, &st);
  if (rc) return rc;
  if (c->gen_len == 0) st.stream_pos = 0;
  st.step = 0;
  st.step_open = 0;
  st.error = 0;
  st.pending = 0;
  st.n_accept = 0;
  long long pos = st.stream_pos, len = c->gen_len;
  DevBuffers B = c->B;
  B.stream = c->d_stream;
  B.log_type = nullptr;
  B.log_accept = nullptr;
  B.log_etot = nullptr;
  B.log_step_de = nullptr;
  c->last_kernels = 0;
  CK(cudaEventRecord(c->ev0, c->s));
  int done = 0;
  while (done < n_moves) {
    // Keep at least `need` unread words: move the unread tail to the front
    // and generate the rest on the device.
    if (len - pos < need) {
      long long tail = len - pos;
      if (tail > 0)
        CK(cudaMemcpyAsync(c->d_stream, c->d_stream + pos, sizeof(uint32_t) * tail,
                           cudaMemcpyDeviceToDevice, c->s));
      launch_mt_fill(c->d_mt, c->d_stream + tail, cap - tail, c->s);
      c->last_kernels++;
      len = cap;
      pos = 0;
      st.stream_pos = 0;
    }
    st.stream_len = len;
    st.step = 0;
    st.step_open = 0;
    CK(cudaMemcpyAsync(c->B.state, &st, sizeof(DevState), cudaMemcpyHostToDevice, c->s));
    int nb = std::min(batch, n_moves - done);
    rc = device_loop(c, nb, B);
    if (rc) return rc;
    rc = read_state(c, &st);
    if (rc) return rc;
    if (st.error) break;
    pos = st.stream_pos;
    done += nb;
    c->since_recompute += nb;
    if (c->recompute_every > 0 && c->since_recompute >= c->recompute_every) {
      // Full FP64 recompute: resets the running totals, S(k) and the fixed-
      // point mirror; the difference is the drift accumulated since the last.
      double fresh[8];
      rc = total_energy(c, fresh);
      if (rc) return rc;
      double run[4] = {st.e_pair, st.e_ewald, st.e_bond, st.e_ext};
      double tot = 0.0;
      for (int q = 0; q < 4; q++) {
        c->drift[q] = run[q] - fresh[q];
        tot += c->drift[q];
      }
      c->drift_max = std::max(c->drift_max, std::fabs(tot));
      c->since_recompute = 0;
      rc = read_state(c, &st);
      if (rc) return rc;
      c->last_kernels += 5;
    }
  }
  CK(cudaEventRecord(c->ev1, c->s));
  CK(cudaStreamSynchronize(c->s));
  float ms = 0;
  cudaEventElapsedTime(&ms, c->ev0, c->ev1);
  c->last_ms = ms;
  c->gen_len = len;
  c->h_pos_valid = false;
  if (accepted_out) *accepted_out = st.n_accept;
  if (st.error == PLUM_ERR_STREAM_DEV) return fail(PLUM_ERR_STREAM, "device stream ran out");
  if (st.error) return fail(st.error, "device reported an error during the moves");
  return PLUM_OK;
}

int plum_time_kernels(plum_ctx* c, int n_moves, double* out2) {
  if (!c || n_moves <= 0 || !out2) return fail(PLUM_ERR_INPUT, "bad argument");
  c->kt_on = true;
  for (cudaEvent_t e : c->kt_ev) cudaEventDestroy(e);
  c->kt_ev.clear();
  c->kt_kind.clear();
  int rc = plum_run(c, n_moves, nullptr);
  c->kt_on = false;
  double sum[2] = {0, 0};
  int cnt[2] = {0, 0};
  for (size_t i = 0; i + 1 < c->kt_ev.size(); i++) {
    const int kind = c->kt_kind[i];
    if (kind > 1 || c->kt_kind[i + 1] != kind + 1) continue;
    float ms = 0;
    if (cudaEventElapsedTime(&ms, c->kt_ev[i], c->kt_ev[i + 1]) != cudaSuccess) continue;
    sum[kind] += ms;
    cnt[kind]++;
  }
  for (cudaEvent_t e : c->kt_ev) cudaEventDestroy(e);
  c->kt_ev.clear();
  c->kt_kind.clear();
  if (rc) return rc;
  for (int q = 0; q < 2; q++) out2[q] = cnt[q] ? sum[q] / cnt[q] : 0.0;
  return PLUM_OK;
}

int plum_get_positions(const plum_ctx* cc, double* xyz) {
  plum_ctx* c = const_cast<plum_ctx*>(cc);
  if (!c || !xyz) return fail(PLUM_ERR_INPUT, "null argument");
  cudaSetDevice(c->device);
  int rc = refresh_host_pos(c);
  if (rc) return rc;
  for (int i = 0; i < c->P.n_bead; i++) {
    xyz[3 * i] = c->h_pos[i].x;
    xyz[3 * i + 1] = c->h_pos[i].y;
    xyz[3 * i + 2] = c->h_pos[i].z;
  }
  return PLUM_OK;
}

int plum_set_positions(plum_ctx* c, const double* xyz) {
  if (!c || !xyz) return fail(PLUM_ERR_INPUT, "null argument");
  if (c->host_pending) return fail(PLUM_ERR_STATE, "a trial move is pending");
  cudaSetDevice(c->device);
  int rc = refresh_host_pos(c);
  if (rc) return rc;
  for (int i = 0; i < c->P.n_bead; i++) {
    c->h_pos[i].x = xyz[3 * i];
    c->h_pos[i].y = xyz[3 * i + 1];
    c->h_pos[i].z = xyz[3 * i + 2];
  }
  CK(cudaMemcpyAsync(c->B.pos, c->h_pos.data(), sizeof(double4_32a) * c->P.n_bead,
                     cudaMemcpyHostToDevice, c->s));
  CK(cudaMemcpyAsync(c->B.trial, c->h_pos.data(), sizeof(double4_32a) * c->P.n_bead,
                     cudaMemcpyHostToDevice, c->s));
  return total_energy(c, nullptr);
}

// Snapshot layout: a header of four ints {magic, n_bead, n_k, n_mol} and
// the form, then DevState, pos [n_bead], sk [n_k], dsk [2 n_k], bond_mol
// [n_mol], then the recompute bookkeeping {since_recompute, drift[4],
// drift_max}.
namespace {
constexpr int kSnapMagic = 0x504c4d53;  // "SMLP"
size_t snap_bytes(const plum_ctx* c) {
  return 5 * sizeof(int) + sizeof(DevState) + sizeof(double4_32a) * c->P.n_bead +
         sizeof(double2) * 3 * (size_t)c->P.n_k + sizeof(double) * c->P.n_mol +
         sizeof(long) + 5 * sizeof(double);
}
}  // namespace

long plum_ctx_snapshot_size(const plum_ctx* c) { return c ? (long)snap_bytes(c) : 0; }

int plum_ctx_save(const plum_ctx* cc, void* buf, long size) {
  plum_ctx* c = const_cast<plum_ctx*>(cc);
  if (!c || !buf || size < (long)snap_bytes(c)) return fail(PLUM_ERR_INPUT, "bad argument");
  if (c->host_pending) return fail(PLUM_ERR_STATE, "a trial move is pending");
  cudaSetDevice(c->device);
  unsigned char* p = static_cast<unsigned char*>(buf);
  const int head[5] = {kSnapMagic, c->P.n_bead, c->P.n_k, c->P.n_mol, c->form};
  std::memcpy(p, head, sizeof(head));
  p += sizeof(head);
  CK(cudaMemcpyAsync(p, c->B.state, sizeof(DevState), cudaMemcpyDeviceToHost, c->s));
  p += sizeof(DevState);
  CK(cudaMemcpyAsync(p, c->B.pos, sizeof(double4_32a) * c->P.n_bead, cudaMemcpyDeviceToHost,
                     c->s));
  p += sizeof(double4_32a) * c->P.n_bead;
  if (c->P.n_k > 0) {
    CK(cudaMemcpyAsync(p, c->B.sk, sizeof(double2) * c->P.n_k, cudaMemcpyDeviceToHost, c->s));
    CK(cudaMemcpyAsync(p + sizeof(double2) * c->P.n_k, c->B.dsk, sizeof(double2) * 2 * c->P.n_k,
                       cudaMemcpyDeviceToHost, c->s));
  }
  p += sizeof(double2) * 3 * (size_t)c->P.n_k;
  CK(cudaMemcpyAsync(p, c->B.bond_mol, sizeof(double) * c->P.n_mol, cudaMemcpyDeviceToHost,
                     c->s));
  p += sizeof(double) * c->P.n_mol;
  CK(cudaStreamSynchronize(c->s));
  std::memcpy(p, &c->since_recompute, sizeof(long));
  p += sizeof(long);
  std::memcpy(p, c->drift, 4 * sizeof(double));
  std::memcpy(p + 4 * sizeof(double), &c->drift_max, sizeof(double));
  return PLUM_OK;
}

int plum_ctx_load(plum_ctx* c, const void* buf, long size) {
  if (!c || !buf || size < (long)(5 * sizeof(int))) return fail(PLUM_ERR_INPUT, "bad argument");
  if (c->host_pending) return fail(PLUM_ERR_STATE, "a trial move is pending");
  const unsigned char* p = static_cast<const unsigned char*>(buf);
  int head[5];
  std::memcpy(head, p, sizeof(head));
  if (head[0] != kSnapMagic || head[1] != c->P.n_bead || head[2] != c->P.n_k ||
      head[3] != c->P.n_mol || head[4] != c->form || size < (long)snap_bytes(c))
    return fail(PLUM_ERR_INPUT, "the snapshot belongs to another system or form");
  cudaSetDevice(c->device);
  p += sizeof(head);
  CK(cudaStreamSynchronize(c->s));
  // the snapshot replaces the device state, the generator's stream cursor
  // included; it is then reset to an empty stream (plum_run refills it)
  DevState st;
  std::memcpy(&st, p, sizeof(DevState));
  st.stream_pos = st.stream_len = 0;
  p += sizeof(DevState);
  CK(cudaMemcpyAsync(c->B.state, &st, sizeof(DevState), cudaMemcpyHostToDevice, c->s));
  CK(cudaMemcpyAsync(c->B.pos, p, sizeof(double4_32a) * c->P.n_bead, cudaMemcpyHostToDevice,
                     c->s));
  CK(cudaMemcpyAsync(c->B.trial, p, sizeof(double4_32a) * c->P.n_bead, cudaMemcpyHostToDevice,
                     c->s));
  std::memcpy(c->h_pos.data(), p, sizeof(double4_32a) * c->P.n_bead);
  p += sizeof(double4_32a) * c->P.n_bead;
  if (c->P.n_k > 0) {
    CK(cudaMemcpyAsync(c->B.sk, p, sizeof(double2) * c->P.n_k, cudaMemcpyHostToDevice, c->s));
    CK(cudaMemcpyAsync(c->B.dsk, p + sizeof(double2) * c->P.n_k, sizeof(double2) * 2 * c->P.n_k,
                       cudaMemcpyHostToDevice, c->s));
  }
  p += sizeof(double2) * 3 * (size_t)c->P.n_k;
  CK(cudaMemcpyAsync(c->B.bond_mol, p, sizeof(double) * c->P.n_mol, cudaMemcpyHostToDevice,
                     c->s));
  p += sizeof(double) * c->P.n_mol;
  std::memcpy(&c->since_recompute, p, sizeof(long));
  p += sizeof(long);
  std::memcpy(c->drift, p, 4 * sizeof(double));
  std::memcpy(&c->drift_max, p + 4 * sizeof(double), sizeof(double));
  if (c->form == PLUM_FORM_FP32) launch_fix_all(c->P, c->B, c->s);  // the fixed-point mirror
  launch_fix64_all(c->P, c->B, c->s);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(c->s));
  c->h_pos_valid = true;
  c->gen_len = 0;
  return PLUM_OK;
}

int plum_structure_factor(const plum_ctx* cc, double* sk_out, int* kn_out) {
  plum_ctx* c = const_cast<plum_ctx*>(cc);
  if (!c) return fail(PLUM_ERR_INPUT, "null context");
  if (c->host_pending) return fail(PLUM_ERR_STATE, "a trial move is pending");
  cudaSetDevice(c->device);
  const int nk = c->P.use_ewald ? c->P.n_k : 0;
  if (nk == 0) return PLUM_OK;
  if (kn_out) {
    std::vector<short4> kn(nk);
    CK(cudaMemcpyAsync(kn.data(), c->B.kn, sizeof(short4) * nk, cudaMemcpyDeviceToHost, c->s));
    CK(cudaStreamSynchronize(c->s));
    for (int k = 0; k < nk; k++) {
      kn_out[3 * k] = kn[k].x;
      kn_out[3 * k + 1] = kn[k].y;
      kn_out[3 * k + 2] = kn[k].z;
    }
  }
  if (sk_out) {
    DevState st;
    int rc = read_state(c, &st);
    if (rc) return rc;
    std::vector<double2> sk(nk), add(nk);
    CK(cudaMemcpyAsync(sk.data(), c->B.sk, sizeof(double2) * nk, cudaMemcpyDeviceToHost, c->s));
    if (st.sk_pending)
      CK(cudaMemcpyAsync(add.data(), c->B.dsk + (size_t)st.sk_buf * nk, sizeof(double2) * nk,
                         cudaMemcpyDeviceToHost, c->s));
    CK(cudaStreamSynchronize(c->s));
    for (int k = 0; k < nk; k++) {
      sk_out[2 * k] = sk[k].x + (st.sk_pending ? add[k].x : 0.0);
      sk_out[2 * k + 1] = sk[k].y + (st.sk_pending ? add[k].y : 0.0);
    }
  }
  return PLUM_OK;
}

int plum_observables(const plum_ctx* cc, double* out) {
  plum_ctx* c = const_cast<plum_ctx*>(cc);
  if (!c || !out) return fail(PLUM_ERR_INPUT, "null argument");
  cudaSetDevice(c->device);
  launch_observables64(c->P, c->B, c->d_obs_per, c->d_out + 32, c->s);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(c->h_out, c->d_out + 32, sizeof(double) * 5, cudaMemcpyDeviceToHost, c->s));
  CK(cudaStreamSynchronize(c->s));
  std::memcpy(out, c->h_out, sizeof(double) * 5);
  return PLUM_OK;
}

int plum_chain_observables(const plum_ctx* cc, double* out, int cap, int* n_chains) {
  plum_ctx* c = const_cast<plum_ctx*>(cc);
  if (!c || (!out && cap > 0) || cap < 0) return fail(PLUM_ERR_INPUT, "bad argument");
  const Input& in = c->in;
  int n = 0;
  for (int m = 0; m < in.n_mol; m++) n += in.mol_start[m + 1] - in.mol_start[m] > 1;
  if (n_chains) *n_chains = n;
  if (cap == 0) return PLUM_OK;
  cudaSetDevice(c->device);
  launch_observables64(c->P, c->B, c->d_obs_per, c->d_out + 32, c->s);
  CK(cudaGetLastError());
  std::vector<double> per(5 * (size_t)in.n_mol);
  CK(cudaMemcpyAsync(per.data(), c->d_obs_per, sizeof(double) * per.size(),
                     cudaMemcpyDeviceToHost, c->s));
  CK(cudaStreamSynchronize(c->s));
  int i = 0;
  for (int m = 0; m < in.n_mol && i < cap; m++) {
    if (in.mol_start[m + 1] - in.mol_start[m] <= 1) continue;
    for (int q = 0; q < 5; q++) out[5 * i + q] = per[5 * (size_t)m + q];
    i++;
  }
  return PLUM_OK;
}

int plum_rhoz(const plum_ctx* cc, double* out, int cap, int* n_bins) {
  plum_ctx* c = const_cast<plum_ctx*>(cc);
  if (!c || (!out && cap > 0) || cap < 0) return fail(PLUM_ERR_INPUT, "bad argument");
  const int nb = c->rhoz_bins;
  if (n_bins) *n_bins = nb;
  if (cap == 0) return PLUM_OK;
  if (c->host_pending) return fail(PLUM_ERR_STATE, "a trial move is pending");
  cudaSetDevice(c->device);
  launch_rhoz(c->P, c->B, kRhoZRes, nb, c->d_rhoz, c->s);
  CK(cudaGetLastError());
  std::vector<unsigned> cnt(3 * (size_t)nb);
  CK(cudaMemcpyAsync(cnt.data(), c->d_rhoz, sizeof(unsigned) * cnt.size(),
                     cudaMemcpyDeviceToHost, c->s));
  CK(cudaStreamSynchronize(c->s));
  const double w = 1.0 / (c->in.box[0] * c->in.box[1] * kRhoZRes);
  const int n = std::min(cap, 3 * nb);
  for (int i = 0; i < n; i++) out[i] = cnt[i] * w;
  return PLUM_OK;
}

int plum_pressure_slit(plum_ctx* c, double* out6) {
  if (!c || !out6) return fail(PLUM_ERR_INPUT, "null argument");
  if (c->host_pending) return fail(PLUM_ERR_STATE, "a trial move is pending");
  cudaSetDevice(c->device);
  const Input& in = c->in;
  const DevParams& P = c->P;
  SlitPressParams S{};
  S.n_bead = P.n_bead;
  S.n_mol = P.n_mol;
  S.phantom = P.phantom;
  S.npbc = P.npbc;
  S.n_type = P.n_type;
  S.use_pair = in.use_pair;
  S.use_ewald = in.use_ewald;
  S.use_ext = in.use_ext;
  S.pair_kind = in.pair_kind;
  S.ext_kind = in.ext_kind;
  for (int a = 0; a < 3; a++) {
    S.box[a] = in.box[a];
    S.ebox[a] = P.ebox[a];
    S.real_cell[a] = P.real_cell[a];
  }
  S.lj_cut = in.lj_cut;
  S.lB = in.lB;
  S.alpha = in.alpha;
  S.real_cut = P.real_cut;
  S.evol = P.ebox[0] * P.ebox[1] * P.ebox[2];
  S.wall_cut = in.wall_cut;
  for (int t = 0; t < P.n_type && t < kSlitMaxTypes; t++) {
    auto il = in.lj.find(in.type_names[t]);
    S.lj_sig[t] = il != in.lj.end() ? il->second.sigma : 0.0;
    S.lj_eps[t] = il != in.lj.end() ? il->second.epsilon : 0.0;
    S.wall_sig[t] = P.wall_sig[t];
    S.wall_eps[t] = P.wall_eps[t];
    S.graft[t] = P.graft[t];
  }
  if (S.phantom < 0 || S.phantom > S.n_mol) return fail(PLUM_ERR_INPUT, "bad number of wall sites");
  const int* ms = in.mol_start.data();
  const long long n_pair = slit_pair_items(S, ms);
  const long long n_wall = slit_wall_items(S, ms);
  const int n_k = (S.use_ewald && S.phantom > 0) ? P.n_k : 0;
  int n1 = 0, n2 = 0;
  const int need = slit_partials_count(n_pair + n_wall, n_k, &n1, &n2);
  if (need > c->press_cap) {
    if (c->d_press) cudaFree(c->d_press);
    c->d_press = nullptr;
    c->press_cap = 0;
    if (dalloc(&c->d_press, need)) return PLUM_ERR_CUDA;
    c->press_cap = need;
  }
  launch_slit_pressure(S, c->B, n_pair, n_wall, ms[S.phantom], n_k, P.kunit, c->d_press, n1, n2,
                       c->s);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(c->h_out, c->d_press + 6 * (size_t)n1 + 3 * (size_t)n2, sizeof(double) * 6,
                     cudaMemcpyDeviceToHost, c->s));
  CK(cudaStreamSynchronize(c->s));
  std::memcpy(out6, c->h_out, sizeof(double) * 6);
  return PLUM_OK;
}

int plum_run_params(const plum_ctx* c, plum_run_info* o) {
  if (!c || !o) return fail(PLUM_ERR_INPUT, "null argument");
  const Input& in = c->in;
  std::memset(o, 0, sizeof(*o));
  o->steps = in.steps;
  o->steps_eq = in.steps_eq;
  o->sample_freq = in.sample_freq;
  o->stat_out_freq = in.stat_out_freq;
  o->traj_out_freq = in.traj_out_freq;
  o->beta = in.beta;
  o->move_size = in.move_size;
  for (int i = 0; i < 5; i++) o->move_prob[i] = in.move_prob[i];
  o->phantom = in.phantom;
  o->coion = in.coion;
  o->grafted = in.grafted;
  o->grafted_counterion = in.grafted_counterion;
  o->calc_chem_pot = in.calc_chem_pot;
  o->use_pair = in.use_pair;
  o->use_ewald = in.use_ewald;
  o->use_bond = in.use_bond;
  o->use_bond_rigid = in.use_rigid;
  o->use_ext = in.use_ext;
  o->use_gc = in.use_gc;
  o->gc_freq = in.gc_freq;
  o->rigid_bond = in.rigid;
  o->eq_bond = in.r0;
  std::snprintf(o->run_name, sizeof(o->run_name), "%s", in.run_name.c_str());
  return PLUM_OK;
}

int plum_get_topology(const plum_ctx* c, int* mol_start, double* q, int* type) {
  if (!c) return fail(PLUM_ERR_INPUT, "null context");
  const Input& in = c->in;
  if (mol_start) std::memcpy(mol_start, in.mol_start.data(), sizeof(int) * (in.n_mol + 1));
  if (q) std::memcpy(q, in.q.data(), sizeof(double) * in.q.size());
  if (type) std::memcpy(type, in.type.data(), sizeof(int) * in.type.size());
  return PLUM_OK;
}

int plum_type_name(const plum_ctx* c, int type, char* buf, int cap) {
  if (!c || !buf || cap <= 0) return fail(PLUM_ERR_INPUT, "bad argument");
  if (type < 0 || type >= (int)c->in.type_names.size()) return fail(PLUM_ERR_INPUT, "bad type");
  std::snprintf(buf, cap, "%s", c->in.type_names[type].c_str());
  return PLUM_OK;
}

// Uploads one growth step's trial sites and grown chain and fills the job
// (and, in the precision form, the one-launch kernel's layout).
static int cbmc_prepare(plum_ctx* c, int n_trials, const double* b1, const double* b2,
                        int chain_len, const double* chain, const double* chain_ci,
                        int delete_mol, CbmcJob* Jp, Cbmc32Layout* Gp) {
  if (!c || n_trials <= 0 || !b1 || chain_len < 0) return fail(PLUM_ERR_INPUT, "bad argument");
  const Input& in = c->in;
  if (!in.use_gc) return fail(PLUM_ERR_INPUT, "run.in has no grand-canonical species");
  const int charged = in.gc_bead_charge != 0;
  if (charged && (!b2 || (chain_len > 0 && !chain_ci)))
    return fail(PLUM_ERR_INPUT, "a charged species needs trial counterions");
  if (chain_len > 0 && !chain) return fail(PLUM_ERR_INPUT, "missing grown chain");
  if (c->host_pending) return fail(PLUM_ERR_STATE, "a trial move is pending");
  cudaSetDevice(c->device);
  const bool fp32 = c->form == PLUM_FORM_FP32;
  Cbmc32Layout G{};
  if (fp32) {
    G = cbmc32_layout(c->P, n_trials, chain_len);
    if (G.smem > cbmc32_max_smem())
      return fail(PLUM_ERR_INPUT, "too many trials or grown beads for the precision form's "
                                  "trial kernel");
  }
  const int cap = std::max(n_trials, std::max(chain_len, in.gc_chain_len));
  const int groups = cbmc_groups(c->P);
  if (cap > c->cb_cap) {
    cudaFree(c->cb_b);
    cudaFree(c->cb_c);
    cudaFree(c->cb_part);
    cudaFree(c->cb_u);
    int rc = dalloc(&c->cb_b, 2 * (size_t)cap) | dalloc(&c->cb_c, 2 * (size_t)cap) |
             dalloc(&c->cb_part, 2 * (size_t)cap * groups) | dalloc(&c->cb_u, cap);
    if (rc) return PLUM_ERR_CUDA;
    c->cb_cap = cap;
  }
  if (!c->cb_so && dalloc(&c->cb_so, std::max(1, c->P.n_k))) return PLUM_ERR_CUDA;
  if (fp32) {
    if (G.slots > c->cb_part32_cap) {
      cudaFree(c->cb_part32);
      c->cb_part32 = nullptr;
      if (dalloc(&c->cb_part32, (size_t)G.slots)) return PLUM_ERR_CUDA;
      c->cb_part32_cap = G.slots;
    }
    if (!c->cb_ticket) {
      if (dalloc(&c->cb_ticket, 1)) return PLUM_ERR_CUDA;
      CK(cudaMemsetAsync(c->cb_ticket, 0, sizeof(int), c->s));
    }
  }
  int type = (int)(std::find(in.type_names.begin(), in.type_names.end(), in.gc_symbol) -
                   in.type_names.begin());
  const double q1 = in.gc_bead_charge, q2 = -in.gc_bead_charge;
  std::vector<double4_32a> hb(2 * n_trials), hc(2 * std::max(chain_len, 1));
  for (int t = 0; t < n_trials; t++) {
    hb[t] = make_double4_32a(b1[3 * t], b1[3 * t + 1], b1[3 * t + 2], q1);
    hb[n_trials + t] = charged ? make_double4_32a(b2[3 * t], b2[3 * t + 1], b2[3 * t + 2], q2)
                               : hb[t];
  }
  for (int i = 0; i < chain_len; i++) {
    hc[i] = make_double4_32a(chain[3 * i], chain[3 * i + 1], chain[3 * i + 2], q1);
    hc[chain_len + i] = charged ? make_double4_32a(chain_ci[3 * i], chain_ci[3 * i + 1],
                                                   chain_ci[3 * i + 2], q2)
                                : hc[i];
  }
  CbmcJob J;
  J.n_trials = n_trials;
  J.charged = charged;
  J.cl = chain_len;
  J.type = type;
  J.ex_lo = J.ex_hi = 0;
  if (delete_mol >= 0) {
    const int last = delete_mol + (charged ? in.gc_chain_len : 0);
    if (last >= in.n_mol) return fail(PLUM_ERR_INPUT, "deleted molecule range out of bounds");
    J.ex_lo = in.mol_start[delete_mol];
    J.ex_hi = in.mol_start[last + 1];
  }
  // copies from pageable memory: the host vectors may go once these return
  CK(cudaMemcpyAsync(c->cb_b, hb.data(), sizeof(double4_32a) * 2 * n_trials,
                     cudaMemcpyHostToDevice, c->s));
  if (chain_len > 0)
    CK(cudaMemcpyAsync(c->cb_c, hc.data(), sizeof(double4_32a) * 2 * chain_len,
                       cudaMemcpyHostToDevice, c->s));
  J.b1 = c->cb_b;
  J.b2 = c->cb_b + n_trials;
  J.chain = c->cb_c;
  J.chain_ci = c->cb_c + chain_len;
  J.s_o = c->cb_so;
  J.part = fp32 ? c->cb_part32 : c->cb_part;
  J.u = c->cb_u;
  *Jp = J;
  *Gp = G;
  return PLUM_OK;
}

// One growth step's trial energies on the context's stream: one launch in the
// precision form, the FP64 kernels (S_o, system sweep, per-trial sums) in the
// plain form.
static int cbmc_launch(plum_ctx* c, const CbmcJob& J, const Cbmc32Layout& G) {
  if (c->form == PLUM_FORM_FP32) {
    if (launch_cbmc32(c->P, c->B, J, G, c->cb_ticket, c->s))
      return fail(PLUM_ERR_CUDA, cudaGetErrorString(cudaGetLastError()));
  } else {
    launch_cbmc(c->P, c->B, J, c->s);
  }
  CK(cudaGetLastError());
  return PLUM_OK;
}

int plum_cbmc_trials(plum_ctx* c, int n_trials, const double* b1, const double* b2,
                     int chain_len, const double* chain, const double* chain_ci, int delete_mol,
                     double* u_out) {
  if (!u_out) return fail(PLUM_ERR_INPUT, "bad argument");
  CbmcJob J;
  Cbmc32Layout G;
  int rc = cbmc_prepare(c, n_trials, b1, b2, chain_len, chain, chain_ci, delete_mol, &J, &G);
  if (rc) return rc;
  rc = cbmc_launch(c, J, G);
  if (rc) return rc;
  CK(cudaMemcpyAsync(u_out, c->cb_u, sizeof(double) * n_trials, cudaMemcpyDeviceToHost, c->s));
  CK(cudaStreamSynchronize(c->s));
  return PLUM_OK;
}

int plum_cbmc_time(plum_ctx* c, int n_trials, const double* b1, const double* b2, int chain_len,
                   const double* chain, const double* chain_ci, int delete_mol, int reps,
                   double* ms_out, int* launches_out) {
  if (!ms_out || reps <= 0) return fail(PLUM_ERR_INPUT, "bad argument");
  CbmcJob J;
  Cbmc32Layout G;
  int rc = cbmc_prepare(c, n_trials, b1, b2, chain_len, chain, chain_ci, delete_mol, &J, &G);
  if (rc) return rc;
  for (int i = 0; i < 3; i++)
    if ((rc = cbmc_launch(c, J, G))) return rc;
  CK(cudaEventRecord(c->ev0, c->s));
  for (int i = 0; i < reps; i++)
    if ((rc = cbmc_launch(c, J, G))) return rc;
  CK(cudaEventRecord(c->ev1, c->s));
  CK(cudaEventSynchronize(c->ev1));
  float ms = 0.0f;
  CK(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
  *ms_out = (double)ms / reps;
  if (launches_out)
    *launches_out = c->form == PLUM_FORM_FP32 ? 1 : ((c->P.use_ewald && c->P.n_k > 0) ? 3 : 2);
  return PLUM_OK;
}

int plum_collect_surrogate_data(plum_ctx* c, int n_moves, long cap, float* d_desc,
                                double* d_de, long* n_logged) {
  if (!c || n_moves < 0 || cap <= 0 || cap > (1L << 31) - 1 || !d_desc || !d_de)
    return fail(PLUM_ERR_INPUT, "bad argument");
  if (c->host_pending) return fail(PLUM_ERR_STATE, "a trial move is pending");
  cudaSetDevice(c->device);
  int rc = ensure_desc(c);
  if (rc) return rc;
  DevState st;
  rc = read_state(c, &st);
  if (rc) return rc;
  st.log_n = 0;
  st.log_cap = (int)cap;
  CK(cudaMemcpyAsync(c->B.state, &st, sizeof(DevState), cudaMemcpyHostToDevice, c->s));
  c->B.desc_acc = c->desc_acc;
  c->B.desc_fine = c->desc_fine;
  c->B.log_desc = d_desc;
  c->B.log_de = d_de;
  rc = plum_run(c, n_moves, nullptr);
  c->B.desc_acc = nullptr;
  c->B.desc_fine = nullptr;
  c->B.log_desc = nullptr;
  c->B.log_de = nullptr;
  int rc2 = read_state(c, &st);
  if (rc) return rc;
  if (rc2) return rc2;
  if (n_logged) *n_logged = st.log_n;
  st.log_cap = 0;
  CK(cudaMemcpyAsync(c->B.state, &st, sizeof(DevState), cudaMemcpyHostToDevice, c->s));
  CK(cudaStreamSynchronize(c->s));
  return PLUM_OK;
}

int plum_cbmc_trials_noalloc(plum_ctx* c, int n_trials, const double* d_b1, const double* d_b2,
                             int chain_len, const double* d_chain, const double* d_chain_ci,
                             int delete_mol, double* d_u_out, char* err, int err_cap) {
  auto say = [&](const char* m) {
    if (err && err_cap > 0) std::snprintf(err, (size_t)err_cap, "%s", m);
  };
  if (!c || !d_b1 || !d_u_out || (chain_len > 0 && !d_chain)) {
    say("plum_cbmc_trials_noalloc: null argument");
    return PLUM_ERR_INPUT;
  }
  const Input& in = c->in;
  if (!in.use_gc) {
    say("plum_cbmc_trials_noalloc: run.in has no grand-canonical species");
    return PLUM_ERR_INPUT;
  }
  const int charged = in.gc_bead_charge != 0;
  if (charged && (!d_b2 || (chain_len > 0 && !d_chain_ci))) {
    say("plum_cbmc_trials_noalloc: a charged species needs trial counterions");
    return PLUM_ERR_INPUT;
  }
  if (c->host_pending) {
    say("plum_cbmc_trials_noalloc: a trial move is pending");
    return PLUM_ERR_STATE;
  }
  int ex_lo = 0, ex_hi = 0;
  if (delete_mol >= 0) {
    const int last = delete_mol + (charged ? in.gc_chain_len : 0);
    if (last >= in.n_mol) {
      say("plum_cbmc_trials_noalloc: deleted molecule range out of bounds");
      return PLUM_ERR_INPUT;
    }
    ex_lo = in.mol_start[delete_mol];
    ex_hi = in.mol_start[last + 1];
  }
  int type = 0;
  while (type < (int)in.type_names.size() && in.type_names[type] != in.gc_symbol) type++;
  if (cudaSetDevice(c->device) != cudaSuccess) {
    say("plum_cbmc_trials_noalloc: cannot select the context's device");
    return PLUM_ERR_CUDA;
  }
  int rc = cbmc_trials_noalloc(c->P, c->B, c->s, c->device, n_trials, d_b1, d_b2, chain_len,
                               d_chain, d_chain_ci, type, charged, in.gc_bead_charge,
                               -in.gc_bead_charge, ex_lo, ex_hi, d_u_out, err, err_cap);
  return rc == 0 ? PLUM_OK : (rc == 1 ? PLUM_ERR_INPUT : PLUM_ERR_CUDA);
}

int plum_set_recompute(plum_ctx* c, long every) {
  if (!c || every < 0) return fail(PLUM_ERR_INPUT, "bad argument");
  c->recompute_every = every;
  c->since_recompute = 0;
  return PLUM_OK;
}

int plum_drift(const plum_ctx* c, double* out) {
  if (!c || !out) return fail(PLUM_ERR_INPUT, "null argument");
  for (int q = 0; q < 4; q++) out[q] = c->drift[q];
  out[4] = c->drift_max;
  return PLUM_OK;
}

int plum_probe_peaks(int device, double* fp32_tflops, double* fp64_tflops) {
  if (cudaSetDevice(device) != cudaSuccess) return fail(PLUM_ERR_CUDA, "cannot select device");
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  float* o32 = nullptr;
  double* o64 = nullptr;
  CK(cudaMalloc(&o32, sizeof(float)));
  CK(cudaMalloc(&o64, sizeof(double)));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int blocks = sms * 8, threads = 256;
  float ms = 0;
  // FP32: warm-up then timed
  const int it32 = 4096;
  k_fma_probe<float><<<blocks, threads>>>(o32, 64, 0.999f, 1e-4f);
  cudaEventRecord(e0);
  k_fma_probe<float><<<blocks, threads>>>(o32, it32, 0.999f, 1e-4f);
  cudaEventRecord(e1);
  CK(cudaEventSynchronize(e1));
  cudaEventElapsedTime(&ms, e0, e1);
  if (fp32_tflops) *fp32_tflops = 2.0 * 8 * it32 * (double)blocks * threads / (ms * 1e-3) / 1e12;
  const int it64 = 256;
  k_fma_probe<double><<<blocks, threads>>>(o64, 16, 0.999, 1e-4);
  cudaEventRecord(e0);
  k_fma_probe<double><<<blocks, threads>>>(o64, it64, 0.999, 1e-4);
  cudaEventRecord(e1);
  CK(cudaEventSynchronize(e1));
  cudaEventElapsedTime(&ms, e0, e1);
  if (fp64_tflops) *fp64_tflops = 2.0 * 8 * it64 * (double)blocks * threads / (ms * 1e-3) / 1e12;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(o32);
  cudaFree(o64);
  return PLUM_OK;
}

int plum_last_timing(const plum_ctx* c, double* ms, long* kernels) {
  if (!c) return fail(PLUM_ERR_INPUT, "null context");
  if (ms) *ms = c->last_ms;
  if (kernels) *kernels = c->last_kernels;
  return PLUM_OK;
}

}  // extern "C"

// ------------------------------------------------------------------ batches
struct plum_batch {
  std::vector<plum_ctx*> reps;
  int device = 0;
  cudaStream_t s = nullptr;
  DevParams* d_rp = nullptr;
  DevBuffers* d_rb = nullptr;
  int* d_item_off = nullptr;
  double* d_slots = nullptr;
  size_t kt_smem = 0;
  BatchTune tune{4096, 128, 0, 2, 1};
  float4* d_htab = nullptr;  // h(u) table of the real-space term (kH32Bins)
  bool htab_ok = false;      // every replica's alpha r_c^2 lies inside the table
  // the cut table (variable u' = cut_scale alpha r^2, zero from the cut-off on)
  // when every replica with the Ewald term has the same alpha and r_c; else
  // d_htab holds the universal table and cut_scale is 0
  float cut_scale = 0.0f;
  // per-replica streams
  std::vector<long long> cap, per_step;
  uint32_t** d_states = nullptr;
  uint32_t** d_outs = nullptr;
  DevState** d_sts = nullptr;
  long long *d_pos = nullptr, *d_len = nullptr, *d_cap = nullptr, *d_gather = nullptr;
  int* d_need = nullptr;
  long long* h_gather = nullptr;
  cudaGraphExec_t gexec = nullptr;
  int g_steps = 0;
  bool g_warm = false;
  int batch_steps = 32;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  double last_ms = 0;
  long last_kernels = 0;
  // delayed acceptance: descriptors [replicas][96] and the surrogate in use
  unsigned* d_desc = nullptr;
  unsigned* d_fine = nullptr;
  const plum_surrogate* sg = nullptr;
  int* d_err = nullptr;
  // descriptor cell lists (replicas that can have one)
  int* d_cells = nullptr;
  int* d_queue = nullptr;  // work queues of the batched energy change [2 groups][2]
  double* d_slots2 = nullptr;  // slots of the second group
  int groups = 1;
  cudaStream_t s2 = nullptr;
  cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
  int cell_moved = 0;     // longest molecule among them (0: none)
  bool cells_on = true;
  bool cells_built = false;  // a batch of steps with the surrogate has rebuilt them
  int max_bead = 0;
  std::vector<DevParams> h_rp;   // host copies of d_rp, d_rb
  std::vector<DevBuffers> h_rb;
  // full FP64 recompute of each replica every rc_every of its moves (0:
  // never); rc_since[r] counts replica r's moves since its last one. The
  // replicas start at staggered phases (r * rc_every / R), so every batch of
  // steps recomputes its share of them and any run of whole batches carries
  // the cost in proportion. d_drift [R][6] as k_assemble_total writes it.
  long rc_every = 10000;
  std::vector<long> rc_since;
  double* d_drift = nullptr;
  double* d_energies = nullptr;    // [R][4] gathered running totals
  std::vector<cudaEvent_t> rc_ev;  // start/end pairs around the recomputes of one run
  double rc_ms = 0.0;              // device time of the last run's recomputes
  long rc_count = 0;               // recomputes in the last run
};

namespace {

// One batch of steps: gen; then per step the exact energy change, finish +
// decide + gen. With a surrogate, each gen is followed by the descriptors of
// the generated chain moves and the surrogate's stage one, which marks the
// moves it rejects so that the delta kernel skips them.
// (Re)allocates the descriptor cell lists of the replicas that have one
// (h_rp[r].cell_cap > 0): per replica cell_key [n_bead], cell_n and
// cell_start [cells + 1] (ints), then on a 16-byte boundary cell_ent
// [n_bead] and cell_extra [cell_cap] (int4); then uploads the parameter and
// buffer tables.
int cells_alloc(plum_batch* b) {
  const int n = (int)b->reps.size();
  if (b->d_cells) {
    CK(cudaStreamSynchronize(b->s));
    cudaFree(b->d_cells);
    b->d_cells = nullptr;
  }
  auto head = [](const DevParams& P) {
    const size_t cells = (size_t)P.cell_nc[0] * P.cell_nc[1] * P.cell_nc[2];
    return ((size_t)P.n_bead + 2 * (cells + 1) + 3) / 4 * 4;
  };
  size_t words = 0;
  std::vector<size_t> off(n, 0);
  for (int r = 0; r < n; r++) {
    const DevParams& P = b->h_rp[r];
    if (!P.cell_cap) continue;
    off[r] = words;
    words += head(P) + 4 * ((size_t)P.n_bead + P.cell_cap);
  }
  if (words && dalloc(&b->d_cells, words)) return PLUM_ERR_CUDA;
  for (int r = 0; r < n; r++) {
    const DevParams& P = b->h_rp[r];
    DevBuffers& B = b->h_rb[r];
    if (!P.cell_cap) continue;
    const size_t cells = (size_t)P.cell_nc[0] * P.cell_nc[1] * P.cell_nc[2];
    B.cell_key = b->d_cells + off[r];
    B.cell_n = B.cell_key + P.n_bead;
    B.cell_start = B.cell_n + cells + 1;
    B.cell_ent = reinterpret_cast<int4*>(B.cell_key + head(P));
    B.cell_extra = B.cell_ent + P.n_bead;
  }
  if (b->d_rp) {
    CK(cudaMemcpyAsync(b->d_rp, b->h_rp.data(), sizeof(DevParams) * n, cudaMemcpyHostToDevice,
                       b->s));
    CK(cudaMemcpyAsync(b->d_rb, b->h_rb.data(), sizeof(DevBuffers) * n, cudaMemcpyHostToDevice,
                       b->s));
    CK(cudaStreamSynchronize(b->s));
  }
  b->cells_built = false;
  return PLUM_OK;
}

// Cell lists are rebuilt from the positions at the start of every batch of
// steps (or marked invalid when switched off).
void cells_enqueue(plum_batch* b) {
  if (b->sg && b->cell_moved)
    launch_cell_rebuild(b->d_rp, b->d_rb, (int)b->reps.size(), b->max_bead, b->cells_on, b->s);
}

// Kernel launches of batch_enqueue(b, steps).
long batch_kernels(const plum_batch* b, int steps) {
  const bool cells = b->sg && b->cell_moved;
  // descriptor (cell kernel, or the all-pairs kernel), smearing, inference
  const long stage = b->sg ? 3 : 0;
  const long chains = (b->groups > 1 && b->reps.size() > 1) ? 2 : 1;
  return (cells ? (b->cells_on ? 4 : 1) : 0) + chains * (1 + 2L * steps + steps * stage);
}

// After a batch of steps: when a replica's list of beads that changed cell
// overflowed, every list's capacity doubles (and the graph is captured again).
int cells_check(plum_batch* b) {
  if (!(b->sg && b->cell_moved && b->cells_on)) return PLUM_OK;
  if (!b->cells_built) {
    b->cells_built = true;
    return PLUM_OK;
  }
  bool over = false;
  for (size_t r = 0; r < b->reps.size(); r++)
    over |= b->h_rp[r].cell_cap && !b->h_gather[6 * r + 5];
  if (!over) return PLUM_OK;
  for (auto& P : b->h_rp)
    if (P.cell_cap) P.cell_cap *= 2;
  if (b->gexec) cudaGraphExecDestroy(b->gexec);
  b->gexec = nullptr;
  b->g_steps = 0;
  return cells_alloc(b);
}

// The step chain of replicas [r0, r0 + n) on stream st with its own slots
// and work queue.
void chain_enqueue(plum_batch* b, int steps, int r0, int n, double* slots, int* queue,
                   cudaStream_t st) {
  const DevParams* rp = b->d_rp + r0;
  const DevBuffers* rb = b->d_rb + r0;
  int* item_off = b->d_item_off + 4 * r0;
  auto stage_one = [&]() {
    if (!b->sg) return;
    launch_desc_batch(rp, rb, n, b->d_desc + (size_t)mlp::kIn * r0, 1,
                      b->cells_on ? b->cell_moved : 0, st);
    launch_mlp_infer_i(b->sg->net, b->d_desc + (size_t)mlp::kIn * r0, n, nullptr,
                       DaArgs{b->d_sts + r0, b->d_rp + r0}, b->d_err, st);
  };
  launch_batch_serial(rp, rb, item_off, slots, n, kModeGen, st);
  stage_one();
  for (int i = 0; i < steps; i++) {
    launch_batch_delta32(rp, rb, n, item_off, slots, b->kt_smem, b->tune, queue, b->d_htab,
                         b->cut_scale, st);
    int mode = kModeFinish | kModeDecide | (i + 1 < steps ? kModeGen : 0);
    launch_batch_serial(rp, rb, item_off, slots, n, mode, st);
    if (i + 1 < steps) stage_one();
  }
}

// One batch of steps. With two groups the replicas are split in halves whose
// chains run on two streams (two branches of the graph): one half's
// latency-bound kernels (serial step, descriptor, inference) overlap the
// other half's energy change.
void batch_enqueue(plum_batch* b, int steps) {
  const int R = (int)b->reps.size();
  cells_enqueue(b);
  if (b->groups < 2 || R < 2) {
    chain_enqueue(b, steps, 0, R, b->d_slots, b->d_queue, b->s);
    return;
  }
  const int h = R / 2;
  cudaEventRecord(b->fork_ev, b->s);
  cudaStreamWaitEvent(b->s2, b->fork_ev, 0);
  chain_enqueue(b, steps, 0, h, b->d_slots, b->d_queue, b->s);
  chain_enqueue(b, steps, h, R - h, b->d_slots2, b->d_queue + 2, b->s2);
  cudaEventRecord(b->join_ev, b->s2);
  cudaStreamWaitEvent(b->s, b->join_ev, 0);
}

int batch_steps_graph(plum_batch* b, int steps) {
  if (b->gexec && b->g_steps == steps) {
    CK(cudaGraphLaunch(b->gexec, b->s));
    return PLUM_OK;
  }
  if (b->g_warm) {
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(b->s, cudaStreamCaptureModeThreadLocal));
    batch_enqueue(b, steps);
    CK(cudaStreamEndCapture(b->s, &g));
    if (b->gexec) cudaGraphExecDestroy(b->gexec);
    b->gexec = nullptr;
    cudaError_t e = cudaGraphInstantiate(&b->gexec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return fail(PLUM_ERR_CUDA, cudaGetErrorString(e));
    b->g_steps = steps;
    CK(cudaGraphLaunch(b->gexec, b->s));
    return PLUM_OK;
  }
  b->g_warm = true;
  batch_enqueue(b, steps);
  CK(cudaGetLastError());
  return PLUM_OK;
}

// After a batch of `steps` steps: the full FP64 recompute (enqueue_total with
// drift) of every replica whose count reached rc_every, on the batch stream
// between CUDA events, so it is part of the run's device time. No move is
// pending between batches of steps (the last step of a batch only finishes
// and decides).
int batch_recompute_due(plum_batch* b, int steps, int* n_pairs) {
  if (b->rc_every <= 0) return PLUM_OK;
  const int R = (int)b->reps.size();
  bool any = false;
  for (int r = 0; r < R; r++) {
    b->rc_since[r] += steps;
    any |= b->rc_since[r] >= b->rc_every;
  }
  if (!any) return PLUM_OK;
  const int i = *n_pairs;
  while ((int)b->rc_ev.size() < 2 * (i + 1)) {
    cudaEvent_t e;
    CK(cudaEventCreate(&e));
    b->rc_ev.push_back(e);
  }
  CK(cudaEventRecord(b->rc_ev[2 * i], b->s));
  for (int r = 0; r < R; r++) {
    if (b->rc_since[r] < b->rc_every) continue;
    b->last_kernels += enqueue_total(b->reps[r], b->s, b->d_drift + 6 * r);
    b->rc_since[r] -= b->rc_every;
    b->rc_count++;
  }
  CK(cudaEventRecord(b->rc_ev[2 * i + 1], b->s));
  CK(cudaGetLastError());
  *n_pairs = i + 1;
  return PLUM_OK;
}

}  // namespace

extern "C" {

int plum_batch_energies(plum_batch* b, double* out) {
  if (!b || !out) return fail(PLUM_ERR_INPUT, "null argument");
  cudaSetDevice(b->device);
  const int R = (int)b->reps.size();
  // one gather launch and one copy for all replicas
  launch_gather_energies(b->d_sts, R, b->d_energies, b->s);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(out, b->d_energies, sizeof(double) * 4 * R, cudaMemcpyDeviceToHost, b->s));
  CK(cudaStreamSynchronize(b->s));
  return PLUM_OK;
}

int plum_batch_set_recompute(plum_batch* b, long every) {
  if (!b || every < 0) return fail(PLUM_ERR_INPUT, "bad argument");
  b->rc_every = every;
  const int R = (int)b->reps.size();
  for (int r = 0; r < R; r++) b->rc_since[r] = every ? (long)((long long)r * every / R) : 0;
  return PLUM_OK;
}

int plum_batch_drift(plum_batch* b, double* out, long* count, double* ms) {
  if (!b || !out) return fail(PLUM_ERR_INPUT, "null argument");
  cudaSetDevice(b->device);
  const int R = (int)b->reps.size();
  CK(cudaMemcpyAsync(out, b->d_drift, sizeof(double) * 6 * R, cudaMemcpyDeviceToHost, b->s));
  CK(cudaStreamSynchronize(b->s));
  if (count) *count = b->rc_count;
  if (ms) *ms = b->rc_ms;
  return PLUM_OK;
}

int plum_batch_destroy(plum_batch* b) {
  if (!b) return PLUM_OK;
  cudaSetDevice(b->device);
  if (b->s) cudaStreamSynchronize(b->s);
  for (plum_ctx* c : b->reps) plum_ctx_destroy(c);
  void* ptrs[] = {b->d_cells, b->d_queue, b->d_slots2, b->d_rp,    b->d_rb,  b->d_item_off, b->d_slots, b->d_states, b->d_outs,
                  b->d_sts,   b->d_pos, b->d_len,      b->d_cap,   b->d_gather, b->d_need,
                  b->d_desc,  b->d_err, b->d_fine,     b->d_drift,  b->d_energies,
                  b->d_htab};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  for (cudaEvent_t e : b->rc_ev) cudaEventDestroy(e);
  if (b->h_gather) cudaFreeHost(b->h_gather);
  if (b->gexec) cudaGraphExecDestroy(b->gexec);
  if (b->ev0) cudaEventDestroy(b->ev0);
  if (b->ev1) cudaEventDestroy(b->ev1);
  if (b->fork_ev) cudaEventDestroy(b->fork_ev);
  if (b->join_ev) cudaEventDestroy(b->join_ev);
  if (b->s2) cudaStreamDestroy(b->s2);
  if (b->s) cudaStreamDestroy(b->s);
  delete b;
  return PLUM_OK;
}

int plum_batch_create(int n, const char* const* dirs, const char* const* runins, int form,
                      int device, plum_batch** out) {
  if (!out || n <= 0 || !dirs || !runins) return fail(PLUM_ERR_INPUT, "bad argument");
  if (n > kMaxReplicas) return fail(PLUM_ERR_INPUT, "too many replicas");
  if (form != PLUM_FORM_FP32) return fail(PLUM_ERR_INPUT, "replica batches run the precision form");
  *out = nullptr;
  plum_batch* b = new plum_batch();
  b->device = device;
  for (int r = 0; r < n; r++) {
    plum_ctx* c = nullptr;
    int rc = plum_ctx_create(dirs[r], runins[r], form, device, &c);
    if (rc) {
      std::string msg = "replica " + std::to_string(r) + ": " + g_err;
      plum_batch_destroy(b);
      return fail(rc, msg);
    }
    if (c->in.use_gc) {
      plum_ctx_destroy(c);
      plum_batch_destroy(b);
      return fail(PLUM_ERR_INPUT, "grand-canonical replicas are not batched");
    }
    b->reps.push_back(c);
  }
  cudaSetDevice(device);
  if (cudaStreamCreateWithFlags(&b->s, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&b->s2, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->fork_ev, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->join_ev, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreate(&b->ev0) != cudaSuccess || cudaEventCreate(&b->ev1) != cudaSuccess) {
    plum_batch_destroy(b);
    return fail(PLUM_ERR_CUDA, "cannot create the batch's streams and events");
  }
  std::vector<DevParams> hp(n);
  std::vector<DevBuffers> hb(n);
  std::vector<uint32_t*> hst(n), hout(n);
  std::vector<DevState*> hsts(n);
  long long items = 0;
  b->cap.resize(n);
  b->per_step.resize(n);
  for (int r = 0; r < n; r++) {
    plum_ctx* c = b->reps[r];
    const DevParams& P = c->P;
    b->per_step[r] = 17 + 10LL * c->max_len;  // + the stage-one draw
    b->cap[r] = std::max<long long>(4 * b->batch_steps * b->per_step[r], 1 << 16);
    int rc = ensure_stream(c, b->cap[r]);
    if (rc) {
      plum_batch_destroy(b);
      return rc;
    }
    hp[r] = P;
    hb[r] = c->B;
    hb[r].stream = c->d_stream;
    hb[r].log_type = nullptr;
    hb[r].log_accept = nullptr;
    hb[r].log_etot = nullptr;
    hb[r].log_step_de = nullptr;
    hst[r] = c->d_mt;
    hout[r] = c->d_stream;
    hsts[r] = c->B.state;
    int most = 0;
    for (int m = 1; m <= c->max_len; m++)
      most = std::max(most, pair_item_count(m, P.n_bead, kMinItemPairs));
    items += most + (P.n_k + kMinKTile - 1) / kMinKTile;
    size_t sm = P.use_ewald ? (size_t)P.kchunk_delta * 2 * P.kper * sizeof(float2) : 0;
    b->kt_smem = std::max(b->kt_smem, sm);
    // staged moved beads of a pair item (trial and current int4, charge)
    b->kt_smem = std::max(b->kt_smem, (size_t)kPairGroup * (2 * sizeof(int4) + sizeof(float)));
  }
  int rc = 0;
  rc |= dalloc(&b->d_rp, n);
  rc |= dalloc(&b->d_rb, n);
  rc |= dalloc(&b->d_item_off, 4 * (size_t)n);
  rc |= dalloc(&b->d_slots, 2 * (size_t)items + 2);
  rc |= dalloc(&b->d_states, n);
  rc |= dalloc(&b->d_outs, n);
  rc |= dalloc(&b->d_sts, n);
  rc |= dalloc(&b->d_pos, n);
  rc |= dalloc(&b->d_len, n);
  rc |= dalloc(&b->d_cap, n);
  rc |= dalloc(&b->d_gather, 6 * (size_t)n);
  rc |= dalloc(&b->d_need, n);
  rc |= dalloc(&b->d_desc, (size_t)mlp::kIn * n);
  rc |= dalloc(&b->d_fine, (size_t)mlp::kFineAll * n);
  rc |= dalloc(&b->d_err, 1);
  rc |= dalloc(&b->d_queue, 4);
  rc |= dalloc(&b->d_slots2, 2 * (size_t)items + 2);
  rc |= dalloc(&b->d_drift, 6 * (size_t)n);
  rc |= dalloc(&b->d_energies, 4 * (size_t)n);
  rc |= dalloc(&b->d_htab, kH32Bins);
  if (rc) {
    plum_batch_destroy(b);
    return PLUM_ERR_CUDA;
  }
  cudaMemset(b->d_drift, 0, sizeof(double) * 6 * n);
  {
    // the h(u) table covers u = alpha r^2 < 2^kH32EHi; a replica whose
    // cut-off reaches past it keeps the erfc fit for the whole batch
    b->htab_ok = true;
    bool same = true;  // every Ewald replica has replica e0's alpha and r_c
    int e0 = -1;
    for (int r = 0; r < n; r++) {
      const DevParams& P = hp[r];
      if (!P.use_ewald) continue;
      if (P.sqrt_alpha * P.sqrt_alpha * P.real_cut * P.real_cut >= std::ldexp(1.0, kH32EHi))
        b->htab_ok = false;
      if (e0 < 0)
        e0 = r;
      else if (P.f_sqrt_alpha != hp[e0].f_sqrt_alpha || P.f_real_cut != hp[e0].f_real_cut)
        same = false;
    }
    std::vector<float4> h(kH32Bins);
    b->cut_scale = 0.0f;
    if (b->htab_ok && same && e0 >= 0) {
      const double a = hp[e0].f_sqrt_alpha, rcut = hp[e0].f_real_cut;
      b->cut_scale = (float)(kH32Cut / (a * a * rcut * rcut));
      build_h32_table(h.data(), (double)b->cut_scale, kH32Cut);
    } else {
      build_h32_table(h.data());
    }
    cudaMemcpy(b->d_htab, h.data(), sizeof(float4) * kH32Bins, cudaMemcpyHostToDevice);
    b->tune.htab = b->htab_ok ? 1 : 0;
  }
  b->rc_since.resize(n);
  for (int r = 0; r < n; r++) b->rc_since[r] = (long)((long long)r * b->rc_every / n);
  cudaMemset(b->d_err, 0, sizeof(int));
  cudaMemset(b->d_queue, 0, 4 * sizeof(int));
  for (int r = 0; r < n; r++) {
    hb[r].desc_acc = b->d_desc + (size_t)mlp::kIn * r;
    hb[r].desc_fine = b->d_fine + (size_t)mlp::kFineAll * r;
  }
  // descriptor cell lists: periodic on every axis with at least 3 cells of
  // the descriptor's cut per axis; cell_cap (the list of beads that changed
  // cell between rebuilds) = max(1024, n_bead / 16), doubled whenever it
  // overflowed during a batch of steps (that replica takes the all-pairs
  // kernel until the next rebuild)
  for (int r = 0; r < n; r++) {
    DevParams& P = hp[r];
    P.cell_cap = 0;
    if (P.form != 1 || P.npbc != 3) continue;
    int nc[3], cells = 1;
    bool ok = true;
    for (int a = 0; a < 3; a++) {
      nc[a] = (int)std::floor(P.ebox[a] / ((double)mlp::kDescCut * 1.001));
      nc[a] = std::min(nc[a], 64);
      ok = ok && nc[a] >= 3;
      cells *= std::max(nc[a], 1);
    }
    if (!ok) continue;
    for (int a = 0; a < 3; a++) P.cell_nc[a] = nc[a];
    P.cell_cap = std::max(1024, P.n_bead / 16);  // beads that change cell per batch of steps
    b->cell_moved = std::max(b->cell_moved, std::min(b->reps[r]->max_len, 512));
    b->max_bead = std::max(b->max_bead, P.n_bead);
  }
  // the cell kernel also takes the replicas without lists (all pairs): its
  // grid covers every replica's longest molecule
  if (b->cell_moved)
    for (int r = 0; r < n; r++)
      b->cell_moved = std::max(b->cell_moved, std::min(b->reps[r]->max_len, 512));
  b->h_rp = hp;
  b->h_rb = hb;
  if (b->cell_moved && cells_alloc(b)) {
    plum_batch_destroy(b);
    return PLUM_ERR_CUDA;
  }
  hp = b->h_rp;
  hb = b->h_rb;
  if (cudaMallocHost(&b->h_gather, sizeof(long long) * 6 * n) != cudaSuccess) {
    b->h_gather = nullptr;
    plum_batch_destroy(b);
    return fail(PLUM_ERR_CUDA, "cannot allocate pinned host memory");
  }
  cudaMemcpy(b->d_rp, hp.data(), sizeof(DevParams) * n, cudaMemcpyHostToDevice);
  cudaMemcpy(b->d_rb, hb.data(), sizeof(DevBuffers) * n, cudaMemcpyHostToDevice);
  cudaMemcpy(b->d_states, hst.data(), sizeof(uint32_t*) * n, cudaMemcpyHostToDevice);
  cudaMemcpy(b->d_outs, hout.data(), sizeof(uint32_t*) * n, cudaMemcpyHostToDevice);
  cudaMemcpy(b->d_sts, hsts.data(), sizeof(DevState*) * n, cudaMemcpyHostToDevice);
  cudaMemcpy(b->d_cap, b->cap.data(), sizeof(long long) * n, cudaMemcpyHostToDevice);
  cudaError_t e = cudaDeviceSynchronize();
  if (e != cudaSuccess) {
    plum_batch_destroy(b);
    return fail(PLUM_ERR_CUDA, cudaGetErrorString(e));
  }
  rc = plum_batch_seed(b, 1u);
  if (rc) {
    plum_batch_destroy(b);
    return rc;
  }
  *out = b;
  return PLUM_OK;
}

int plum_batch_seed(plum_batch* b, uint32_t seed) {
  if (!b) return fail(PLUM_ERR_INPUT, "null batch");
  std::vector<uint32_t> seeds(b->reps.size());
  for (size_t r = 0; r < seeds.size(); r++) seeds[r] = seed + (uint32_t)r;
  return plum_batch_seed_each(b, seeds.data());
}

int plum_batch_seed_each(plum_batch* b, const uint32_t* seeds) {
  if (!b || !seeds) return fail(PLUM_ERR_INPUT, "null argument");
  for (size_t r = 0; r < b->reps.size(); r++) {
    int rc = plum_seed(b->reps[r], seeds[r]);
    if (rc) return rc;
    // empty stream: the next run refills it
    DevState st;
    rc = read_state(b->reps[r], &st);
    if (rc) return rc;
    st.stream_pos = 0;
    st.stream_len = 0;
    st.pending = 0;
    st.error = 0;
    CK(cudaMemcpy(b->reps[r]->B.state, &st, sizeof(DevState), cudaMemcpyHostToDevice));
  }
  return PLUM_OK;
}

int plum_batch_run(plum_batch* b, int n_steps, long* accepted_out) {
  if (!b || n_steps < 0) return fail(PLUM_ERR_INPUT, "bad argument");
  cudaSetDevice(b->device);
  const int R = (int)b->reps.size();
  std::vector<int> need(R);
  std::vector<long long> pos(R), len(R);
  long long acc0 = 0, acc1 = 0;
  b->last_kernels = 0;
  b->rc_count = 0;
  b->rc_ms = 0.0;
  int n_pairs = 0;  // event pairs recorded around recomputes in this run
  CK(cudaEventRecord(b->ev0, b->s));
  int done = 0;
  bool first = true;
  while (done < n_steps) {
    const int steps = std::min(b->batch_steps, n_steps - done);
    launch_gather_states(b->d_sts, R, b->d_gather, b->s);
    CK(cudaMemcpyAsync(b->h_gather, b->d_gather, sizeof(long long) * 6 * R,
                       cudaMemcpyDeviceToHost, b->s));
    CK(cudaStreamSynchronize(b->s));
    bool any = false;
    for (int r = 0; r < R; r++) {
      const long long* g = b->h_gather + 6 * r;
      if (g[2]) return fail((int)g[2], "replica " + std::to_string(r) + " reported an error");
      if (first) acc0 += g[3];
      pos[r] = g[0];
      len[r] = g[1];
      need[r] = len[r] - pos[r] < (long long)steps * b->per_step[r];
      any |= need[r] != 0;
    }
    first = false;
    const int crc = cells_check(b);
    if (crc) return crc;
    if (any) {
      CK(cudaMemcpyAsync(b->d_need, need.data(), sizeof(int) * R, cudaMemcpyHostToDevice, b->s));
      CK(cudaMemcpyAsync(b->d_pos, pos.data(), sizeof(long long) * R, cudaMemcpyHostToDevice, b->s));
      CK(cudaMemcpyAsync(b->d_len, len.data(), sizeof(long long) * R, cudaMemcpyHostToDevice, b->s));
      launch_mt_fill_batch(b->d_states, b->d_outs, b->d_pos, b->d_len, b->d_cap, b->d_need,
                           b->d_sts, R, b->s);
      b->last_kernels++;
    }
    int rc = batch_steps_graph(b, steps);
    if (rc) return rc;
    b->last_kernels += batch_kernels(b, steps);
    done += steps;
    rc = batch_recompute_due(b, steps, &n_pairs);
    if (rc) return rc;
  }
  CK(cudaEventRecord(b->ev1, b->s));
  launch_gather_states(b->d_sts, R, b->d_gather, b->s);
  CK(cudaMemcpyAsync(b->h_gather, b->d_gather, sizeof(long long) * 6 * R, cudaMemcpyDeviceToHost,
                     b->s));
  CK(cudaStreamSynchronize(b->s));
  float ms = 0;
  cudaEventElapsedTime(&ms, b->ev0, b->ev1);
  b->last_ms = ms;
  for (int i = 0; i < n_pairs; i++) {
    float t = 0;
    cudaEventElapsedTime(&t, b->rc_ev[2 * i], b->rc_ev[2 * i + 1]);
    b->rc_ms += t;
  }
  for (int r = 0; r < R; r++) {
    const long long* g = b->h_gather + 6 * r;
    if (g[2] == PLUM_ERR_STREAM_DEV) return fail(PLUM_ERR_STREAM, "replica stream ran out");
    if (g[2]) return fail((int)g[2], "replica " + std::to_string(r) + " reported an error");
    acc1 += g[3];
    b->reps[r]->h_pos_valid = false;
  }
  if (b->sg) {
    int e = 0;
    CK(cudaMemcpy(&e, b->d_err, sizeof(int), cudaMemcpyDeviceToHost));
    if (e) return fail(PLUM_ERR_TIMEOUT, "tensor-core wait timed out in the surrogate stage");
  }
  if (accepted_out) *accepted_out = (long)(acc1 - acc0);
  return PLUM_OK;
}

int plum_batch_time_kernels(plum_batch* b, int n_steps, double* out4) {
  if (!b || n_steps <= 0 || !out4) return fail(PLUM_ERR_INPUT, "bad argument");
  cudaSetDevice(b->device);
  const int R = (int)b->reps.size();
  // the stream words these steps need (as plum_batch_run refills them)
  launch_gather_states(b->d_sts, R, b->d_gather, b->s);
  CK(cudaMemcpyAsync(b->h_gather, b->d_gather, sizeof(long long) * 6 * R, cudaMemcpyDeviceToHost,
                     b->s));
  CK(cudaStreamSynchronize(b->s));
  std::vector<int> need(R);
  std::vector<long long> pos(R), len(R);
  bool any = false;
  for (int r = 0; r < R; r++) {
    const long long* g = b->h_gather + 6 * r;
    if (g[2]) return fail((int)g[2], "replica " + std::to_string(r) + " reported an error");
    pos[r] = g[0];
    len[r] = g[1];
    need[r] = len[r] - pos[r] < (long long)(n_steps + 1) * b->per_step[r];
    any |= need[r] != 0;
  }
  if ((long long)(n_steps + 1) * *std::max_element(b->per_step.begin(), b->per_step.end()) >
      *std::min_element(b->cap.begin(), b->cap.end()))
    return fail(PLUM_ERR_INPUT, "too many steps for one timing run");
  if (any) {
    CK(cudaMemcpyAsync(b->d_need, need.data(), sizeof(int) * R, cudaMemcpyHostToDevice, b->s));
    CK(cudaMemcpyAsync(b->d_pos, pos.data(), sizeof(long long) * R, cudaMemcpyHostToDevice, b->s));
    CK(cudaMemcpyAsync(b->d_len, len.data(), sizeof(long long) * R, cudaMemcpyHostToDevice, b->s));
    launch_mt_fill_batch(b->d_states, b->d_outs, b->d_pos, b->d_len, b->d_cap, b->d_need,
                         b->d_sts, R, b->s);
  }
  cells_enqueue(b);
  // events around every kernel of the steps (plain launches, no graph)
  std::vector<cudaEvent_t> ev(2 * (4 * n_steps + 4));
  for (auto& e : ev) CK(cudaEventCreate(&e));
  int k = 0;
  std::vector<std::pair<int, int>> marks;  // (kind, event index of the start)
  auto timed = [&](int kind, auto&& launch) {
    CK(cudaEventRecord(ev[k], b->s));
    launch();
    CK(cudaEventRecord(ev[k + 1], b->s));
    marks.push_back({kind, k});
    k += 2;
    return PLUM_OK;
  };
  auto stage_one = [&]() {
    if (!b->sg) return PLUM_OK;
    int rc = timed(2, [&] {
      launch_desc_batch(b->d_rp, b->d_rb, R, b->d_desc, 1, b->cells_on ? b->cell_moved : 0, b->s);
    });
    if (rc) return rc;
    return timed(3, [&] {
      launch_mlp_infer_i(b->sg->net, b->d_desc, R, nullptr, DaArgs{b->d_sts, b->d_rp}, b->d_err,
                         b->s);
    });
  };
  int rc = timed(1, [&] {
    launch_batch_serial(b->d_rp, b->d_rb, b->d_item_off, b->d_slots, R, kModeGen, b->s);
  });
  if (!rc) rc = stage_one();
  for (int i = 0; i < n_steps && !rc; i++) {
    rc = timed(0, [&] {
      launch_batch_delta32(b->d_rp, b->d_rb, R, b->d_item_off, b->d_slots, b->kt_smem, b->tune,
                         b->d_queue, b->d_htab, b->cut_scale, b->s);
    });
    const int mode = kModeFinish | kModeDecide | (i + 1 < n_steps ? kModeGen : 0);
    if (!rc)
      rc = timed(1, [&] {
        launch_batch_serial(b->d_rp, b->d_rb, b->d_item_off, b->d_slots, R, mode, b->s);
      });
    if (!rc && i + 1 < n_steps) rc = stage_one();
  }
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(b->s));
  double sum[4] = {0, 0, 0, 0};
  int cnt[4] = {0, 0, 0, 0};
  for (auto& m : marks) {
    float ms = 0;
    cudaEventElapsedTime(&ms, ev[m.second], ev[m.second + 1]);
    sum[m.first] += ms;
    cnt[m.first]++;
  }
  for (auto& e : ev) cudaEventDestroy(e);
  if (rc) return rc;
  for (int q = 0; q < 4; q++) out4[q] = cnt[q] ? sum[q] / cnt[q] : 0.0;
  for (plum_ctx* c : b->reps) c->h_pos_valid = false;
  return PLUM_OK;
}

int plum_batch_set_tune(plum_batch* b, int item_pairs, int k_tile, int grid, int min_blocks) {
  if (!b || item_pairs < kMinItemPairs || item_pairs % 256 || k_tile < kMinKTile ||
      k_tile > 4 * kPairThreads || (k_tile > kPairThreads && k_tile % kPairThreads) ||
      grid < 0 || grid > 65535 || min_blocks < 2 || min_blocks > 4)
    return fail(PLUM_ERR_INPUT, "bad work-item sizes");
  b->tune = BatchTune{item_pairs, k_tile, grid, min_blocks, b->tune.htab};
  if (b->gexec) cudaGraphExecDestroy(b->gexec);
  b->gexec = nullptr;
  b->g_steps = 0;
  return PLUM_OK;
}

int plum_batch_descriptors(plum_batch* b, float* out) {
  if (!b || !out) return fail(PLUM_ERR_INPUT, "bad argument");
  cudaSetDevice(b->device);
  const size_t n = (size_t)mlp::kIn * b->reps.size();
  std::vector<unsigned> h(n);
  CK(cudaMemcpyAsync(h.data(), b->d_desc, sizeof(unsigned) * n, cudaMemcpyDeviceToHost, b->s));
  CK(cudaStreamSynchronize(b->s));
  for (size_t i = 0; i < n; i++) out[i] = (float)h[i] * mlp::kDescUnit;
  return PLUM_OK;
}

int plum_batch_cell_stats(plum_batch* b, int* out4) {
  if (!b || !out4) return fail(PLUM_ERR_INPUT, "bad argument");
  cudaSetDevice(b->device);
  int with = 0, ok = 0, most = 0, cap = 0;
  std::vector<DevBuffers> hb(b->reps.size());
  std::vector<DevParams> hp(b->reps.size());
  CK(cudaMemcpyAsync(hb.data(), b->d_rb, sizeof(DevBuffers) * hb.size(), cudaMemcpyDeviceToHost,
                     b->s));
  CK(cudaMemcpyAsync(hp.data(), b->d_rp, sizeof(DevParams) * hp.size(), cudaMemcpyDeviceToHost,
                     b->s));
  CK(cudaStreamSynchronize(b->s));
  for (size_t r = 0; r < b->reps.size(); r++) {
    if (!hp[r].cell_cap || !hb[r].cell_n) continue;
    with++;
    cap = std::max(cap, hp[r].cell_cap);
    DevState st;
    int rc = read_state(b->reps[r], &st);
    if (rc) return rc;
    ok += st.cell_ok ? 1 : 0;
    const int cells = hp[r].cell_nc[0] * hp[r].cell_nc[1] * hp[r].cell_nc[2];
    int used = 0;
    CK(cudaMemcpyAsync(&used, hb[r].cell_n + cells, sizeof(int), cudaMemcpyDeviceToHost, b->s));
    CK(cudaStreamSynchronize(b->s));
    most = std::max(most, used);
  }
  out4[0] = with;
  out4[1] = ok;
  out4[2] = most;
  out4[3] = cap;
  return PLUM_OK;
}

int plum_batch_set_groups(plum_batch* b, int groups) {
  if (!b || groups < 1 || groups > 2) return fail(PLUM_ERR_INPUT, "groups must be 1 or 2");
  b->groups = groups;
  if (b->gexec) cudaGraphExecDestroy(b->gexec);
  b->gexec = nullptr;
  b->g_steps = 0;
  return PLUM_OK;
}

int plum_batch_set_cell_cap(plum_batch* b, int cap) {
  if (!b || cap < 1 || cap > (1 << 20)) return fail(PLUM_ERR_INPUT, "bad argument");
  cudaSetDevice(b->device);
  if (!b->cell_moved) return PLUM_OK;
  for (auto& P : b->h_rp)
    if (P.cell_cap) P.cell_cap = cap;
  if (b->gexec) cudaGraphExecDestroy(b->gexec);
  b->gexec = nullptr;
  b->g_steps = 0;
  return cells_alloc(b);
}

int plum_batch_set_cells(plum_batch* b, int on) {
  if (!b) return fail(PLUM_ERR_INPUT, "null batch");
  b->cells_on = on != 0;
  b->cells_built = false;
  if (b->gexec) cudaGraphExecDestroy(b->gexec);
  b->gexec = nullptr;
  b->g_steps = 0;
  return PLUM_OK;
}

int plum_batch_autotune(plum_batch* b, int steps, int* out4) {
  if (!b || steps <= 0) return fail(PLUM_ERR_INPUT, "bad argument");
  int sms = 152;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device);
  const int pairs[] = {4096, 8192, 16384, 32768};
  const int ktiles[] = {128, 256, 512, 1024};
  const int per_sm[] = {2, 3, 4, 6, 8};
  const int occ[] = {2, 3, 4};
  double best = 1e300;
  BatchTune pick = b->tune;
  for (int mb : occ)
    for (int ip : pairs)
      for (int kt : ktiles)
        for (int ps : per_sm) {
          b->tune = BatchTune{ip, kt, ps * sms, mb, b->htab_ok ? 1 : 0};
          double ms[4];
          int rc = plum_batch_time_kernels(b, steps, ms);
          if (rc) return rc;
          if (ms[0] < best) {
            best = ms[0];
            pick = b->tune;
          }
        }
  if (pick.htab) {
    // the erfc fit at the chosen sizes, kept if it is faster
    b->tune = pick;
    b->tune.htab = 0;
    double ms[4];
    int rc = plum_batch_time_kernels(b, steps, ms);
    if (rc) return rc;
    if (ms[0] < best) pick = b->tune;
  }
  b->tune.htab = pick.htab;
  int rc = plum_batch_set_tune(b, pick.item_pairs, pick.k_tile, pick.grid, pick.min_blocks);
  if (rc) return rc;
  if (out4) {
    out4[0] = pick.item_pairs;
    out4[1] = pick.k_tile;
    out4[2] = pick.grid;
    out4[3] = pick.min_blocks;
  }
  return PLUM_OK;
}

int plum_batch_set_real_term(plum_batch* b, int table) {
  if (!b) return fail(PLUM_ERR_INPUT, "null batch");
  if (table && !b->htab_ok)
    return fail(PLUM_ERR_INPUT, "a replica's real-space cut-off lies outside the h(u) table");
  b->tune.htab = table ? 1 : 0;
  if (b->gexec) cudaGraphExecDestroy(b->gexec);
  b->gexec = nullptr;
  b->g_steps = 0;
  return PLUM_OK;
}

int plum_batch_real_term(const plum_batch* b) { return b ? b->tune.htab : -1; }

int plum_h64_table(double* out, int cap) {
  std::vector<double> h((size_t)kH64Bins * kH64Stride);
  build_h64_table(h.data());
  for (int i = 0; i < std::min(cap, kH64Bins); i++)
    for (int q = 0; q < kH64Stride; q++) out[(size_t)i * kH64Stride + q] = h[(size_t)i * kH64Stride + q];
  return kH64Bins;
}

int plum_h32_table(float* out, int cap, double scale, double cut) {
  if (!(scale > 0.0) || !(cut >= 0.0)) {
    fail(PLUM_ERR_INPUT, "table scale must be > 0, cut >= 0");
    return -1;
  }
  std::vector<float4> h(kH32Bins);
  build_h32_table(h.data(), scale, cut);
  for (int i = 0; i < std::min(cap, kH32Bins); i++) {
    out[4 * i] = h[i].x;
    out[4 * i + 1] = h[i].y;
    out[4 * i + 2] = h[i].z;
    out[4 * i + 3] = h[i].w;
  }
  return kH32Bins;
}

int plum_batch_set_surrogate(plum_batch* b, const plum_surrogate* sg) {
  if (!b) return fail(PLUM_ERR_INPUT, "null batch");
  if (sg && sg->device != b->device)
    return fail(PLUM_ERR_INPUT, "the surrogate lives on another device");
  cudaSetDevice(b->device);
  if (sg) CK(cudaStreamSynchronize(sg->s));
  for (plum_ctx* c : b->reps) {
    DevState st;
    int rc = read_state(c, &st);
    if (rc) return rc;
    st.da_on = sg ? 1 : 0;
    st.da_active = 0;
    st.da_skip = 0;
    st.da_n_moves = st.da_n_pass = st.da_n_accept = 0;
    CK(cudaMemcpy(c->B.state, &st, sizeof(DevState), cudaMemcpyHostToDevice));
  }
  b->sg = sg;
  b->cells_built = false;
  if (b->gexec) cudaGraphExecDestroy(b->gexec);
  b->gexec = nullptr;
  b->g_steps = 0;
  b->g_warm = false;
  return PLUM_OK;
}

int plum_batch_da_stats(plum_batch* b, long* out3) {
  if (!b || !out3) return fail(PLUM_ERR_INPUT, "null argument");
  cudaSetDevice(b->device);
  out3[0] = out3[1] = out3[2] = 0;
  int e = 0;
  CK(cudaMemcpy(&e, b->d_err, sizeof(int), cudaMemcpyDeviceToHost));
  if (e) return fail(PLUM_ERR_TIMEOUT, "tensor-core wait timed out in the surrogate stage");
  for (plum_ctx* c : b->reps) {
    DevState st;
    int rc = read_state(c, &st);
    if (rc) return rc;
    out3[0] += st.da_n_moves;
    out3[1] += st.da_n_pass;
    out3[2] += st.da_n_accept;
  }
  return PLUM_OK;
}

int plum_batch_size(const plum_batch* b) { return b ? (int)b->reps.size() : 0; }

int plum_batch_replica(plum_batch* b, int r, plum_ctx** ctx) {
  if (!b || !ctx || r < 0 || r >= (int)b->reps.size()) return fail(PLUM_ERR_INPUT, "bad replica");
  *ctx = b->reps[r];
  return PLUM_OK;
}

int plum_batch_last_timing(const plum_batch* b, double* ms, long* kernels) {
  if (!b) return fail(PLUM_ERR_INPUT, "null batch");
  if (ms) *ms = b->last_ms;
  if (kernels) *kernels = b->last_kernels;
  return PLUM_OK;
}

}  // extern "C"
