// Configurational-bias trial-site energies (ForceField::BeadsEnergy,
// cbmc.cc:5-151) for all trial sites of one growth step at once.
//
//   k_cbmc_so     S_o(k): the committed S(k) (plus any pending accepted
//                 change), minus the molecules being deleted, plus the grown
//                 chain and its counterions
//   k_cbmc_sys    grid (bead groups) x (trials): LJ and real-space Ewald of
//                 each trial bead (and its trial counterion) with every
//                 system bead outside the deleted molecules; per-block sums
//   k_cbmc_fin    one block per trial: the block sums in order, the grown
//                 chain terms (no LJ with the preceding grown bead,
//                 cbmc.cc:57-58), bead-counterion cross terms, self terms,
//                 k-space |S_o + q1 e1 + q2 e2|^2 - |S_o|^2, walls, dipole
//                 change; 1e8 when the pair sum reaches 1e8 (cbmc.cc:146-148)
// The arithmetic is the plain form's (FP64) with the same pair functions as
// the move kernels.
#include <cstdio>
#include <mutex>

#include "device_common.cuh"
#include "engine.h"

namespace plum {

// pair helpers shared with kern_energy.cu (same formulas, inlined here)
__device__ __forceinline__ double cb_wrap(double d, double L, double invL) {
  return d - L * rint(d * invL);
}

__device__ __forceinline__ double cb_lj(const DevParams& P, int ta, int tb, double4_32a a,
                                        double4_32a b) {
  double x = cb_wrap(b.x - a.x, P.box[0], P.inv_box[0]);
  double y = cb_wrap(b.y - a.y, P.box[1], P.inv_box[1]);
  double z = P.npbc > 2 ? cb_wrap(b.z - a.z, P.box[2], P.inv_box[2]) : b.z - a.z;
  double r2 = x * x + y * y + z * z;
  int k = ta * P.n_type + tb;
  if (P.pair_kind == 1) return sqrt(r2) <= P.hs_sum[k] ? kVeryLarge : 0.0;  // hard spheres
  if (r2 <= 0.0) return kVeryLarge;
  if (r2 < P.lj_rc2[k]) {
    double s2 = P.lj_sig2[k] / r2;
    double s6 = s2 * s2 * s2;
    return P.lj_eps4[k] * (s6 * s6 - s6) - P.lj_eref[k];
  }
  return 0.0;
}

__device__ __forceinline__ double cb_real(const DevParams& P, double4_32a a, double4_32a b) {
  double qq = a.w * b.w;
  if (qq == 0.0) return 0.0;
  double dx = cb_wrap(b.x - a.x, P.ebox[0], P.inv_ebox[0]);
  double dy = cb_wrap(b.y - a.y, P.ebox[1], P.inv_ebox[1]);
  double dz = P.npbc > 2 ? cb_wrap(b.z - a.z, P.ebox[2], P.inv_ebox[2]) : b.z - a.z;
  double e = 0.0;
  const double rc = P.real_cut;
  for (int i = -P.real_cell[0]; i <= P.real_cell[0]; i++) {
    double x = dx + i * P.ebox[0];
    if (fabs(x) > rc) continue;
    for (int j = -P.real_cell[1]; j <= P.real_cell[1]; j++) {
      double y = dy + j * P.ebox[1];
      if (fabs(y) > rc) continue;
      for (int k = -P.real_cell[2]; k <= P.real_cell[2]; k++) {
        double z = dz + k * P.ebox[2];
        if (fabs(z) > rc) continue;
        const double r2 = x * x + y * y + z * z;
        if (r2 > 0.0 && r2 <= rc * rc) e += real_term64(P, r2);
      }
    }
  }
  return P.lB * qq * e;
}

__device__ __forceinline__ double2 cb_phase(const DevParams& P, short4 kn, double4_32a p) {
  double w[3] = {p.x, p.y, p.z};
  for (int a = 0; a < P.npbc; a++) w[a] -= P.ebox[a] * floor(w[a] * P.inv_ebox[a]);
  double ph = kn.x * P.kunit[0] * w[0] + kn.y * P.kunit[1] * w[1] + kn.z * P.kunit[2] * w[2];
  double s, c;
  sincos(ph, &s, &c);
  return make_double2(p.w * c, p.w * s);
}

__global__ void k_cbmc_so(const DevParams P, const DevBuffers B, CbmcJob J) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= P.n_k) return;
  const DevState* st = B.state;
  const short4 kn = B.kn[k];
  double2 s = B.sk[k];
  if (st->sk_pending) {
    double2 d = B.dsk[(size_t)st->sk_buf * P.n_k + k];
    s.x += d.x;
    s.y += d.y;
  }
  for (int j = J.ex_lo; j < J.ex_hi; j++) {
    double2 e = cb_phase(P, kn, B.pos[j]);
    s.x -= e.x;
    s.y -= e.y;
  }
  for (int i = 0; i < J.cl; i++) {
    double2 e = cb_phase(P, kn, J.chain[i]);
    s.x += e.x;
    s.y += e.y;
    if (J.charged) {
      e = cb_phase(P, kn, J.chain_ci[i]);
      s.x += e.x;
      s.y += e.y;
    }
  }
  J.s_o[k] = s;
}

template <int NT>
__device__ __forceinline__ double cb_bsum(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) sh[w] = v;
  __syncthreads();
  double t = 0.0;
  for (int i = 0; i < NT / 32; i++) t += sh[i];
  __syncthreads();
  return t;
}

constexpr int kCbThreads = 256;

__global__ void __launch_bounds__(kCbThreads)
    k_cbmc_sys(const DevParams P, const DevBuffers B, CbmcJob J) {
  __shared__ double red[kCbThreads / 32];
  const int t = blockIdx.y;
  const double4_32a b1 = J.b1[t];
  const double4_32a b2 = J.charged ? J.b2[t] : b1;
  double lj = 0.0, re = 0.0;
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < P.n_bead; j += gridDim.x * blockDim.x) {
    if (j >= J.ex_lo && j < J.ex_hi) continue;
    const double4_32a pj = B.pos[j];
    const int tj = B.type[j];
    if (P.use_pair) {
      lj += cb_lj(P, J.type, tj, b1, pj);
      if (J.charged) lj += cb_lj(P, J.type, tj, b2, pj);
    }
    if (P.use_ewald) {
      re += cb_real(P, b1, pj);
      if (J.charged) re += cb_real(P, b2, pj);
    }
  }
  lj = cb_bsum<kCbThreads>(lj, red);
  re = cb_bsum<kCbThreads>(re, red);
  if (threadIdx.x == 0) {
    J.part[2 * (t * gridDim.x + blockIdx.x)] = lj;
    J.part[2 * (t * gridDim.x + blockIdx.x) + 1] = re;
  }
}

__global__ void __launch_bounds__(kCbThreads)
    k_cbmc_fin(const DevParams P, const DevBuffers B, CbmcJob J, int n_groups) {
  __shared__ double red[kCbThreads / 32];
  const int t = blockIdx.x;
  const double4_32a b1 = J.b1[t];
  const double4_32a b2 = J.charged ? J.b2[t] : b1;
  const int ty = J.type;
  double lj = 0.0, re = 0.0, ek = 0.0, mz = 0.0;
  for (int g = threadIdx.x; g < n_groups; g += blockDim.x) {
    lj += J.part[2 * (t * n_groups + g)];
    re += J.part[2 * (t * n_groups + g) + 1];
  }
  for (int i = threadIdx.x; i < J.cl; i += blockDim.x) {
    const double4_32a ci = J.chain[i];
    const double4_32a cc = J.charged ? J.chain_ci[i] : ci;
    if (P.use_pair) {
      if (i < J.cl - 1) lj += cb_lj(P, ty, ty, b1, ci);
      if (J.charged) {
        lj += cb_lj(P, ty, ty, b1, cc);
        lj += cb_lj(P, ty, ty, b2, ci);
        lj += cb_lj(P, ty, ty, b2, cc);
      }
    }
    if (P.use_ewald) {
      re += cb_real(P, b1, ci);
      if (J.charged) re += cb_real(P, b1, cc) + cb_real(P, b2, ci) + cb_real(P, b2, cc);
    }
    mz += ci.w * ci.z + (J.charged ? cc.w * cc.z : 0.0);
  }
  if (P.use_ewald)
    for (int k = threadIdx.x; k < P.n_k; k += blockDim.x) {
      const double2 so = J.s_o[k];
      const short4 kn = B.kn[k];
      double2 e = cb_phase(P, kn, b1);
      if (J.charged) {
        double2 e2 = cb_phase(P, kn, b2);
        e.x += e2.x;
        e.y += e2.y;
      }
      const double nx = so.x + e.x, ny = so.y + e.y;
      ek += B.kw[k] * ((nx * nx + ny * ny) - (so.x * so.x + so.y * so.y));
    }
  // dipole base: the system minus the deleted molecules, plus the grown chain
  if (P.dipole)
    for (int j = J.ex_lo + threadIdx.x; j < J.ex_hi; j += blockDim.x) {
      const double4_32a p = B.pos[j];
      mz -= p.w * p.z;
    }
  lj = cb_bsum<kCbThreads>(lj, red);
  re = cb_bsum<kCbThreads>(re, red);
  ek = cb_bsum<kCbThreads>(ek, red);
  mz = cb_bsum<kCbThreads>(mz, red);
  if (threadIdx.x == 0) {
    double pair_e = lj;
    if (P.use_pair && J.charged) pair_e += cb_lj(P, ty, ty, b1, b2);
    double ew = 0.0;
    if (P.use_ewald && pair_e < kVeryLarge) {
      ew = re + P.kpref * ek;
      ew += P.self_coef * b1.w * b1.w + 0.5 * cb_real(P, b1, b1);
      if (J.charged)
        ew += P.self_coef * b2.w * b2.w + cb_real(P, b1, b2) + 0.5 * cb_real(P, b2, b2);
      if (P.dipole) {
        const double mzo = B.state->mz + mz;
        const double mzn = mzo + b1.w * b1.z + (J.charged ? b2.w * b2.z : 0.0);
        ew += P.dip_coef * (mzn * mzn - mzo * mzo);
      }
    }
    if (P.use_ext) {
      pair_e += wall64(P, b1.z, ty);
      if (J.charged) pair_e += wall64(P, b2.z, ty);
    }
    J.u[t] = pair_e >= kVeryLarge ? kVeryLarge : pair_e + ew;
  }
}

int cbmc_groups(const DevParams& P) {
  int g = (P.n_bead + kCbThreads * 4 - 1) / (kCbThreads * 4);
  return g < 1 ? 1 : (g > 64 ? 64 : g);
}

void launch_cbmc(const DevParams& P, const DevBuffers& B, const CbmcJob& J, cudaStream_t s) {
  if (P.use_ewald && P.n_k > 0) k_cbmc_so<<<(P.n_k + 255) / 256, 256, 0, s>>>(P, B, J);
  const int g = cbmc_groups(P);
  k_cbmc_sys<<<dim3(g, J.n_trials), kCbThreads, 0, s>>>(P, B, J);
  k_cbmc_fin<<<J.n_trials, kCbThreads, 0, s>>>(P, B, J, g);
}


// ------------------------------------------------------------- no-alloc
// Working memory of plum_cbmc_trials_noalloc, for callers that must not
// allocate device memory (hosts whose device memory belongs to their own
// allocator, or drivers that cannot take the device-wide synchronisation of
// cudaMalloc/cudaFree). One fixed array on every GPU
// that loads the library, held until the process exits:
//   trial beads + counterions  2 * kMaxTrials double4          16 KiB
//   grown chain + counterions  2 * kMaxChain  double4          64 KiB
//   S_o(k)                     kMaxK          double2         512 KiB
//   per-block sums             2 * kMaxTrials * kMaxGroups    256 KiB
//   results                    kMaxTrials     double            2 KiB
// Nothing in it has to start at zero: each call writes every element it
// reads (k_na_pack the beads and chain, k_cbmc_so all n_k entries of S_o,
// k_cbmc_sys one sum pair per (trial, block), k_cbmc_fin one result per
// trial) before reading it. All calls on a device share the array, so calls
// that overlap on the GPU race.
namespace na {
constexpr int kMaxTrials = 256, kMaxChain = 1024, kMaxK = 32768, kMaxGroups = 64;
constexpr size_t kBeadsOff = 0;
constexpr size_t kChainOff = kBeadsOff + sizeof(double4_32a) * 2 * kMaxTrials;
constexpr size_t kSoOff = kChainOff + sizeof(double4_32a) * 2 * kMaxChain;
constexpr size_t kPartOff = kSoOff + sizeof(double2) * kMaxK;
constexpr size_t kUOff = kPartOff + sizeof(double) * 2 * kMaxTrials * kMaxGroups;
constexpr size_t kBytes = kUOff + sizeof(double) * kMaxTrials;
}  // namespace na

static __device__ __align__(256) unsigned char g_cbmc_noalloc_scratch[na::kBytes];

// Device address of the scratch array per device, resolved on the first call
// made with that device current (a host-side name of a __device__ array is
// not a device address).
static std::mutex g_na_mu;
static unsigned char* g_na_ptr[64];

// Packs caller device arrays (xyz triples) into the scratch's double4 rows.
__global__ void k_na_pack(const double* b1, const double* b2, int T, const double* chain,
                          const double* chain_ci, int cl, double q1, double q2, int charged,
                          double4_32a* beads, double4_32a* cbuf) {
  for (int i = threadIdx.x; i < T; i += blockDim.x) {
    beads[i] = make_double4_32a(b1[3 * i], b1[3 * i + 1], b1[3 * i + 2], q1);
    beads[T + i] = charged ? make_double4_32a(b2[3 * i], b2[3 * i + 1], b2[3 * i + 2], q2)
                           : beads[i];
  }
  for (int i = threadIdx.x; i < cl; i += blockDim.x) {
    cbuf[i] = make_double4_32a(chain[3 * i], chain[3 * i + 1], chain[3 * i + 2], q1);
    cbuf[cl + i] = charged ? make_double4_32a(chain_ci[3 * i], chain_ci[3 * i + 1],
                                              chain_ci[3 * i + 2], q2)
                           : cbuf[i];
  }
}

int cbmc_trials_noalloc(const DevParams& P, const DevBuffers& B, cudaStream_t s, int device,
                        int n_trials, const double* d_b1, const double* d_b2, int chain_len,
                        const double* d_chain, const double* d_chain_ci, int type, int charged,
                        double q1, double q2, int ex_lo, int ex_hi, double* d_u, char* err,
                        int err_cap) {
  auto say = [&](const char* m) {
    if (err && err_cap > 0) snprintf(err, (size_t)err_cap, "%s", m);
  };
  if (n_trials < 1 || n_trials > na::kMaxTrials) {
    say("plum_cbmc_trials_noalloc: n_trials must be 1..256");
    return 1;
  }
  if (chain_len < 0 || chain_len > na::kMaxChain) {
    say("plum_cbmc_trials_noalloc: chain_len must be 0..1024");
    return 1;
  }
  if (P.n_k > na::kMaxK) {
    say("plum_cbmc_trials_noalloc: more than 32768 half-space k-vectors");
    return 1;
  }
  static_assert(na::kMaxGroups >= 64, "cbmc_groups() is at most 64");
  if (device < 0 || device >= 64) {
    say("plum_cbmc_trials_noalloc: device index out of range");
    return 1;
  }
  unsigned char* base = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_na_mu);
    if (!g_na_ptr[device]) {
      void* p = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&p, g_cbmc_noalloc_scratch);
      if (e != cudaSuccess || !p) {
        say("plum_cbmc_trials_noalloc: cudaGetSymbolAddress failed");
        return 2;
      }
      g_na_ptr[device] = static_cast<unsigned char*>(p);
    }
    base = g_na_ptr[device];
  }
  double4_32a* beads = reinterpret_cast<double4_32a*>(base + na::kBeadsOff);
  double4_32a* cbuf = reinterpret_cast<double4_32a*>(base + na::kChainOff);
  k_na_pack<<<1, 256, 0, s>>>(d_b1, d_b2, n_trials, d_chain, d_chain_ci, chain_len, q1, q2,
                              charged, beads, cbuf);
  CbmcJob J;
  J.n_trials = n_trials;
  J.charged = charged;
  J.cl = chain_len;
  J.type = type;
  J.ex_lo = ex_lo;
  J.ex_hi = ex_hi;
  J.b1 = beads;
  J.b2 = beads + n_trials;
  J.chain = cbuf;
  J.chain_ci = cbuf + chain_len;
  J.s_o = reinterpret_cast<double2*>(base + na::kSoOff);
  J.part = reinterpret_cast<double*>(base + na::kPartOff);
  J.u = reinterpret_cast<double*>(base + na::kUOff);
  launch_cbmc(P, B, J, s);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_u, J.u, sizeof(double) * n_trials, cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    say(cudaGetErrorString(e));
    return 2;
  }
  return 0;
}

}  // namespace plum
