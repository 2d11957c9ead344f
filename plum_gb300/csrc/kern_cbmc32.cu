// Configurational-bias trial-site energies (ForceField::BeadsEnergy,
// cbmc.cc:5-151) in the precision form: every trial site of one growth step
// in ONE launch, FP32 pair and k-space arithmetic on 32-bit fixed-point
// coordinates, FP64 across blocks.
//
// The grid holds three kinds of blocks, told apart by blockIdx.x:
//   pair items   (trial group of 8) x (chunk of system beads): LJ and
//                real-space Ewald of each trial bead (and its counterion)
//                with every system bead outside the deleted molecules; each
//                system bead is loaded once for the 8 trials
//   chain items  one per trial group: a warp per trial, lanes over the grown
//                chain (no LJ with the preceding grown bead, cbmc.cc:57-58)
//   k items      256 k-vectors each: S_o(k) = committed S(k) (plus a pending
//                accepted change) - deleted molecules + grown chain, then
//                kw (|S_o + e_t|^2 - |S_o|^2) = kw (2 S_o.e_t + |e_t|^2) for
//                every trial t, e_t its (and its counterion's) e^{ik.r} q
// Phases are exact integers: k.r = 2 pi (n_x X + n_y Y + n_z Z) / 2^32 with
// X, Y, Z the fixed-point coordinates, so e^{ik.r} is one sincospi of a
// wrapped 32-bit integer. Per-block sums are FP32 and go to per-item slots;
// the last block to finish (a ticket counter) adds the slots of each trial
// in a fixed order in FP64, adds the bead-counterion cross terms, the self
// terms, the walls and the dipole change, and writes 1e8 when the pair sum
// reaches 1e8 (cbmc.cc:146-148). The result does not depend on the launch
// order of the blocks.
#include "device_common.cuh"
#include "engine.h"
#include "fp32_pair.cuh"

namespace plum {

namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kGrp = 8;      // trials per pair / chain item
constexpr int kKPer = 256;   // k-vectors per k item
constexpr int kSlot = 2 * kGrp;
constexpr size_t kMaxSmem = 200 * 1024;

__device__ __forceinline__ float warp_sum(float v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ float lj_only(const DevParams& P, int4 a, int4 b) {
  const float dx = fdiff(a.x, b.x, P.f_scale[0]);
  const float dy = fdiff(a.y, b.y, P.f_scale[1]);
  const float dz = fdiff(a.z, b.z, P.f_scale[2]);
  return lj32(P, a.w * P.n_type + b.w, dx * dx + dy * dy + dz * dz);
}

__device__ __forceinline__ float real_only(const DevParams& P, int4 a, float qa, int4 b,
                                           float qb) {
  const float qq = qa * qb;
  if (qq == 0.0f) return 0.0f;
  const float dx = fdiff(a.x, b.x, P.f_scale[0]);
  const float dy = fdiff(a.y, b.y, P.f_scale[1]);
  const float dz = fdiff(a.z, b.z, P.f_scale[2]);
  return P.f_lB * qq * real_images32(P, dx, dy, dz);
}

// q e^{ik.r} from the fixed-point coordinates (integer phase, wrapped mod 2^32)
__device__ __forceinline__ float2 cis_q(short4 k, int4 f, float q) {
  const unsigned ph = (unsigned)(int)k.x * (unsigned)f.x + (unsigned)(int)k.y * (unsigned)f.y +
                      (unsigned)(int)k.z * (unsigned)f.z;
  float s, c;
  sincospif((float)(int)ph * 4.6566128730773926e-10f, &s, &c);  // * 2^-31
  return make_float2(q * c, q * s);
}

}  // namespace

__global__ void __launch_bounds__(kThreads)
    k_cbmc32(const DevParams P, const DevBuffers B, CbmcJob J, Cbmc32Layout G,
             int* __restrict__ ticket) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int T = J.n_trials, cl = J.cl, tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  // staged fixed-point trial sites [b1 (T), b2 (T)] and grown chain
  // [chain (cl), counterions (cl)], then per-warp k partials [kWarps][T]
  int4* s_tf = reinterpret_cast<int4*>(smem);
  int4* s_cf = s_tf + 2 * T;
  float* s_tq = reinterpret_cast<float*>(s_cf + 2 * cl);
  float* s_cq = s_tq + 2 * T;
  float* s_red = s_cq + 2 * cl;
  __shared__ float red[kWarps][kSlot];
  __shared__ int s_last;
  __shared__ double s_mz;

  for (int i = tid; i < 2 * T; i += kThreads) {
    const double4_32a p = i < T ? J.b1[i] : (J.charged ? J.b2[i - T] : J.b1[i - T]);
    s_tf[i] = fix_point(P, p, J.type);
    s_tq[i] = (float)p.w;
  }
  for (int i = tid; i < 2 * cl; i += kThreads) {
    const double4_32a p = i < cl ? J.chain[i] : (J.charged ? J.chain_ci[i - cl] : J.chain[i - cl]);
    s_cf[i] = fix_point(P, p, J.type);
    s_cq[i] = (float)p.w;
  }
  __syncthreads();

  const int item = blockIdx.x;
  if (item < G.n_pair) {
    // ---------------------------------------------------------- pair item
    const int g = item / G.n_chunk, ch = item - g * G.n_chunk;
    const int t0 = g * kGrp, tn = min(kGrp, T - t0);
    float lj[kGrp], re[kGrp];
#pragma unroll
    for (int u = 0; u < kGrp; u++) lj[u] = re[u] = 0.0f;
    const int j1 = min(P.n_bead, (ch + 1) * G.chunk);
    for (int j = ch * G.chunk + tid; j < j1; j += kThreads) {
      if (j >= J.ex_lo && j < J.ex_hi) continue;
      const int4 pj = B.fpos[j];
      const float qj = B.fq[j];
#pragma unroll
      for (int u = 0; u < kGrp; u++) {
        if (u < tn) {
          pair32(P, s_tf[t0 + u], s_tq[t0 + u], pj, qj, lj[u], re[u]);
          if (J.charged) pair32(P, s_tf[T + t0 + u], s_tq[T + t0 + u], pj, qj, lj[u], re[u]);
        }
      }
    }
#pragma unroll
    for (int u = 0; u < kGrp; u++) {
      const float a = warp_sum(lj[u]), b = warp_sum(re[u]);
      if (lane == 0) {
        red[w][2 * u] = a;
        red[w][2 * u + 1] = b;
      }
    }
    __syncthreads();
    if (tid < kSlot) {
      float s = 0.0f;
      for (int q = 0; q < kWarps; q++) s += red[q][tid];
      J.part[(size_t)item * kSlot + tid] = (double)s;
    }
  } else if (item < G.n_pair + G.n_grp) {
    // --------------------------------------------------------- chain item
    const int g = item - G.n_pair, t = g * kGrp + w;
    float lj = 0.0f, re = 0.0f;
    if (t < T) {
      const int4 a = s_tf[t], a2 = s_tf[T + t];
      const float qa = s_tq[t], qa2 = s_tq[T + t];
      for (int i = lane; i < cl; i += 32) {
        const int4 ci = s_cf[i], cc = s_cf[cl + i];
        const float qi = s_cq[i], qc = s_cq[cl + i];
        if (P.use_pair) {
          if (i < cl - 1) lj += lj_only(P, a, ci);
          if (J.charged) lj += lj_only(P, a, cc) + lj_only(P, a2, ci) + lj_only(P, a2, cc);
        }
        if (P.use_ewald) {
          re += real_only(P, a, qa, ci, qi);
          if (J.charged)
            re += real_only(P, a, qa, cc, qc) + real_only(P, a2, qa2, ci, qi) +
                  real_only(P, a2, qa2, cc, qc);
        }
      }
    }
    lj = warp_sum(lj);
    re = warp_sum(re);
    if (lane == 0) {
      J.part[(size_t)G.chain_off + (size_t)g * kSlot + 2 * w] = (double)lj;
      J.part[(size_t)G.chain_off + (size_t)g * kSlot + 2 * w + 1] = (double)re;
    }
  } else {
    // ------------------------------------------------------------- k item
    const int kt = item - G.n_pair - G.n_grp;
    const int k = kt * kKPer + tid;
    const bool mine = k < P.n_k;
    short4 kv = make_short4(0, 0, 0, 0);
    float2 so = make_float2(0.0f, 0.0f);
    float kw = 0.0f;
    if (mine) {
      kv = B.kn[k];
      const DevState* st = B.state;
      double2 s = B.sk[k];
      if (st->sk_pending) {
        const double2 d = B.dsk[(size_t)st->sk_buf * P.n_k + k];
        s.x += d.x;
        s.y += d.y;
      }
      float ax = 0.0f, ay = 0.0f;
      for (int j = J.ex_lo; j < J.ex_hi; j++) {
        const float2 e = cis_q(kv, B.fpos[j], B.fq[j]);
        ax -= e.x;
        ay -= e.y;
      }
      for (int i = 0; i < cl; i++) {
        float2 e = cis_q(kv, s_cf[i], s_cq[i]);
        ax += e.x;
        ay += e.y;
        if (J.charged) {
          e = cis_q(kv, s_cf[cl + i], s_cq[cl + i]);
          ax += e.x;
          ay += e.y;
        }
      }
      so = make_float2((float)(s.x + (double)ax), (float)(s.y + (double)ay));
      kw = (float)B.kw[k];
    }
    for (int t = 0; t < T; t++) {
      float c = 0.0f;
      if (mine) {
        float2 e = cis_q(kv, s_tf[t], s_tq[t]);
        if (J.charged) {
          const float2 e2 = cis_q(kv, s_tf[T + t], s_tq[T + t]);
          e.x += e2.x;
          e.y += e2.y;
        }
        c = kw * (2.0f * (so.x * e.x + so.y * e.y) + (e.x * e.x + e.y * e.y));
      }
      c = warp_sum(c);
      if (lane == 0) s_red[w * T + t] = c;
    }
    __syncthreads();
    for (int t = tid; t < T; t += kThreads) {
      float s = 0.0f;
      for (int q = 0; q < kWarps; q++) s += s_red[q * T + t];
      J.part[(size_t)G.k_off + (size_t)kt * T + t] = (double)s;
    }
  }

  // ------------------------------------------------ last block: per trial
  __threadfence();
  __syncthreads();
  if (tid == 0) s_last = atomicAdd(ticket, 1) == (int)gridDim.x - 1;
  __syncthreads();
  if (!s_last) return;
  __threadfence();

  // dipole base: the grown chain minus the deleted molecules (trial-independent)
  if (P.dipole) {
    double mz = 0.0;
    for (int i = tid; i < cl; i += kThreads) {
      const double4_32a ci = J.chain[i];
      mz += ci.w * ci.z;
      if (J.charged) {
        const double4_32a cc = J.chain_ci[i];
        mz += cc.w * cc.z;
      }
    }
    for (int j = J.ex_lo + tid; j < J.ex_hi; j += kThreads) {
      const double4_32a p = B.pos[j];
      mz -= p.w * p.z;
    }
    for (int o = 16; o > 0; o >>= 1) mz += __shfl_xor_sync(0xffffffffu, mz, o);
    __shared__ double mzw[kWarps];
    if (lane == 0) mzw[w] = mz;
    __syncthreads();
    if (tid == 0) {
      double s = 0.0;
      for (int q = 0; q < kWarps; q++) s += mzw[q];
      s_mz = s;
    }
    __syncthreads();
  }
  for (int t = tid; t < T; t += kThreads) {
    const int g = t / kGrp, u = t - g * kGrp;
    double lj = 0.0, re = 0.0, ek = 0.0;
    if (G.n_pair > 0)
      for (int ch = 0; ch < G.n_chunk; ch++) {
        const double* sl = J.part + (size_t)(g * G.n_chunk + ch) * kSlot;
        lj += sl[2 * u];
        re += sl[2 * u + 1];
      }
    lj += J.part[(size_t)G.chain_off + (size_t)g * kSlot + 2 * u];
    re += J.part[(size_t)G.chain_off + (size_t)g * kSlot + 2 * u + 1];
    for (int kt = 0; kt < G.n_kt; kt++) ek += J.part[(size_t)G.k_off + (size_t)kt * T + t];
    const int4 a = s_tf[t], a2 = s_tf[T + t];
    const float qa = s_tq[t], qa2 = s_tq[T + t];
    const double4_32a b1 = J.b1[t];
    const double4_32a b2 = J.charged ? J.b2[t] : b1;
    double pair_e = lj;
    if (P.use_pair && J.charged) pair_e += (double)lj_only(P, a, a2);
    double ew = 0.0;
    if (P.use_ewald && pair_e < kVeryLarge) {
      ew = re + P.kpref * ek;
      ew += P.self_coef * b1.w * b1.w + 0.5 * (double)real_only(P, a, qa, a, qa);
      if (J.charged)
        ew += P.self_coef * b2.w * b2.w + (double)real_only(P, a, qa, a2, qa2) +
              0.5 * (double)real_only(P, a2, qa2, a2, qa2);
      if (P.dipole) {
        const double mzo = B.state->mz + s_mz;
        const double mzn = mzo + b1.w * b1.z + (J.charged ? b2.w * b2.z : 0.0);
        ew += P.dip_coef * (mzn * mzn - mzo * mzo);
      }
    }
    if (P.use_ext) {
      pair_e += wall64(P, b1.z, J.type);
      if (J.charged) pair_e += wall64(P, b2.z, J.type);
    }
    J.u[t] = pair_e >= kVeryLarge ? kVeryLarge : pair_e + ew;
  }
  if (tid == 0) *ticket = 0;  // ready for the next launch on this stream
}

Cbmc32Layout cbmc32_layout(const DevParams& P, int n_trials, int chain_len) {
  Cbmc32Layout G{};
  G.n_grp = (n_trials + kGrp - 1) / kGrp;
  G.n_kt = (P.use_ewald && P.n_k > 0) ? (P.n_k + kKPer - 1) / kKPer : 0;
  const int max_chunks = std::max(1, (P.n_bead + kThreads - 1) / kThreads);
  const int want = std::max(1, (2 * 152 + G.n_grp - 1) / G.n_grp);
  int n_chunk = std::min(want, max_chunks);
  const int per = (P.n_bead + n_chunk - 1) / n_chunk;
  G.chunk = std::max(kThreads, (per + kThreads - 1) / kThreads * kThreads);
  G.n_chunk = std::max(1, (P.n_bead + G.chunk - 1) / G.chunk);
  G.n_pair = (P.use_pair || P.use_ewald) ? G.n_grp * G.n_chunk : 0;
  G.chain_off = (long long)G.n_pair * kSlot;
  G.k_off = G.chain_off + (long long)G.n_grp * kSlot;
  G.slots = G.k_off + (long long)G.n_kt * n_trials;
  G.grid = G.n_pair + G.n_grp + G.n_kt;
  G.smem = (size_t)(2 * n_trials + 2 * chain_len) * (sizeof(int4) + sizeof(float)) +
           (size_t)kWarps * n_trials * sizeof(float);
  return G;
}

size_t cbmc32_max_smem() { return kMaxSmem; }

int launch_cbmc32(const DevParams& P, const DevBuffers& B, const CbmcJob& J,
                  const Cbmc32Layout& G, int* ticket, cudaStream_t s) {
  static bool attr = false;
  if (!attr) {
    if (cudaFuncSetAttribute(k_cbmc32, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)kMaxSmem) != cudaSuccess)
      return 1;
    attr = true;
  }
  if (G.smem > kMaxSmem) return 1;
  k_cbmc32<<<G.grid, kThreads, G.smem, s>>>(P, B, J, G, ticket);
  return cudaGetLastError() == cudaSuccess ? 0 : 1;
}

}  // namespace plum
