// FP64 energy kernels of the plain form.
//
//  k_delta64   energy difference of the pending move (one fused launch):
//                pairs        every (moved, other) pair: LJ
//                             (potential_truncated_lj.cc:49-85) and Ewald real
//                             space (potential_ewald_coul.cc:134-164) at trial
//                             minus current positions; moved x moved pairs once
//                             (potential_pair.cc:156-175, potential_ewald.cc:436-476)
//                k items      half-space k tiles x moved-bead groups: dS(k) and
//                             the |S|^2 change, which equals the reference's
//                             pairwise PairEnergyRepl sum
//                             (potential_ewald_coul.cc:198-225) on the same k-set
//              Every block writes its own partial sums; the serial kernel adds
//              them in a fixed order, so results are run-to-run identical.
//  k_total64   all i<j pairs from scratch (tile pairs of 128 x 128)
//  k_sk64      S(k) from scratch (k tile x bead group partials)
//  k_misc64    bonds, walls, self energy, self images, sum q z
//
// Phases e^{i k.r} come from per-axis tables e^{i n theta_a}, n = 0..kmax,
// built by complex recursion from one sincos per bead and axis, with theta_a
// = 2 kPi w_a / L_a on coordinates wrapped into the primary cell (periodic
// axes). This replaces the reference's cos(k.r) per pair and k.
#include <algorithm>
#include <cmath>
#include <cstdio>

#include "engine.h"
#include "device_common.cuh"

namespace plum {

__device__ __forceinline__ double wrap_d(double d, double L, double invL) {
  return d - L * rint(d * invL);
}

// LJ of one pair at squared distance r2 (the reference's r <= 0 overlap gives
// the 1e8 sentinel).
__device__ __forceinline__ double lj64(const DevParams& P, int k, double r2) {
  if (P.pair_kind == 1) return sqrt(r2) <= P.hs_sum[k] ? kVeryLarge : 0.0;  // hard spheres
  if (r2 <= 0.0) return kVeryLarge;
  if (r2 < P.lj_rc2[k]) {
    double s2 = P.lj_sig2[k] / r2;
    double s6 = s2 * s2 * s2;
    return P.lj_eps4[k] * (s6 * s6 - s6) - P.lj_eref[k];
  }
  return 0.0;
}

// sum over periodic images with 0 < |d + n L| <= r_c of erfc(sqrt(a) r)/r.
// An image whose single component already exceeds r_c cannot be inside the
// cut-off, so those shifts are skipped per axis.
__device__ __forceinline__ double real_images64(const DevParams& P, double dx,
                                                double dy, double dz) {
  double e = 0.0;
  const double rc = P.real_cut;
  const double rc2 = rc * rc;
  if (P.single_image) {
    // r_c <= L/2 on every axis: any other image has a component >= L/2 >= r_c
    // (ties at exactly L/2 are a set of measure zero)
    const double r2 = dx * dx + dy * dy + dz * dz;
    if (r2 > 0.0 && r2 <= rc2) e = real_term64(P, r2);
    return e;
  }
  for (int a = -P.real_cell[0]; a <= P.real_cell[0]; a++) {
    double x = dx + a * P.ebox[0];
    if (fabs(x) > rc) continue;
    for (int b = -P.real_cell[1]; b <= P.real_cell[1]; b++) {
      double y = dy + b * P.ebox[1];
      if (fabs(y) > rc) continue;
      for (int c = -P.real_cell[2]; c <= P.real_cell[2]; c++) {
        double z = dz + c * P.ebox[2];
        if (fabs(z) > rc) continue;
        const double r2 = x * x + y * y + z * z;
        if (r2 > 0.0 && r2 <= rc2) e += real_term64(P, r2);
      }
    }
  }
  return e;
}

// LJ and real-space Ewald of bead a (type ta) with bead b (type tb).
__device__ __forceinline__ void pair64(const DevParams& P, double4_32a a, int ta,
                                       double4_32a b, int tb, double& lj, double& re) {
  double dx = b.x - a.x, dy = b.y - a.y, dz = b.z - a.z;
  if (P.same_wrap) {
    // the pair box wraps every periodic axis as the Ewald box does: one
    // minimum-image vector for both terms
    const double x = wrap_d(dx, P.box[0], P.inv_box[0]);
    const double y = wrap_d(dy, P.box[1], P.inv_box[1]);
    const double z = P.npbc > 2 ? wrap_d(dz, P.box[2], P.inv_box[2]) : dz;
    const double r2 = x * x + y * y + z * z;
    if (P.use_pair && r2 < P.lj_max2) lj += lj64(P, ta * P.n_type + tb, r2);
    if (P.use_ewald) {
      const double qq = a.w * b.w;
      if (qq != 0.0) re += P.lB * qq * real_images64(P, x, y, z);
    }
    return;
  }
  if (P.use_pair) {
    double x = wrap_d(dx, P.box[0], P.inv_box[0]);
    double y = wrap_d(dy, P.box[1], P.inv_box[1]);
    double z = P.npbc > 2 ? wrap_d(dz, P.box[2], P.inv_box[2]) : dz;
    lj += lj64(P, ta * P.n_type + tb, x * x + y * y + z * z);
  }
  if (P.use_ewald) {
    double qq = a.w * b.w;
    if (qq != 0.0) {
      double x = wrap_d(dx, P.ebox[0], P.inv_ebox[0]);
      double y = wrap_d(dy, P.ebox[1], P.inv_ebox[1]);
      double z = P.npbc > 2 ? wrap_d(dz, P.ebox[2], P.inv_ebox[2]) : dz;
      re += P.lB * qq * real_images64(P, x, y, z);
    }
  }
}

// e^{i n theta} tables for one bead: tab[koff[axis] + n], n = 0..kmax[axis];
// q folded into the x table.
__device__ __forceinline__ void build_axis_table(const DevParams& P, double4_32a p,
                                                 int axis, double2* tab) {
  double w = axis == 0 ? p.x : (axis == 1 ? p.y : p.z);
  if (axis < P.npbc) w -= P.ebox[axis] * floor(w * P.inv_ebox[axis]);
  double s, c;
  sincos(P.kunit[axis] * w, &s, &c);
  double2 e = axis == 0 ? make_double2(p.w, 0.0) : make_double2(1.0, 0.0);
  double2* t = tab + P.koff[axis];
  t[0] = e;
  for (int n = 1; n <= P.kmax[axis]; n++) {
    double re = e.x * c - e.y * s;
    double im = e.x * s + e.y * c;
    e = make_double2(re, im);
    t[n] = e;
  }
}

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// q e^{i k.r} from a bead's tables for k = (nx >= 0, ny, nz).
__device__ __forceinline__ double2 phase_from(const DevParams& P, const double2* tab, short4 k) {
  double2 ex = tab[P.koff[0] + k.x];
  double2 ey = tab[P.koff[1] + (k.y >= 0 ? k.y : -k.y)];
  if (k.y < 0) ey.y = -ey.y;
  double2 ez = tab[P.koff[2] + (k.z >= 0 ? k.z : -k.z)];
  if (k.z < 0) ez.y = -ez.y;
  return cmul(cmul(ex, ey), ez);
}

template <int NT>
__device__ __forceinline__ double block_sum(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) sh[w] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < NT / 32; i++) t += sh[i];
  return t;  // valid in thread 0
}

// Constants of the fixed-point pair form: squared distances in units of
// (L / 2^64)^2 ("raw"). A non-negative double orders like its bit pattern
// read as an integer, so the cut-off tests are integer compares (off the
// FP64 pipe).
struct FixConst {
  double s2, ua, pref;
  long long rc2_bits, lj2_bits;  // raw r_c^2 and raw LJ reach, as bits
};
__device__ __forceinline__ FixConst fix_const(const DevParams& P) {
  FixConst F;
  const double s = P.ebox[0] * 0x1p-64;  // L / 2^64
  F.s2 = s * s;
  F.ua = P.alpha * F.s2;
  F.pref = P.lB * P.sqrt_alpha;
  F.rc2_bits = __double_as_longlong(P.real_cut * P.real_cut / F.s2);
  F.lj2_bits = P.use_pair ? __double_as_longlong(P.lj_max2 / F.s2) : 0;
  return F;
}

// One pair in the fixed-point form: adds its LJ energy at (k, r^2) to lj and
// returns h(alpha r^2) inside the real-space cut-off (0 outside, and at
// r = 0 as the reference's r > 0 test has it); the caller multiplies by the
// charge product with lB sqrt(alpha) folded in.
__device__ __forceinline__ double pair_fix(const DevParams& P, const FixConst& F,
                                           unsigned long long ax, unsigned long long ay,
                                           unsigned long long az, unsigned long long bx,
                                           unsigned long long by, unsigned long long bz, int k,
                                           double& lj) {
  const double dx = __ll2double_rn((long long)(bx - ax));
  const double dy = __ll2double_rn((long long)(by - ay));
  const double dz = __ll2double_rn((long long)(bz - az));
  const double raw = fma(dx, dx, fma(dy, dy, dz * dz));
  const long long rb = __double_as_longlong(raw);
  if (rb < F.lj2_bits) lj += lj64(P, k, raw * F.s2);
  if (rb > 0 && rb <= F.rc2_bits) {
    const long long bits = __double_as_longlong(raw * F.ua);
    return bits >= kH64LoBits ? h64_tab(P.htab64, bits)
                              : real_term64(P, raw * F.s2) / P.sqrt_alpha;
  }
  return 0.0;
}

// ---------------------------------------------------------------- delta
// Pair sweep: the m x N (moved, other) pairs are numbered p = i*N + j and dealt
// to every thread of the grid in turn, so even a one-bead move spreads over
// all SMs (FP64 issue rate per SM is low on GB300; parallel width is what
// counts). Pairs with both beads moved are taken once (j > i), at trial
// positions for both.
// k-space: items (k tile of kKTile vectors) x (group of kchunk_delta moved
// beads); each item stores its dS(k) part, and the last item of a k tile to
// finish (atomic ticket) adds the groups in order -- deterministic -- and
// writes dS(k) and the tile's energy change.
constexpr int kKTile = 128;
constexpr int kFixStage = 128;  // moved beads the fixed-point pair form stages
constexpr size_t kFixBytes = kFixStage * (6 * sizeof(unsigned long long) + sizeof(double) +
                                          sizeof(int));

__global__ void __launch_bounds__(kPairThreads)
    k_delta64(const DevParams P, const DevBuffers B) {
  extern __shared__ __align__(32) unsigned char smem[];
  __shared__ double red[kPairThreads / 32];
  __shared__ int s_last;
  const DevState* st = B.state;
  const int b_lo = st->b_lo, b_hi = st->b_hi;
  const int m = st->pending ? b_hi - b_lo : 0;
  const int sk_pend = st->sk_pending, sk_buf = st->sk_buf, cur_buf = st->cur_buf;
  __shared__ int s_final;
  const int N = P.n_bead;

  double acc_lj = 0.0, acc_re = 0.0;
  if (m > 0 && m <= kFixStage && B.fpos64 && fix_pairs(P)) {
    // Fixed-point pair form: the moved beads (trial and current) are staged
    // once per block as 64-bit fixed-point fractions of the box, the other
    // beads come from the context's 64-bit mirror; pairs are dealt over the
    // grid by the same flat index as below. A moved other bead j pairs once
    // with each moved bead i < j, both at trial or both at current positions.
    unsigned long long* fx = reinterpret_cast<unsigned long long*>(smem);  // [6][kFixStage]
    double* fq = reinterpret_cast<double*>(fx + 6 * kFixStage);
    int* fk = reinterpret_cast<int*>(fq + kFixStage);
    const FixConst F = fix_const(P);
    for (int t = threadIdx.x; t < m; t += blockDim.x) {
      const ulonglong4_32a a = fix64x4(P, B.trial[b_lo + t]), c = fix64x4(P, B.pos[b_lo + t]);
      fx[t] = a.x;
      fx[kFixStage + t] = a.y;
      fx[2 * kFixStage + t] = a.z;
      fx[3 * kFixStage + t] = c.x;
      fx[4 * kFixStage + t] = c.y;
      fx[5 * kFixStage + t] = c.z;
      fq[t] = __longlong_as_double((long long)c.w) * F.pref;
      fk[t] = B.type[b_lo + t] * P.n_type;
    }
    __syncthreads();
    const long long total = (long long)m * N;
    const long long G = (long long)gridDim.x * blockDim.x;
    const long long p0 = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int gq = (int)(G / N), gr = (int)(G % N);
    int ii = (int)(p0 / N), j = (int)(p0 % N);
    double lj0 = 0.0;  // LJ at current positions, subtracted at the end
    for (long long p = p0; p < total; p += G, ii += gq, j += gr) {
      if (j >= N) {
        j -= N;
        ii++;
      }
      const bool jm = j >= b_lo && j < b_hi;
      if (jm && j <= b_lo + ii) continue;
      const ulonglong4_32a o = B.fpos64[j];
      const int k = fk[ii] + B.type[j];
      const double qq = fq[ii] * __longlong_as_double((long long)o.w);
      const int l = jm ? j - b_lo : 0;
      const double h1 =
          pair_fix(P, F, fx[ii], fx[kFixStage + ii], fx[2 * kFixStage + ii],
                   jm ? fx[l] : o.x, jm ? fx[kFixStage + l] : o.y,
                   jm ? fx[2 * kFixStage + l] : o.z, k, acc_lj);
      const double h0 = pair_fix(P, F, fx[3 * kFixStage + ii], fx[4 * kFixStage + ii],
                                 fx[5 * kFixStage + ii], o.x, o.y, o.z, k, lj0);
      acc_re = fma(qq, h1 - h0, acc_re);
    }
    acc_lj -= lj0;
  } else if (P.use_pair || P.use_ewald) {
    // pair p = ii * N + j, dealt with stride G; (ii, j) advanced without a
    // division per pair
    const long long total = (long long)m * N;
    const long long G = (long long)gridDim.x * blockDim.x;
    const long long p0 = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int gq = (int)(G / N), gr = (int)(G % N);
    int ii = (int)(p0 / N), j = (int)(p0 % N);
    for (long long p = p0; p < total; p += G, ii += gq, j += gr) {
      if (j >= N) {
        j -= N;
        ii++;
      }
      const int i = b_lo + ii;
      const bool jm = j >= b_lo && j < b_hi;
      if (jm && j <= i) continue;
      const double4_32a ti = B.trial[i], ci = B.pos[i];
      const int tyi = B.type[i], tyj = B.type[j];
      const double4_32a cj = B.pos[j];
      const double4_32a tj = jm ? B.trial[j] : cj;
      double l1 = 0, r1 = 0, l0 = 0, r0 = 0;
      pair64(P, ti, tyi, tj, tyj, l1, r1);
      pair64(P, ci, tyi, cj, tyj, l0, r0);
      if (!hs_bonded(P, B.mol_start, i, j)) acc_lj += l1 - l0;
      acc_re += r1 - r0;
    }
  }
  double t0 = block_sum<kPairThreads>(acc_lj, red);
  double t1 = block_sum<kPairThreads>(acc_re, red);
  if (threadIdx.x == 0) {
    B.partial[4 * blockIdx.x + 0] = t0;
    B.partial[4 * blockIdx.x + 1] = t1;
  }

  const bool kwork = P.use_ewald && m > 0;
  const int chunk = P.kchunk_delta;
  const int n_groups = kwork ? (m + chunk - 1) / chunk : 0;
  const int n_tiles = (P.n_k + kKTile - 1) / kKTile;
  const int n_items = n_tiles * n_groups;
  double2* tabs = reinterpret_cast<double2*>(smem);  // [chunk][2][kper]
  const int per = P.kper;
  for (int item = blockIdx.x; item < n_items; item += gridDim.x) {
    const int tile = item % n_tiles, grp = item / n_tiles;
    const int c0 = b_lo + grp * chunk;
    const int cnt = min(chunk, b_hi - c0);
    __syncthreads();
    for (int t = threadIdx.x; t < cnt * 6; t += blockDim.x) {
      int bead = t / 6, which = (t / 3) & 1, axis = t % 3;
      double4_32a p = which ? B.pos[c0 + bead] : B.trial[c0 + bead];
      build_axis_table(P, p, axis, tabs + (bead * 2 + which) * per);
    }
    __syncthreads();
    const int k = tile * kKTile + threadIdx.x;
    const bool mine = threadIdx.x < kKTile && k < P.n_k;
    if (mine) {
      const short4 kv = B.kn[k];
      double2 ds = make_double2(0.0, 0.0);
      for (int b = 0; b < cnt; b++) {
        double2 e1 = phase_from(P, tabs + (b * 2 + 0) * per, kv);
        double2 e0 = phase_from(P, tabs + (b * 2 + 1) * per, kv);
        ds.x += e1.x - e0.x;
        ds.y += e1.y - e0.y;
      }
      B.dsk_part[(size_t)grp * P.n_k + k] = ds;
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) s_last = atomicAdd(&B.ktile_count[tile], 1) == n_groups - 1;
    __syncthreads();
    if (s_last) {
      __threadfence();
      double e = 0.0;
      if (mine) {
        double2 ds = make_double2(0.0, 0.0);
        for (int g = 0; g < n_groups; g++) {
          double2 v = __ldcg(&B.dsk_part[(size_t)g * P.n_k + k]);
          ds.x += v.x;
          ds.y += v.y;
        }
        double2 s = B.sk[k];
        if (sk_pend) {
          const double2 p = B.dsk[(size_t)sk_buf * P.n_k + k];
          s = make_double2(s.x + p.x, s.y + p.y);
          B.sk[k] = s;
        }
        B.dsk[(size_t)cur_buf * P.n_k + k] = ds;
        e = B.kw[k] * (2.0 * (s.x * ds.x + s.y * ds.y) + (ds.x * ds.x + ds.y * ds.y));
      }
      e = block_sum<kPairThreads>(e, red);
      if (threadIdx.x == 0) {
        B.kpartial[tile] = e;
        B.ktile_count[tile] = 0;
      }
    }
  }
  // Last block to finish adds every block's and every k tile's sums in a
  // fixed order (deterministic) for the serial kernel.
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) s_final = atomicAdd(B.done_count, 1) == (int)gridDim.x - 1;
  __syncthreads();
  if (s_final) {
    __threadfence();
    double a = 0.0, b = 0.0, c = 0.0;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) {
      a += __ldcg(&B.partial[4 * i]);
      b += __ldcg(&B.partial[4 * i + 1]);
    }
    if (kwork)
      for (int i = threadIdx.x; i < n_tiles; i += blockDim.x) c += __ldcg(&B.kpartial[i]);
    a = block_sum<kPairThreads>(a, red);
    b = block_sum<kPairThreads>(b, red);
    c = block_sum<kPairThreads>(c, red);
    if (threadIdx.x == 0) {
      DevState* ws = B.state;
      ws->red_lj = a;
      ws->red_re = b;
      ws->red_k = c;
      *B.done_count = 0;
    }
  }
}

int ktile_count(const DevParams& P) { return (P.n_k + kKTile - 1) / kKTile; }

static int g_pair_grid = 0;

int pair_grid() {
  if (g_pair_grid == 0) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    g_pair_grid = 2 * (sms > 0 ? sms : 152);
  }
  return g_pair_grid;
}

static size_t delta_smem(const DevParams& P) {
  const size_t k = P.use_ewald ? (size_t)P.kchunk_delta * 2 * P.kper * sizeof(double2) : 0;
  return fix_pairs(P) ? std::max(k, kFixBytes) : k;
}

void launch_delta_pairs64(const DevParams& P, const DevBuffers& B, cudaStream_t s) {
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_delta64, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         std::max((size_t)kKTableBytes + 4096, kFixBytes));
    attr = true;
  }
  k_delta64<<<pair_grid(), kPairThreads, delta_smem(P), s>>>(P, B);
}

// ---------------------------------------------------------------- totals
constexpr int kTotTile = 128;

__device__ __forceinline__ void tri_unrank(long long t, int n, int& a, int& b) {
  // t-th (a <= b) pair of an n x n upper triangle, row-major.
  int r = (int)((2.0 * n + 1 - sqrt((2.0 * n + 1) * (2.0 * n + 1) - 8.0 * t)) / 2);
  if (r < 0) r = 0;
  auto start = [n](long long rr) { return rr * n - rr * (rr - 1) / 2; };
  while (r > 0 && start(r) > t) r--;
  while (r + 1 < n && start(r + 1) <= t) r++;
  a = r;
  b = r + (int)(t - start(r));
}

__global__ void __launch_bounds__(kTotTile)
    k_total64(const DevParams P, const DevBuffers B, double* out) {
  __shared__ double4_32a sp[kTotTile];
  __shared__ int st[kTotTile];
  __shared__ double red[kTotTile / 32];
  const int nt = (P.n_bead + kTotTile - 1) / kTotTile;
  int ta, tb;
  tri_unrank(blockIdx.x, nt, ta, tb);
  const int j0 = tb * kTotTile;
  const int jn = min(kTotTile, P.n_bead - j0);
  if (threadIdx.x < jn) {
    sp[threadIdx.x] = B.pos[j0 + threadIdx.x];
    st[threadIdx.x] = B.type[j0 + threadIdx.x];
  }
  __syncthreads();
  double lj = 0.0, re = 0.0;
  const int i = ta * kTotTile + threadIdx.x;
  if (i < P.n_bead) {
    const double4_32a pi = B.pos[i];
    const int ti = B.type[i];
    for (int jj = 0; jj < jn; jj++) {
      if (ta == tb && jj <= (int)threadIdx.x) continue;
      double l = 0.0;
      pair64(P, pi, ti, sp[jj], st[jj], l, re);
      if (!hs_bonded(P, B.mol_start, i, j0 + jj)) lj += l;
    }
  }
  double a = block_sum<kTotTile>(lj, red);
  double b = block_sum<kTotTile>(re, red);
  if (threadIdx.x == 0) {
    out[2 * blockIdx.x] = a;
    out[2 * blockIdx.x + 1] = b;
  }
}

// k_total64 for LJ + Ewald in a cubic box periodic on every axis, one image
// (r_c <= L/2) and one box for both terms: positions as 64-bit fixed-point
// fractions of the box, staged per tile, so one integer subtraction is the
// minimum-image difference (each fraction carries the rounding of x / L, about
// one ulp of the coordinate, as its FP64 value does; the subtraction is exact
// and the conversion to FP64 rounds once). r^2 in FP64, in units of
// (L / 2^64)^2; the cut-off tests as integer compares of the FP64 bit
// patterns; the real-space term sqrt(alpha) h(alpha r^2) from the FP64 table,
// with lB sqrt(alpha) q_i folded into the thread's charge.
__global__ void __launch_bounds__(kTotTile)
    k_total64_fix(const DevParams P, const DevBuffers B, double* out) {
  __shared__ unsigned long long sx[kTotTile], sy[kTotTile], sz[kTotTile];
  __shared__ double sq[kTotTile];
  __shared__ int st[kTotTile];
  __shared__ double red[2 * (kTotTile / 32)];
  const int nt = (P.n_bead + kTotTile - 1) / kTotTile;
  int ta, tb;
  tri_unrank(blockIdx.x, nt, ta, tb);
  const int j0 = tb * kTotTile;
  const int jn = min(kTotTile, P.n_bead - j0);
  const double inv = P.inv_ebox[0];
  if (threadIdx.x < jn) {
    const double4_32a p = B.pos[j0 + threadIdx.x];
    sx[threadIdx.x] = fix64(p.x, inv);
    sy[threadIdx.x] = fix64(p.y, inv);
    sz[threadIdx.x] = fix64(p.z, inv);
    sq[threadIdx.x] = p.w;
    st[threadIdx.x] = B.type[j0 + threadIdx.x];
  }
  __syncthreads();
  const FixConst F = fix_const(P);
  double lj = 0.0, re = 0.0;
  const int i = ta * kTotTile + threadIdx.x;
  if (i < P.n_bead) {
    const double4_32a pi = B.pos[i];
    const unsigned long long ux = fix64(pi.x, inv), uy = fix64(pi.y, inv), uz = fix64(pi.z, inv);
    const double qi = pi.w * F.pref;
    const int kt = B.type[i] * P.n_type;
    for (int jj = ta == tb ? (int)threadIdx.x + 1 : 0; jj < jn; jj++)
      re = fma(qi * sq[jj], pair_fix(P, F, ux, uy, uz, sx[jj], sy[jj], sz[jj], kt + st[jj], lj),
               re);
  }
  const double a = block_sum<kTotTile>(lj, red);
  const double b = block_sum<kTotTile>(re, red + kTotTile / 32);
  if (threadIdx.x == 0) {
    out[2 * blockIdx.x] = a;
    out[2 * blockIdx.x + 1] = b;
  }
}

// The plain form's 64-bit mirror of every bead's position.
__global__ void k_fix64_all(const DevParams P, const DevBuffers B) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P.n_bead; i += gridDim.x * blockDim.x)
    B.fpos64[i] = fix64x4(P, B.pos[i]);
}

void launch_fix64_all(const DevParams& P, const DevBuffers& B, cudaStream_t s) {
  if (B.fpos64 && P.n_bead > 0) k_fix64_all<<<(P.n_bead + 255) / 256, 256, 0, s>>>(P, B);
}

int total_partials_count(const DevParams& P) {
  long long nt = (P.n_bead + kTotTile - 1) / kTotTile;
  return (int)(nt * (nt + 1) / 2);
}

void launch_total64(const DevParams& P, const DevBuffers& B, double* out, int n_part,
                    cudaStream_t s) {
  if (fix_pairs(P))
    k_total64_fix<<<n_part, kTotTile, 0, s>>>(P, B, out);
  else
    k_total64<<<n_part, kTotTile, 0, s>>>(P, B, out);
}

// S(k) from scratch: block (k tile, bead group) writes a partial; a second
// pass adds the groups in order.
// Each thread takes kSkPer consecutive k-vectors (a tile of kSkTile per
// block); vectors of one (n_x, n_y) column (n_z runs fastest in the k list)
// share the product e^{i(k_x x + k_y y)} per bead, and each phase is the same
// cmul(cmul(ex, ey), ez) as phase_from's. Bead groups split the beads so that
// the grid is one wave of two blocks per SM; a second pass adds the groups in
// order.
constexpr int kSkPer = 4;
constexpr int kSkTile = kSkPer * kPairThreads;
constexpr int kSkGroupsMax = 512;

int sk_full_groups(const DevParams& P) {
  const int tiles = std::max(1, (P.n_k + kSkTile - 1) / kSkTile);
  const int want = (pair_grid() + tiles - 1) / tiles;  // two blocks per SM, one wave
  return std::max(1, std::min(kSkGroupsMax, want));  // groups past the beads add zero
}

__global__ void __launch_bounds__(kPairThreads)
    k_sk64(const DevParams P, const DevBuffers B, double2* part, int groups) {
  extern __shared__ __align__(32) unsigned char smem[];
  double2* tabs = reinterpret_cast<double2*>(smem);
  const int per = P.kper;
  const int chunk = P.kchunk_sk;
  const int g = blockIdx.y;
  const int per_g = (P.n_bead + groups - 1) / groups;
  const int b0 = g * per_g, b1 = min(P.n_bead, b0 + per_g);
  int kk[kSkPer], ox[kSkPer], oy[kSkPer], oz[kSkPer];
  bool mine[kSkPer], col[kSkPer], ny[kSkPer], nz[kSkPer];
  double2 s[kSkPer];
#pragma unroll
  for (int q = 0; q < kSkPer; q++) {
    kk[q] = blockIdx.x * kSkTile + threadIdx.x * kSkPer + q;
    mine[q] = kk[q] < P.n_k;
    const short4 kv = mine[q] ? B.kn[kk[q]] : make_short4(0, 0, 0, 0);
    ox[q] = P.koff[0] + kv.x;
    oy[q] = P.koff[1] + (kv.y >= 0 ? kv.y : -kv.y);
    oz[q] = P.koff[2] + (kv.z >= 0 ? kv.z : -kv.z);
    ny[q] = kv.y < 0;
    nz[q] = kv.z < 0;
    col[q] = q == 0 || ox[q] != ox[q - 1] || oy[q] != oy[q - 1] || ny[q] != ny[q - 1];
    s[q] = make_double2(0.0, 0.0);
  }
  for (int c0 = b0; c0 < b1; c0 += chunk) {
    const int cnt = min(chunk, b1 - c0);
    __syncthreads();
    for (int t = threadIdx.x; t < cnt * 3; t += blockDim.x)
      build_axis_table(P, B.pos[c0 + t / 3], t % 3, tabs + (t / 3) * per);
    __syncthreads();
    if (mine[0])
      for (int b = 0; b < cnt; b++) {
        const double2* tb = tabs + b * per;
        double2 xy = make_double2(0.0, 0.0);
#pragma unroll
        for (int q = 0; q < kSkPer; q++)
          if (mine[q]) {
            if (col[q]) {
              double2 ey = tb[oy[q]];
              if (ny[q]) ey.y = -ey.y;
              xy = cmul(tb[ox[q]], ey);
            }
            double2 ez = tb[oz[q]];
            if (nz[q]) ez.y = -ez.y;
            const double2 e = cmul(xy, ez);
            s[q].x += e.x;
            s[q].y += e.y;
          }
      }
  }
#pragma unroll
  for (int q = 0; q < kSkPer; q++)
    if (mine[q]) part[(size_t)g * P.n_k + kk[q]] = s[q];
}

__global__ void k_sk_sum(int n_k, int groups, const double2* part, double2* sk) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n_k) return;
  double2 s = make_double2(0.0, 0.0);
  for (int g = 0; g < groups; g++) {
    double2 p = part[(size_t)g * n_k + k];
    s.x += p.x;
    s.y += p.y;
  }
  sk[k] = s;
}

void launch_sk_full64(const DevParams& P, const DevBuffers& B, double2* part, cudaStream_t s) {
  if (!P.use_ewald || P.n_k == 0) return;
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_sk64, cudaFuncAttributeMaxDynamicSharedMemorySize, kKTableBytes + 4096);
    attr = true;
  }
  size_t smem = (size_t)P.kchunk_sk * P.kper * sizeof(double2);
  const int groups = sk_full_groups(P);
  dim3 grid((P.n_k + kSkTile - 1) / kSkTile, groups);
  k_sk64<<<grid, kPairThreads, smem, s>>>(P, B, part, groups);
  k_sk_sum<<<(P.n_k + 255) / 256, 256, 0, s>>>(P.n_k, groups, part, B.sk);
}

// Bond energy of molecule m on coordinates p (potential_spring.cc:22-48),
// summed in bond order.
__device__ double bond_mol64(const DevParams& P, const double4_32a* p, int b0, int b1) {
  double e = 0.0;
  for (int i = b0; i < b1 - 1; i++) {
    double dx = p[i].x - p[i + 1].x, dy = p[i].y - p[i + 1].y, dz = p[i].z - p[i + 1].z;
    double r = sqrt(dx * dx + dy * dy + dz * dz);
    e += 0.5 * P.k_bond * (r - P.r0) * (r - P.r0);
  }
  return e;
}

// Misc totals: out6 = {bond, ext, self, self_images, mz, unused}.
// Also fills bond_mol[]. One block, fixed-order reduction.
__global__ void __launch_bounds__(256) k_misc64(const DevParams P, const DevBuffers B,
                                                double* out6) {
  __shared__ double red[8];
  double eb = 0, ee = 0, es = 0, ei = 0, mz = 0;
  double img = 0.0;
  if (P.use_ewald) img = real_images64(P, 0.0, 0.0, 0.0);
  for (int m = threadIdx.x; m < P.n_mol; m += blockDim.x) {
    double e = 0.0;
    if (P.use_bond) e = bond_mol64(P, B.pos, B.mol_start[m], B.mol_start[m + 1]);
    B.bond_mol[m] = e;
    eb += e;
  }
  for (int i = threadIdx.x; i < P.n_bead; i += blockDim.x) {
    double4_32a p = B.pos[i];
    if (P.use_ext) ee += wall64(P, p.z, B.type[i]);
    if (P.use_ewald) {
      es += P.self_coef * p.w * p.w;
      ei += 0.5 * P.lB * p.w * p.w * img;
      mz += p.w * p.z;
    }
  }
  double v[5] = {eb, ee, es, ei, mz};
  for (int q = 0; q < 5; q++) {
    double t = block_sum<256>(v[q], red);
    if (threadIdx.x == 0) out6[q] = t;
  }
  if (threadIdx.x == 0) out6[5] = 0.0;
}

void launch_misc_total64(const DevParams& P, const DevBuffers& B, double* out6,
                         cudaStream_t s) {
  k_misc64<<<1, 256, 0, s>>>(P, B, out6);
}

// Rg^2, axis components and end-to-end^2 (simulation.cc:406-500); one block
// per chain writes its terms, thread 0 of a final pass adds them in order.
__global__ void k_obs_chain(const DevParams P, const DevBuffers B, double* per_mol) {
  __shared__ double red[8];
  const int m = blockIdx.x;
  const int b0 = B.mol_start[m], n = B.mol_start[m + 1] - b0;
  double g = 0, gx = 0, gy = 0, gz = 0;
  if (n > 1) {
    long long np = (long long)n * (n - 1) / 2;
    for (long long p = threadIdx.x; p < np; p += blockDim.x) {
      int j = (int)((2.0 * n - 1 - sqrt((2.0 * n - 1) * (2.0 * n - 1) - 8.0 * p)) / 2);
      auto st = [n](long long jj) { return jj * (2 * n - jj - 1) / 2; };
      while (j > 0 && st(j) > p) j--;
      while (st(j + 1) <= p) j++;
      int k = j + 1 + (int)(p - st(j));
      double4_32a a = B.pos[b0 + j], b = B.pos[b0 + k];
      double x = fabs(a.x - b.x), y = fabs(a.y - b.y), z = fabs(a.z - b.z);
      double r = sqrt(x * x + y * y + z * z);
      g += r * r;
      gx += x * x, gy += y * y, gz += z * z;
    }
  }
  double v[4] = {g, gx, gy, gz};
  for (int q = 0; q < 4; q++) {
    double t = block_sum<256>(v[q], red);
    if (threadIdx.x == 0) per_mol[5 * m + q] = n > 1 ? t / ((double)n * n) : 0.0;
  }
  if (threadIdx.x == 0) {
    double e = 0.0;
    if (n > 1) {
      double4_32a a = B.pos[b0], b = B.pos[b0 + n - 1];
      double x = a.x - b.x, y = a.y - b.y, z = a.z - b.z;
      double r = sqrt(x * x + y * y + z * z);
      e = r * r;
    }
    per_mol[5 * m + 4] = e;
  }
}

__global__ void k_obs_sum(int n_mol, int n_chains, const double* per_mol, double* out5) {
  if (threadIdx.x != 0) return;
  double s[5] = {0, 0, 0, 0, 0};
  for (int m = 0; m < n_mol; m++)
    for (int q = 0; q < 5; q++) s[q] += per_mol[5 * m + q];
  for (int q = 0; q < 5; q++) out5[q] = n_chains > 0 ? s[q] / n_chains : s[q];
}

void launch_observables64(const DevParams& P, const DevBuffers& B, double* per_mol,
                          double* out5, cudaStream_t s) {
  k_obs_chain<<<P.n_mol, 256, 0, s>>>(P, B, per_mol);
  k_obs_sum<<<1, 32, 0, s>>>(P.n_mol, P.n_chain_total, per_mol, out5);
}

// rho(z) counts of one configuration (Simulation::CalcRhoZ,
// simulation.cc:1029-1045): molecules from `phantom` on, category 0 for
// chains, 1 for ions with q >= 0, 2 for q < 0; z wrapped into [0, Lz) by
// floor; bin floor(z / res) kept when inside [0, n_bins). Integer counts
// (order-independent); the host scales them by 1 / (Lx Ly res).
__global__ void k_rhoz(const DevParams P, const DevBuffers B, double res, int n_bins,
                       unsigned* cnt) {
  for (int m = P.phantom + blockIdx.x; m < P.n_mol; m += gridDim.x) {
    const int b0 = B.mol_start[m], n = B.mol_start[m + 1] - b0;
    const int id = n > 1 ? 0 : (B.pos[b0].w >= 0.0 ? 1 : 2);
    for (int j = b0 + threadIdx.x; j < b0 + n; j += blockDim.x) {
      double z = B.pos[j].z;
      z -= P.box[2] * floor(z / P.box[2]);
      const int bz = (int)floor(z / res);
      if (bz >= 0 && bz < n_bins) atomicAdd(&cnt[3 * bz + id], 1u);
    }
  }
}

void launch_rhoz(const DevParams& P, const DevBuffers& B, double res, int n_bins, unsigned* cnt,
                 cudaStream_t s) {
  cudaMemsetAsync(cnt, 0, sizeof(unsigned) * 3 * (size_t)n_bins, s);
  const int m = P.n_mol - P.phantom;
  if (m > 0) k_rhoz<<<std::min(m, 4 * 152), 128, 0, s>>>(P, B, res, n_bins, cnt);
}


// The FP64 h(u) table: per bin the degree-8 Chebyshev interpolant of
// h(u) = erfc(sqrt u) / sqrt u at the 9 Chebyshev nodes of y in [-1/2, 1/2]
// (u = lo + (y + 1/2) w), in long double, then rewritten in powers of y.
void build_h64_table(double* out) {
  constexpr int n = 9;
  const long double pi = 3.141592653589793238462643383279503L;
  long double T[n][n] = {};  // T_j(t) coefficients in powers of t
  T[0][0] = 1.0L;
  T[1][1] = 1.0L;
  for (int j = 2; j < n; j++)
    for (int q = 0; q < n; q++)
      T[j][q] = (q ? 2.0L * T[j - 1][q - 1] : 0.0L) - T[j - 2][q];
  int b = 0;
  for (int e = kH64ELo; e < kH64EHi; e++)
    for (int j = 0; j < kH64Per; j++, b++) {
      const long double lo = std::ldexp(1.0L + (long double)j / kH64Per, e);
      const long double w = std::ldexp(1.0L / kH64Per, e);
      long double f[n], tk[n];
      for (int k = 0; k < n; k++) {
        tk[k] = std::cos(pi * (k + 0.5L) / n);  // t = 2 y in [-1, 1]
        const long double u = lo + (0.5L * tk[k] + 0.5L) * w;
        const long double r = std::sqrt(u);
        f[k] = std::erfc(r) / r;
      }
      long double mono[n] = {};  // powers of y
      for (int jj = 0; jj < n; jj++) {
        long double a = 0.0L;
        for (int k = 0; k < n; k++) a += f[k] * std::cos(pi * jj * (k + 0.5L) / n);
        a *= (jj ? 2.0L : 1.0L) / n;
        for (int q = 0; q < n; q++) mono[q] += a * T[jj][q] * std::ldexp(1.0L, q);
      }
      for (int q = 0; q < kH64Stride; q++) out[(size_t)b * kH64Stride + q] = q < n ? (double)mono[q] : 0.0;
    }
}

}  // namespace plum
