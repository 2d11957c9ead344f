// Precision form: the pending move's energy difference with FP32 pair and
// k-space arithmetic (FP64 kept for S(k), the running totals and the
// periodic full recompute, see kern_energy.cu / capi.cu).
//
// Coordinates are mirrored as 32-bit fixed-point fractions of the Ewald box
// (fpos: X = round(w / L * 2^32), w wrapped into the primary cell on periodic
// axes). Then
//   * a minimum-image difference is one integer subtraction: int32 wraparound
//     is the periodic wrap, and the difference converts to FP32 with a
//     relative error of 2^-24 of |d| (close pairs stay accurate);
//   * the phase of k = 2 pi n / L is n * X mod 2^32 exactly (integer
//     multiply-add), so e^{i k.r} = sincospi(phase * 2^-31) has no FP32
//     range-reduction error.
// In the slab geometry z is not wrapped (|dz| < H < L_z,Ewald / 2), so the same
// subtraction gives the raw dz the reference uses (GetDistVector, npbc = 2).
//
// Work decomposition is the FP64 kernel's: every (moved, other) pair dealt
// across the grid, k tiles x moved-bead groups with a last-arrival reduction.
// Per-thread and per-block sums are FP32; blocks are added in FP64 by the
// serial kernel.
#include <algorithm>
#include <cmath>

#include "engine.h"
#include "device_common.cuh"
#include "fp32_pair.cuh"

namespace plum {

constexpr int kKTile32 = 128;

template <int NT>
__device__ __forceinline__ float block_sum32(float v, float* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) sh[w] = v;
  __syncthreads();
  float t = 0.0f;
  if (threadIdx.x == 0)
    for (int i = 0; i < NT / 32; i++) t += sh[i];
  return t;
}

// Two sums at once (one pair of barriers); each value is added in
// block_sum32's order, so the results are the same bits as two calls.
// sh: 2 NT / 32 floats. Valid in thread 0.
template <int NT>
__device__ __forceinline__ float2 block_sum32x2(float a, float b, float* sh) {
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) {
    sh[w] = a;
    sh[NT / 32 + w] = b;
  }
  __syncthreads();
  float2 t = make_float2(0.0f, 0.0f);
  if (threadIdx.x == 0)
    for (int i = 0; i < NT / 32; i++) {
      t.x += sh[i];
      t.y += sh[NT / 32 + i];
    }
  return t;
}

__device__ __forceinline__ double block_sum_d(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) sh[w] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)blockDim.x / 32; i++) t += sh[i];
  return t;
}

// Exact per-entry table: e^{i 2 pi n X / 2^32}, n = 0..kmax, q folded into x.
__device__ __forceinline__ void table32(const DevParams& P, int4 f, float q, int axis,
                                        float2* tab) {
  const unsigned X = (unsigned)(axis == 0 ? f.x : (axis == 1 ? f.y : f.z));
  float2* t = tab + P.koff[axis];
  const float w = axis == 0 ? q : 1.0f;
  for (int n = 0; n <= P.kmax[axis]; n++) {
    unsigned ph = X * (unsigned)n;
    float s, c;
    sincospif((float)(int)ph * 4.6566128730773926e-10f, &s, &c);  // * 2^-31
    t[n] = make_float2(w * c, w * s);
  }
}

__device__ __forceinline__ float2 cmul32(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

__device__ __forceinline__ float2 phase32(const DevParams& P, const float2* tab, short4 k) {
  float2 ex = tab[P.koff[0] + k.x];
  float2 ey = tab[P.koff[1] + (k.y >= 0 ? k.y : -k.y)];
  if (k.y < 0) ey.y = -ey.y;
  float2 ez = tab[P.koff[2] + (k.z >= 0 ? k.z : -k.z)];
  if (k.z < 0) ez.y = -ez.y;
  return cmul32(cmul32(ex, ey), ez);
}

__global__ void __launch_bounds__(kPairThreads)
    k_delta32(const DevParams P, const DevBuffers B) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ float red[kPairThreads / 32];
  __shared__ double redd[kPairThreads / 32];
  __shared__ int s_last;
  const DevState* st = B.state;
  const int b_lo = st->b_lo, b_hi = st->b_hi;
  const int m = st->pending ? b_hi - b_lo : 0;
  const int sk_pend = st->sk_pending, sk_buf = st->sk_buf, cur_buf = st->cur_buf;
  __shared__ int s_final;
  const int N = P.n_bead;

  float acc_lj = 0.0f, acc_re = 0.0f;
  if (P.use_pair || P.use_ewald) {
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
      const int4 ti = B.ftrial[ii], ci = B.fpos[i];
      const float qi = B.fq[i], qj = B.fq[j];
      const int4 cj = B.fpos[j];
      const int4 tj = jm ? B.ftrial[j - b_lo] : cj;
      float l1 = 0, r1 = 0, l0 = 0, r0 = 0;
      pair32(P, ti, qi, tj, qj, l1, r1);
      pair32(P, ci, qi, cj, qj, l0, r0);
      if (!hs_bonded(P, B.mol_start, i, j)) acc_lj += l1 - l0;
      acc_re += r1 - r0;
    }
  }
  float t0 = block_sum32<kPairThreads>(acc_lj, red);
  float t1 = block_sum32<kPairThreads>(acc_re, red);
  if (threadIdx.x == 0) {
    B.partial[4 * blockIdx.x + 0] = (double)t0;
    B.partial[4 * blockIdx.x + 1] = (double)t1;
  }

  const bool kwork = P.use_ewald && m > 0;
  const int chunk = P.kchunk_delta;
  const int n_groups = kwork ? (m + chunk - 1) / chunk : 0;
  const int n_tiles = (P.n_k + kKTile32 - 1) / kKTile32;
  const int n_items = n_tiles * n_groups;
  float2* tabs = reinterpret_cast<float2*>(smem);  // [chunk][2][kper]
  const int per = P.kper;
  for (int item = blockIdx.x; item < n_items; item += gridDim.x) {
    const int tile = item % n_tiles, grp = item / n_tiles;
    const int c0 = b_lo + grp * chunk;
    const int cnt = min(chunk, b_hi - c0);
    __syncthreads();
    for (int t = threadIdx.x; t < cnt * 6; t += blockDim.x) {
      int bead = t / 6, which = (t / 3) & 1, axis = t % 3;
      int4 f = which ? B.fpos[c0 + bead] : B.ftrial[c0 - b_lo + bead];
      table32(P, f, B.fq[c0 + bead], axis, tabs + (bead * 2 + which) * per);
    }
    __syncthreads();
    const int k = tile * kKTile32 + threadIdx.x;
    const bool mine = threadIdx.x < kKTile32 && k < P.n_k;
    if (mine) {
      const short4 kv = B.kn[k];
      float2 ds = make_float2(0.0f, 0.0f);
      for (int b = 0; b < cnt; b++) {
        float2 e1 = phase32(P, tabs + (b * 2 + 0) * per, kv);
        float2 e0 = phase32(P, tabs + (b * 2 + 1) * per, kv);
        ds.x += e1.x - e0.x;
        ds.y += e1.y - e0.y;
      }
      B.dsk_part32[(size_t)grp * P.n_k + k] = ds;
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) s_last = atomicAdd(&B.ktile_count[tile], 1) == n_groups - 1;
    __syncthreads();
    if (s_last) {
      __threadfence();
      float e = 0.0f;
      if (mine) {
        float2 ds = make_float2(0.0f, 0.0f);
        for (int g = 0; g < n_groups; g++) {
          float2 v = __ldcg(&B.dsk_part32[(size_t)g * P.n_k + k]);
          ds.x += v.x;
          ds.y += v.y;
        }
        double2 s = B.sk[k];
        if (sk_pend) {
          const double2 p = B.dsk[(size_t)sk_buf * P.n_k + k];
          s = make_double2(s.x + p.x, s.y + p.y);
          B.sk[k] = s;
        }
        B.dsk[(size_t)cur_buf * P.n_k + k] = make_double2((double)ds.x, (double)ds.y);
        float sx = (float)s.x, sy = (float)s.y;
        e = (float)B.kw[k] * (2.0f * (sx * ds.x + sy * ds.y) + (ds.x * ds.x + ds.y * ds.y));
      }
      e = block_sum32<kPairThreads>(e, red);
      if (threadIdx.x == 0) {
        B.kpartial[tile] = (double)e;
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
    a = block_sum_d(a, redd);
    b = block_sum_d(b, redd);
    c = block_sum_d(c, redd);
    if (threadIdx.x == 0) {
      DevState* ws = B.state;
      ws->red_lj = a;
      ws->red_re = b;
      ws->red_k = c;
      *B.done_count = 0;
    }
  }
}

static int g_grid32 = 0;
int pair_grid32() {
  if (g_grid32 == 0) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    g_grid32 = 4 * (sms > 0 ? sms : 152);
  }
  return g_grid32;
}

void launch_delta_pairs32(const DevParams& P, const DevBuffers& B, cudaStream_t s) {
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_delta32, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         kKTableBytes + 4096);
    attr = true;
  }
  size_t smem = P.use_ewald ? (size_t)P.kchunk_delta * 2 * P.kper * sizeof(float2) : 0;
  k_delta32<<<pair_grid32(), kPairThreads, smem, s>>>(P, B);
}

// Loop constants of a replica's pair sweep, in registers.
struct PairConst {
  float sx, sy, sz, rc, sa, lB, ljmax2;
  int nt, use_pair, use_ewald;
};

__device__ __forceinline__ PairConst pair_const(const DevParams& P) {
  PairConst K;
  K.sx = P.f_scale[0];
  K.sy = P.f_scale[1];
  K.sz = P.f_scale[2];
  K.rc = P.f_real_cut;
  K.sa = P.f_sqrt_alpha;
  K.lB = P.f_lB;
  K.nt = P.n_type;
  K.use_pair = P.use_pair;
  K.use_ewald = P.use_ewald;
  // r2 = 0 (coincident beads) must reach lj32, which returns the overlap value
  float m2 = 1e-30f;
  for (int k = 0; k < P.n_type * P.n_type; k++) m2 = fmaxf(m2, P.f_lj_rc2[k]);
  K.ljmax2 = m2;
  return K;
}

// pair32 with the LJ table read only inside the largest LJ cut-off and, for
// kSingle (r_c <= L/2 on every axis), the minimum image inlined.
template <bool kSingle>
__device__ __forceinline__ void pair32k(const DevParams& P, const PairConst& K, int4 a, float qa,
                                        int4 b, float qb, float& lj, float& re) {
  const float dx = fdiff(a.x, b.x, K.sx);
  const float dy = fdiff(a.y, b.y, K.sy);
  const float dz = fdiff(a.z, b.z, K.sz);
  const float r2 = dx * dx + dy * dy + dz * dz;
  if (K.use_pair && r2 < K.ljmax2) lj += lj32(P, a.w * K.nt + b.w, r2);
  if (K.use_ewald) {
    const float qq = qa * qb;
    if (qq != 0.0f) {
      float e = 0.0f;
      if (kSingle) {
        if (r2 <= K.rc * K.rc) e = real_term32(P, r2);
      } else {
        e = real_images32(P, dx, dy, dz);
      }
      re += K.lB * qq * e;
    }
  }
}

// One thread per other bead j in [c0, c1) (moved beads skipped), against the
// gn staged moved beads at their trial (s_mt[u]) and current
// (s_mt[kPairGroup + u]) positions.
template <bool kSingle>
__device__ __forceinline__ void pair_sweep(const DevParams& P, const PairConst& K,
                                           const DevBuffers& B, const int4* s_mt,
                                           const float* s_mq, int gn, int g_lo, int c0, int c1,
                                           int b_lo, int b_hi, float& acc_lj, float& acc_re) {
  const bool hs = P.pair_kind == 1;
  for (int j = c0 + threadIdx.x; j < c1; j += kPairThreads) {
    if (j >= b_lo && j < b_hi) continue;  // moved pairs: the last item
    const int4 cj = B.fpos[j];
    const float qj = B.fq[j];
#pragma unroll 2
    for (int u = 0; u < gn; u++) {
      float l1 = 0, r1 = 0, l0 = 0, r0 = 0;
      pair32k<kSingle>(P, K, s_mt[u], s_mq[u], cj, qj, l1, r1);
      pair32k<kSingle>(P, K, s_mt[kPairGroup + u], s_mq[u], cj, qj, l0, r0);
      if (!(hs && hs_bonded(P, B.mol_start, g_lo + u, j))) acc_lj += l1 - l0;
      acc_re += r1 - r0;
    }
  }
}

// ------------------------------------------------ table-driven real space
// pair_sweep for LJ + Ewald with r_c <= L/2 on every axis, the real-space term
// from the h(u) table: per (moved u, other j) the trial and current distances
// share the other bead's load, one LJ pre-test and the packed (two-lane FP32)
// arithmetic of r^2 and u, so a warp runs no divergent erfc. Each thread takes
// two other beads per staged bead, so one load of the staged trial and
// current entries serves four evaluations; the other bead's charge multiplies
// its sum once, after the staged beads. kCubic (equal fixed-point scales on
// the three axes): r^2 stays in fixed-point units and the box scale is folded
// into the constants. kCut: the table is the batch's cut table (variable
// u' = cut_scale u, zero from the cut-off on), so the cut-off costs nothing;
// else the universal table and a select at r_c. gn4 staged beads, a multiple
// of 4; the trial entry's w holds the staged bead's charge (float bits) and
// the current entry's w its type; the padding beads have q = 0 and equal
// trial and current positions, so they add exactly zero.
template <bool kCubic, bool kCut>
__device__ __forceinline__ void pair_sweep_tab(const DevParams& P, const DevBuffers& B,
                                               const int4* s_mt, const float4* s_h, int gn4,
                                               int c0, int c1, int b_lo, int b_hi,
                                               float cut_scale, float& acc_lj, float& acc_re) {
  const float sx = P.f_scale[0], sy = P.f_scale[1], sz = P.f_scale[2];
  const float cs = kCubic ? sx * sx : 1.0f;  // real r^2 per unit of r2 below
  const float ics = 1.0f / cs;
  const float rc2 = P.f_real_cut * P.f_real_cut * ics;
  const float ua = P.f_sqrt_alpha * P.f_sqrt_alpha * cs * (kCut ? cut_scale : 1.0f);
  const float ius = kCut ? 1.0f / cut_scale : 1.0f;  // table variable -> u
  float ljm = 1e-30f;  // r2 = 0 (coincident beads) must reach lj32
  for (int k = 0; k < P.n_type * P.n_type; k++) ljm = fmaxf(ljm, P.f_lj_rc2[k]);
  const float ljlim = ljm * ics;
  const float pref = P.f_lB * P.f_sqrt_alpha;
  const int nt = P.n_type;
  const bool use_pair = P.use_pair;
  const float2 ua2 = make_float2(ua, ua);
  const float2 s2x = make_float2(sx, sx), s2y = make_float2(sy, sy), s2z = make_float2(sz, sz);
  // one evaluation pair (trial, current) of staged bead (t, c) with other
  // bead o; ok: o is an other bead of this item (not moved, inside the chunk)
  auto eval = [&](const int4 t, const int4 c, const int4 o, bool ok, float& acc) {
    float2 dx = make_float2((float)(int)((unsigned)o.x - (unsigned)t.x),
                            (float)(int)((unsigned)o.x - (unsigned)c.x));
    float2 dy = make_float2((float)(int)((unsigned)o.y - (unsigned)t.y),
                            (float)(int)((unsigned)o.y - (unsigned)c.y));
    float2 dz = make_float2((float)(int)((unsigned)o.z - (unsigned)t.z),
                            (float)(int)((unsigned)o.z - (unsigned)c.z));
    if (!kCubic) {
      dx = __fmul2_rn(dx, s2x);
      dy = __fmul2_rn(dy, s2y);
      dz = __fmul2_rn(dz, s2z);
    }
    const float2 r = __ffma2_rn(dx, dx, __ffma2_rn(dy, dy, __fmul2_rn(dz, dz)));
    if (use_pair && ok && fminf(r.x, r.y) < ljlim) {
      const int k = c.w * nt + o.w;  // trial and current share the type
      acc_lj += lj32(P, k, r.x * cs) - lj32(P, k, r.y * cs);
    }
    const float2 u = __fmul2_rn(r, ua2);
    const int b1 = __float_as_int(u.x), b0 = __float_as_int(u.y);
    float h1 = h32_tab(s_h, b1), h0 = h32_tab(s_h, b0);
    if (min(b1, b0) < kH32LoBits) {
      if (b1 < kH32LoBits) h1 = h32_small(u.x * ius);
      if (b0 < kH32LoBits) h0 = h32_small(u.y * ius);
    }
    if (!kCut) {
      h1 = r.x <= rc2 ? h1 : 0.0f;
      h0 = r.y <= rc2 ? h0 : 0.0f;
    }
    acc = fmaf(__int_as_float(t.w), h1 - h0, acc);
  };
  for (int j0 = c0 + threadIdx.x; j0 < c1; j0 += 2 * kPairThreads) {
    const int j1 = j0 + kPairThreads;
    const bool ok0 = !(j0 >= b_lo && j0 < b_hi);  // moved pairs: the last item
    const bool ok1 = j1 < c1 && !(j1 >= b_lo && j1 < b_hi);
    const int4 o0 = B.fpos[j0];
    const int4 o1 = j1 < c1 ? B.fpos[j1] : o0;
    const float q0 = ok0 ? B.fq[j0] * pref : 0.0f;
    const float q1 = ok1 ? B.fq[j1] * pref : 0.0f;
    float a0 = 0.0f, a1 = 0.0f;
#pragma unroll 4
    for (int u = 0; u < gn4; u++) {
      const int4 t = s_mt[u], c = s_mt[kPairGroup + u];
      eval(t, c, o0, ok0, a0);
      eval(t, c, o1, ok1, a1);
    }
    acc_re = fmaf(q0, a0, fmaf(q1, a1, acc_re));
  }
}

// The table (kH32Bins float4): per bin the cubic in w = f / 32 (f the
// bin-local fraction) through h(u' / scale) at the four Chebyshev nodes of the
// bin, h in double precision from std::erfc; the 4 x 4 Vandermonde system in
// f solved by Gaussian elimination with partial pivoting, the coefficients
// then scaled by powers of 32 (exactly) to the kernel's w. With cut > 0 every
// bin at or above u' = cut is zero.
void build_h32_table(float4* out, double scale, double cut) {
  const double kPi = 3.14159265358979323846;
  int i = 0;
  for (int e = kH32ELo; e < kH32EHi; e++)
    for (int j = 0; j < kH32Per; j++, i++) {
      const double lo = std::ldexp(1.0 + (double)j / kH32Per, e);
      const double w = std::ldexp(1.0 / kH32Per, e);
      if (cut > 0.0 && lo >= cut) {
        out[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        continue;
      }
      double A[4][5];
      for (int k = 0; k < 4; k++) {
        const double f = 0.5 + 0.5 * std::cos(kPi * (k + 0.5) / 4.0);  // in (0, 1)
        const double u = (lo + f * w) / scale;
        const double r = std::sqrt(u);
        double p = 1.0;
        for (int q = 0; q < 4; q++, p *= f) A[k][q] = p;
        A[k][4] = std::erfc(r) / r;
      }
      for (int col = 0; col < 4; col++) {
        int piv = col;
        for (int rr = col + 1; rr < 4; rr++)
          if (std::fabs(A[rr][col]) > std::fabs(A[piv][col])) piv = rr;
        for (int q = 0; q < 5; q++) std::swap(A[col][q], A[piv][q]);
        for (int rr = 0; rr < 4; rr++) {
          if (rr == col) continue;
          const double g = A[rr][col] / A[col][col];
          for (int q = col; q < 5; q++) A[rr][q] -= g * A[col][q];
        }
      }
      double c[4];
      for (int q = 0; q < 4; q++) c[q] = std::ldexp(A[q][4] / A[q][q], 5 * q);  // f^q = 32^q w^q
      out[i] = make_float4((float)c[0], (float)c[1], (float)c[2], (float)c[3]);
    }
}

// ------------------------------------------------------------ replicas
constexpr int kMaxKPerThread = 4;  // k vectors per thread of a k item (k_tile <= 1024)
static_assert(kMaxKPerThread * kPairThreads >= 1024, "k items of up to 1024 vectors");
// Batched replicas: every replica's pending move contributes pair items
// (up to kPairGroup moved beads, staged in shared memory at their trial and
// current positions, x a chunk of other beads, one per thread), one item for
// the pairs among the moved beads, and k items (one k tile of kKTile32
// vectors over all moved beads). Every block derives the same item list from
// the replicas' states and takes items one at a time from a queue; each item
// writes its own slot: pair items {lj, real}, k items {k-space energy
// change}. The serial step of each replica adds its slots in item order, so
// the result does not depend on which block took which item.
// The item sizes, the grid and the register budget (kMinBlocks resident
// blocks per SM) are run-time choices (BatchTune, picked by
// plum_batch_autotune); defaults: 4096 pairs per item, 128-vector k tiles,
// 4 blocks per SM, 2 resident.
template <int kMinBlocks>
__global__ void __launch_bounds__(kPairThreads, kMinBlocks)
    k_batch_delta32(const DevParams* __restrict__ rp, const DevBuffers* __restrict__ rb,
                    int n_rep, int* __restrict__ item_off, double* __restrict__ slots,
                    BatchTune tune, int* __restrict__ queue, const float4* __restrict__ htab,
                    float cut_scale) {
  const int kItemPairs = tune.item_pairs, kKTile32 = tune.k_tile;
  extern __shared__ __align__(16) unsigned char smem_all[];
  // with the h(u) table: the table first, then the staging / k-table area
  float4* s_h = reinterpret_cast<float4*>(smem_all);
  unsigned char* smem = smem_all + (htab ? kH32Bins * sizeof(float4) : 0);
  if (htab)
    for (int i = threadIdx.x; i < kH32Bins; i += blockDim.x) s_h[i] = htab[i];
  __shared__ float red[2 * (kPairThreads / 32)];
  __shared__ int s_pref[kMaxReplicas + 1];
  __shared__ int s_np[kMaxReplicas];
  __shared__ int s_total, s_item;
  // 1. item counts per replica and their prefix (same in every block)
  for (int r = threadIdx.x; r < n_rep; r += blockDim.x) {
    const DevState* st = rb[r].state;
    // a move rejected by the surrogate's stage one has no exact change
    const int m = (st->pending && !st->da_skip) ? st->b_hi - st->b_lo : 0;
    const DevParams& pr = rp[r];
    const int np = (pr.use_pair || pr.use_ewald) ? pair_item_count(m, pr.n_bead, kItemPairs) : 0;
    const int nk = (pr.use_ewald && m > 0) ? (pr.n_k + kKTile32 - 1) / kKTile32 : 0;
    s_np[r] = np;
    s_pref[r + 1] = np + nk;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    s_pref[0] = 0;
    for (int r = 0; r < n_rep; r++) s_pref[r + 1] += s_pref[r];
    s_total = s_pref[n_rep];
  }
  __syncthreads();
  if (blockIdx.x == 0)
    for (int r = threadIdx.x; r < n_rep; r += blockDim.x) {
      item_off[4 * r] = s_pref[r];
      item_off[4 * r + 1] = s_np[r];
      item_off[4 * r + 2] = s_pref[r] + s_np[r];
      item_off[4 * r + 3] = s_pref[r + 1] - s_pref[r] - s_np[r];
    }
  // 2. items are taken from a queue (queue[0]) one at a time: blocks that
  // drew cheap items take more. Every item writes only its own slot, so
  // the results do not depend on which block took it. The last block to
  // run out resets the queue for the next launch.
  const int T = s_total;
  for (;;) {
    __syncthreads();  // the previous item is done with s_item and the staging area
    if (threadIdx.x == 0) s_item = atomicAdd(&queue[0], 1);
    __syncthreads();
    const int item = s_item;
    if (item >= T) break;
    // replica of this item (s_pref is ascending)
    int lo = 0, hi = n_rep - 1;
    while (lo < hi) {
      int mid = (lo + hi + 1) >> 1;
      if (s_pref[mid] <= item) lo = mid; else hi = mid - 1;
    }
    const int r = lo;
    const DevParams& P = rp[r];
    const DevBuffers& B = rb[r];
    const DevState* st = B.state;
    const int b_lo = st->b_lo, b_hi = st->b_hi, m = b_hi - b_lo, N = P.n_bead;
    const int local = item - s_pref[r];
    if (local < s_np[r]) {
      float acc_lj = 0.0f, acc_re = 0.0f;
      const int chunk = pair_chunk(m, kItemPairs);
      const int n_chunk = (N + chunk - 1) / chunk;
      const int n_grid = ((m + kPairGroup - 1) / kPairGroup) * n_chunk;
      if (local < n_grid) {
        const int g0 = (local / n_chunk) * kPairGroup, gn = min(kPairGroup, m - g0);
        const int c0 = (local % n_chunk) * chunk, c1 = min(N, c0 + chunk);
        int4* s_mt = reinterpret_cast<int4*>(smem);  // trial, then current
        float* s_mq = reinterpret_cast<float*>(s_mt + 2 * kPairGroup);
        const bool tab = htab && P.single_image && P.pair_kind == 0 && P.use_ewald;
        // the table path pads the staged beads to a multiple of 4 with the
        // last bead's current position at both places and q = 0
        const int gn4 = tab ? (gn + 3) & ~3 : gn;
        // (the barrier at the top of the item loop: every thread is done
        // with the previous item's staging area)
        for (int u = threadIdx.x; u < gn4; u += kPairThreads) {
          if (u < gn) {
            int4 t = B.ftrial[g0 + u];
            if (tab) t.w = __float_as_int(B.fq[b_lo + g0 + u]);  // the type stays in c.w
            s_mt[u] = t;
            s_mt[kPairGroup + u] = B.fpos[b_lo + g0 + u];
            s_mq[u] = B.fq[b_lo + g0 + u];
          } else {
            const int4 p = B.fpos[b_lo + g0 + gn - 1];
            s_mt[u] = make_int4(p.x, p.y, p.z, __float_as_int(0.0f));
            s_mt[kPairGroup + u] = p;
            s_mq[u] = 0.0f;
          }
        }
        __syncthreads();
        const PairConst K = pair_const(P);
        if (tab) {
          const bool cubic =
              P.npbc == 3 && P.f_scale[0] == P.f_scale[1] && P.f_scale[1] == P.f_scale[2];
          if (cut_scale > 0.0f) {
            if (cubic)
              pair_sweep_tab<true, true>(P, B, s_mt, s_h, gn4, c0, c1, b_lo, b_hi, cut_scale,
                                         acc_lj, acc_re);
            else
              pair_sweep_tab<false, true>(P, B, s_mt, s_h, gn4, c0, c1, b_lo, b_hi, cut_scale,
                                          acc_lj, acc_re);
          } else if (cubic) {
            pair_sweep_tab<true, false>(P, B, s_mt, s_h, gn4, c0, c1, b_lo, b_hi, 0.0f, acc_lj,
                                        acc_re);
          } else {
            pair_sweep_tab<false, false>(P, B, s_mt, s_h, gn4, c0, c1, b_lo, b_hi, 0.0f, acc_lj,
                                         acc_re);
          }
        } else if (P.single_image)
          pair_sweep<true>(P, K, B, s_mt, s_mq, gn, b_lo + g0, c0, c1, b_lo, b_hi, acc_lj,
                           acc_re);
        else
          pair_sweep<false>(P, K, B, s_mt, s_mq, gn, b_lo + g0, c0, c1, b_lo, b_hi, acc_lj,
                            acc_re);
      } else {
        // pairs among the moved beads, each once (both trial / both current)
        const int lane = threadIdx.x & 31;
        for (int a = threadIdx.x >> 5; a < m; a += kPairThreads / 32)
          for (int bb = a + 1 + lane; bb < m; bb += 32) {
          float l1 = 0, r1 = 0, l0 = 0, r0 = 0;
          pair32(P, B.ftrial[a], B.fq[b_lo + a], B.ftrial[bb], B.fq[b_lo + bb], l1, r1);
          pair32(P, B.fpos[b_lo + a], B.fq[b_lo + a], B.fpos[b_lo + bb], B.fq[b_lo + bb], l0,
                 r0);
          // the moved beads are one molecule's: neighbours are bonded
          if (!(P.pair_kind == 1 && bb == a + 1)) acc_lj += l1 - l0;
          acc_re += r1 - r0;
        }
      }
      const float2 ab = block_sum32x2<kPairThreads>(acc_lj, acc_re, red);
      if (threadIdx.x == 0) {
        slots[2 * item] = (double)ab.x;
        slots[2 * item + 1] = (double)ab.y;
      }
    } else {
      // a k item of up to kMaxKPerThread * kPairThreads vectors: thread t
      // takes nq consecutive vectors k = tile * k_tile + t nq + q, so the
      // moved beads' phase tables, built once per item, serve up to four
      // vectors per thread, and vectors of one (nx, ny) column (n_z runs
      // fastest in the k list) share the product e^{i(kx x + ky y)}: the
      // phase of each is the same cmul(cmul(ex, ey), ez) as phase32's
      const int tile = local - s_np[r];
      const int sk_pend = st->sk_pending, sk_buf = st->sk_buf, cur_buf = st->cur_buf;
      const int nq = (kKTile32 + kPairThreads - 1) / kPairThreads;
      int kk[kMaxKPerThread];
      bool mine[kMaxKPerThread], col[kMaxKPerThread];
      int ox[kMaxKPerThread], oy[kMaxKPerThread], oz[kMaxKPerThread];
      bool ny[kMaxKPerThread], nz[kMaxKPerThread];
      float2 ds[kMaxKPerThread];
#pragma unroll
      for (int q = 0; q < kMaxKPerThread; q++) {
        const int t = threadIdx.x * nq + q;
        kk[q] = tile * kKTile32 + t;
        mine[q] = q < nq && t < kKTile32 && kk[q] < P.n_k;
        const short4 kv = mine[q] ? B.kn[kk[q]] : make_short4(0, 0, 0, 0);
        ox[q] = P.koff[0] + kv.x;
        oy[q] = P.koff[1] + (kv.y >= 0 ? kv.y : -kv.y);
        oz[q] = P.koff[2] + (kv.z >= 0 ? kv.z : -kv.z);
        ny[q] = kv.y < 0;
        nz[q] = kv.z < 0;
        // a new (nx, ny) column: recompute the xy product
        col[q] = q == 0 || ox[q] != ox[q - 1] || oy[q] != oy[q - 1] || ny[q] != ny[q - 1];
        ds[q] = make_float2(0.0f, 0.0f);
      }
      float2* tabs = reinterpret_cast<float2*>(smem);
      const int per = P.kper, chunk = P.kchunk_delta;
      for (int c0 = b_lo; c0 < b_hi; c0 += chunk) {
        const int cnt = min(chunk, b_hi - c0);
        __syncthreads();
        for (int t = threadIdx.x; t < cnt * 6; t += blockDim.x) {
          int bead = t / 6, which = (t / 3) & 1, axis = t % 3;
          int4 f = which ? B.fpos[c0 + bead] : B.ftrial[c0 - b_lo + bead];
          table32(P, f, B.fq[c0 + bead], axis, tabs + (bead * 2 + which) * per);
        }
        __syncthreads();
        if (mine[0])
          for (int bb = 0; bb < cnt; bb++) {
            const float2* t1 = tabs + (bb * 2 + 0) * per;
            const float2* t0 = t1 + per;
            float2 xy1 = make_float2(0.0f, 0.0f), xy0 = xy1;
#pragma unroll
            for (int q = 0; q < kMaxKPerThread; q++)
              if (mine[q]) {
                if (col[q]) {
                  float2 y1 = t1[oy[q]], y0 = t0[oy[q]];
                  if (ny[q]) {
                    y1.y = -y1.y;
                    y0.y = -y0.y;
                  }
                  xy1 = cmul32(t1[ox[q]], y1);
                  xy0 = cmul32(t0[ox[q]], y0);
                }
                float2 z1 = t1[oz[q]], z0 = t0[oz[q]];
                if (nz[q]) {
                  z1.y = -z1.y;
                  z0.y = -z0.y;
                }
                const float2 e1 = cmul32(xy1, z1), e0 = cmul32(xy0, z0);
                ds[q].x += e1.x - e0.x;
                ds[q].y += e1.y - e0.y;
              }
          }
      }
      float e = 0.0f;
#pragma unroll
      for (int q = 0; q < kMaxKPerThread; q++)
        if (mine[q]) {
          const int k = kk[q];
          double2 sv = B.sk[k];
          if (sk_pend) {
            const double2 pd = B.dsk[(size_t)sk_buf * P.n_k + k];
            sv = make_double2(sv.x + pd.x, sv.y + pd.y);
            B.sk[k] = sv;
          }
          const float2 d = ds[q];
          B.dsk[(size_t)cur_buf * P.n_k + k] = make_double2((double)d.x, (double)d.y);
          const float sx = (float)sv.x, sy = (float)sv.y;
          e += (float)B.kw[k] * (2.0f * (sx * d.x + sy * d.y) + (d.x * d.x + d.y * d.y));
        }
      e = block_sum32<kPairThreads>(e, red);
      if (threadIdx.x == 0) {
        slots[2 * item] = (double)e;
        slots[2 * item + 1] = 0.0;
      }
    }
  }
  // every block takes its last (empty) item before it counts itself out, so
  // the last one out knows that no block will read the queue again
  if (threadIdx.x == 0 && atomicAdd(&queue[1], 1) == (int)gridDim.x - 1) {
    queue[0] = 0;
    queue[1] = 0;
  }
}

void launch_batch_delta32(const DevParams* rp, const DevBuffers* rb, int n_rep, int* item_off,
                          double* slots, size_t smem, BatchTune tune, int* queue,
                          const float4* htab, float cut_scale, cudaStream_t s) {
  static bool attr = false;
  if (!attr) {
    const int most = kKTableBytes + 4096 + kH32Bins * (int)sizeof(float4);
    cudaFuncSetAttribute(k_batch_delta32<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, most);
    cudaFuncSetAttribute(k_batch_delta32<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, most);
    cudaFuncSetAttribute(k_batch_delta32<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, most);
    attr = true;
  }
  const int grid = tune.grid > 0 ? tune.grid : pair_grid32();
  if (!tune.htab) htab = nullptr;
  if (!htab) cut_scale = 0.0f;
  if (htab) smem += kH32Bins * sizeof(float4);
  if (tune.min_blocks == 4)
    k_batch_delta32<4><<<grid, kPairThreads, smem, s>>>(rp, rb, n_rep, item_off, slots, tune,
                                                        queue, htab, cut_scale);
  else if (tune.min_blocks == 3)
    k_batch_delta32<3><<<grid, kPairThreads, smem, s>>>(rp, rb, n_rep, item_off, slots, tune,
                                                        queue, htab, cut_scale);
  else
    k_batch_delta32<2><<<grid, kPairThreads, smem, s>>>(rp, rb, n_rep, item_off, slots, tune,
                                                        queue, htab, cut_scale);
}

__global__ void k_fix_all(const DevParams P, const DevBuffers B) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P.n_bead; i += gridDim.x * blockDim.x) {
    double4_32a p = B.pos[i];
    B.fpos[i] = fix_point(P, p, B.type[i]);
    B.fq[i] = (float)p.w;
  }
}

__global__ void k_fix_trial(const DevParams P, const DevBuffers B) {
  const DevState* st = B.state;
  for (int i = st->b_lo + threadIdx.x; i < st->b_hi; i += blockDim.x)
    B.ftrial[i - st->b_lo] = fix_point(P, B.trial[i], B.type[i]);
}

void launch_fix_all(const DevParams& P, const DevBuffers& B, cudaStream_t s) {
  k_fix_all<<<(P.n_bead + 255) / 256, 256, 0, s>>>(P, B);
}

void launch_fix_trial(const DevParams& P, const DevBuffers& B, cudaStream_t s) {
  k_fix_trial<<<1, 256, 0, s>>>(P, B);
}

}  // namespace plum
