// Serial part of a Monte Carlo step (one CTA):
//
//   finish  adds the per-block partials of k_delta64 in a fixed order, adds
//           the wall (potential_external.cc:100-117) and bond
//           (potential_spring.cc:63-80) terms, and composes dE exactly as
//           ForceField::EnergyDifference does (force_field.cc:407-434): pair,
//           early return at >= 1e8, external, early return, Ewald (real +
//           reciprocal + the dipole term from the *current* z, which is what
//           the reference evaluates at potential_ewald.cc:527-531), bond.
//   decide  one draw u; accept if dE < 1e8 and u < exp(-beta dE); no draw at
//           dE >= 1e8 (simulation.cc:324-332)
//   commit  trial -> current, S(k) += dS(k), running totals
//           (force_field.cc:436-451, simulation.cc:336-351)
//   gen     the next step's draws in the reference's order: one draw for the
//           GC check (simulation.cc:221), chain and ion picks, move type
//           (simulation.cc:247-276), then the move itself (molecule.cc:103-312)
//
// Build note: this file is compiled with -fmad=false. The draw-consuming
// tests (randSphere's r1^2 + r2^2 > 1, the move-type and pick thresholds)
// must round exactly like the reference or the draw sequence would diverge.
#include "engine.h"
#include "mlp.h"
#include "device_common.cuh"
#include "unit_draw.h"

namespace plum {


struct Draws {
  const uint32_t* g;
  const uint32_t* win;
  long long pos, len, wbase;
  int wlen;
  int overrun;
  __device__ uint32_t next() {
    if (pos >= len) {
      overrun = 1;
      return 0u;
    }
    long long o = pos - wbase;
    uint32_t v = (o >= 0 && o < wlen) ? win[o] : g[pos];
    pos++;
    return v;
  }
  __device__ double u() { return unit_draw(next()); }
  __device__ uint32_t at(long long o) const {
    long long w = o - wbase;
    return (w >= 0 && w < wlen) ? win[w] : g[o];
  }
};

// randSphere (misc.cc:95-109) rejects the pair (u1, u2) while
// r1^2 + r2^2 > 1 with r = 1 - 2 u / M, M = 2^32 - 1. In exact arithmetic
// that is (M - 2 u1)^2 + (M - 2 u2)^2 > M^2, decided here in 64-bit integers.
// The reference decides it in FP64, whose rounding can only matter within a
// few ulps of the unit circle; there (|difference| < 2^26 of M^2 ~ 1.8e19)
// the reference's own FP64 expression decides.
__device__ __forceinline__ bool sphere_reject(uint32_t u1, uint32_t u2) {
  const long long M = 4294967295LL;
  long long a = M - 2LL * (long long)u1, b = M - 2LL * (long long)u2;
  unsigned long long a2 = (unsigned long long)(a < 0 ? -a : a);
  unsigned long long b2 = (unsigned long long)(b < 0 ? -b : b);
  a2 *= a2;
  b2 *= b2;
  const unsigned long long M2 = 18446744065119617025ull;  // (2^32 - 1)^2
  const unsigned long long rhs = M2 - b2;
  const unsigned long long diff = a2 > rhs ? a2 - rhs : rhs - a2;
  if (diff > (1ull << 26)) return a2 > rhs;
  double r1 = 1.0 - 2.0 * unit_draw(u1);
  double r2 = 1.0 - 2.0 * unit_draw(u2);
  return r1 * r1 + r2 * r2 > 1.0;
}

// Consumes randSphere's draws; returns the stream index of the accepted pair.
__device__ long long sphere_scan(Draws& d) {
  for (int guard = 0; guard < (1 << 20); guard++) {
    long long o = d.pos;
    uint32_t u1 = d.next(), u2 = d.next();
    if (d.overrun) return -1;
    if (!sphere_reject(u1, u2)) return o;
  }
  d.overrun = 1;
  return -1;
}

// Same, using accept bits precomputed by the block for every window
// position p: bit p set when the pair (p, p+1) is accepted. A pair starting at
// `pos` is followed by the pair at pos+2, so thread 0 looks for the next set
// bit of pos's parity; past the window it falls back to sphere_scan.
__device__ long long sphere_scan_bits(Draws& d, const unsigned* accbits) {
  const long long rel0 = d.pos - d.wbase;
  if (rel0 < 0) return sphere_scan(d);
  long long rel = rel0;
  while (rel + 1 < d.wlen) {
    const int w = (int)(rel >> 5), b = (int)(rel & 31);
    const unsigned par = (rel & 1) ? 0xAAAAAAAAu : 0x55555555u;
    const unsigned msk = accbits[w] & par & (0xFFFFFFFFu << b);
    if (msk) {
      const long long p = ((long long)w << 5) + (__ffs(msk) - 1);
      d.pos = d.wbase + p + 2;
      return d.wbase + p;
    }
    rel = ((long long)(w + 1) << 5) + (rel0 & 1);
  }
  // every pair of this parity inside the window was rejected: continue from
  // the first pair not covered by the bits
  if (rel0 + 1 < d.wlen) d.pos = d.wbase + rel0 + 2 * ((d.wlen - rel0) / 2);
  return sphere_scan(d);
}

// The unit vector randSphere returns for an accepted pair.
__device__ void sphere_vec(uint32_t u1, uint32_t u2, double* v) {
  double r1 = 1.0 - 2.0 * unit_draw(u1);
  double r2 = 1.0 - 2.0 * unit_draw(u2);
  double rs = r1 * r1 + r2 * r2;
  double ranh = 2.0 * sqrt(1.0 - rs);
  v[0] = r1 * ranh;
  v[1] = r2 * ranh;
  v[2] = (1.0 - 2.0 * rs);
}

__device__ void rand_sphere(Draws& d, double* v, const unsigned* accbits) {
  long long o = sphere_scan_bits(d, accbits);
  if (o < 0) {
    v[0] = v[1] = 0.0;
    v[2] = 1.0;
    return;
  }
  sphere_vec(d.at(o), d.at(o + 1), v);
}

template <int NT>
__device__ __forceinline__ double bsum(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) sh[w] = v;
  __syncthreads();
  double t = 0.0;
  for (int i = 0; i < NT / 32; i++) t += sh[i];
  __syncthreads();
  return t;  // valid in every thread
}

// Three block sums at once (two barriers for all three, plus one before sh
// is reused); each value is added in bsum's order, so the results are the
// same bits as three bsum calls. sh: 3 NT / 32 doubles.
template <int NT>
__device__ __forceinline__ void bsum3(double& a, double& b, double& c, double* sh) {
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
    c += __shfl_xor_sync(0xffffffffu, c, o);
  }
  constexpr int W = NT / 32;
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) {
    sh[w] = a;
    sh[W + w] = b;
    sh[2 * W + w] = c;
  }
  __syncthreads();
  double ta = 0.0, tb = 0.0, tc = 0.0;
  for (int i = 0; i < W; i++) {
    ta += sh[i];
    tb += sh[W + i];
    tc += sh[2 * W + i];
  }
  __syncthreads();
  a = ta;
  b = tb;
  c = tc;
}

struct GenPlan {
  int type;      // move type, -1 none
  int mol, b0, b1, b_lo, b_hi;
  double vec[3];  // COM shift / reptation end step
  double R[9];    // crankshaft rotation
  int first;      // crankshaft first bead (molecule-relative)
  int dir;        // reptation direction
  int end;        // reptation end bead (molecule-relative)
  double s;       // pivot displacement size
  int pivot;      // pivot bead (molecule-relative); -1: generated sequentially
  int scan;       // pivot: the block locates the beads' draws (pivot_draws)
  int scan_rel;   // window offset of the first bead's draws
  int scan_ok;    // every bead's draws lay inside the window
  int scan_end;   // window offset after the last bead's draws
};

constexpr int kPivotMax = 512;  // chains up to this length pivot in parallel
constexpr int kJumpLevels = 9;  // 2^9 >= kPivotMax - 1 beads per pivot

// First window position q >= x of x's parity whose pair (q, q+1) randSphere
// accepts, kDrawWindow if there is none: the bit scan sphere_scan_bits makes
// from window offset x, without consuming anything.
__device__ __forceinline__ int next_accept(const unsigned* accbits, int wlen, int x) {
  if (x + 1 >= wlen) return kDrawWindow;
  const unsigned par = (x & 1) ? 0xAAAAAAAAu : 0x55555555u;
  int w = x >> 5;
  unsigned m = accbits[w] & par & (0xFFFFFFFFu << (x & 31));
  while (!m) {
    if (++w >= kDrawWindow / 32) return kDrawWindow;
    m = accbits[w] & par;
  }
  return (w << 5) + (__ffs(m) - 1);
}

// Molecule::Pivot's draws for every bead at once. Bead k of the scan order
// (forward from the pivot, then backward) takes randSphere's accepted pair at
// p_k and, with the bond potential on, one bond-length draw at p_k + 2, so
// p_{k+1} = next_accept(p_k + step) with step 2 or 3: thread 0's sequential
// scan is the chain p_0 = next_accept(rel0), p_k = F^k(p_0). The block tabulates
// F^(2^l) for every window offset (pointer doubling) and each thread composes
// the jumps of its bead's rank. Offsets, and therefore results, are those of
// the sequential scan; plan.scan_ok is cleared when any bead's draws run past
// the window, and thread 0 then makes the sequential scan instead.
__device__ __forceinline__ void pivot_draws(const DevParams& P, int wlen, GenPlan& plan,
                                            int* s_off, int* s_boff,
                                            short (*jump)[kDrawWindow + 1],
                                            const unsigned* accbits) {
  const int step = P.vary_bond ? 3 : 2;
  const int len = plan.b1 - plan.b0, pv = plan.pivot;
  const int n = len - 1, nf = len - 1 - pv;
  int nl = 0;
  while ((1 << nl) < n) nl++;  // ranks 0 .. n-1 need nl bits
  for (int x = threadIdx.x; x <= kDrawWindow; x += blockDim.x)
    jump[0][x] = (short)(x < kDrawWindow ? next_accept(accbits, wlen, x + step) : kDrawWindow);
  for (int l = 1; l < nl; l++) {
    __syncthreads();
    for (int x = threadIdx.x; x <= kDrawWindow; x += blockDim.x)
      jump[l][x] = jump[l - 1][jump[l - 1][x]];
  }
  if (threadIdx.x == 0) {
    plan.scan_ok = 1;
    plan.scan_end = plan.scan_rel;
  }
  __syncthreads();
  const int p0 = next_accept(accbits, wlen, plan.scan_rel);
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    int p = p0;
    for (int l = 0; l < nl; l++)
      if ((k >> l) & 1) p = jump[l][p];
    const int i = k < nf ? pv + 1 + k : pv - 1 - (k - nf);
    if (p >= kDrawWindow || p + step > wlen) {
      plan.scan_ok = 0;  // every writer stores the same value
    } else {
      s_off[i] = p;
      s_boff[i] = p + 2;
    }
    if (k == n - 1) plan.scan_end = p + step;
  }
  __syncthreads();
}

// Thread 0, after the move's own draws: delayed acceptance's stage-one draw,
// the stream check and the stream position.
__device__ __forceinline__ void gen_tail(DevState* st, const DevBuffers& B, Draws& d,
                                         GenPlan& plan) {
  // Delayed acceptance: a chain move (pivot, crankshaft, reptation) takes
  // its stage-one draw right after its own draws.
  if (plan.type >= 2 && st->da_on && B.desc_acc && B.desc_fine) st->da_u1 = d.u();
  if (d.overrun) {
    st->error = PLUM_ERR_STREAM_DEV;
    plan.type = -1;
  }
  st->stream_pos = d.pos;
}

// Thread 0's sequential pivot scan for chains up to kPivotMax beads: records
// each bead's draw offsets for the block.
__device__ __forceinline__ void pivot_draws_seq(const DevParams& P, Draws& d, long long wbase,
                                                int len, int pivot, int* s_off, int* s_boff,
                                                const unsigned* accbits) {
  for (int dirn = 0; dirn < 2; dirn++) {
    int i = dirn == 0 ? pivot + 1 : pivot - 1;
    for (; dirn == 0 ? i < len : i >= 0; i += dirn == 0 ? 1 : -1) {
      long long o = sphere_scan_bits(d, accbits);
      s_off[i] = (int)(o - wbase);
      if (P.vary_bond) {
        s_boff[i] = (int)(d.pos - wbase);
        (void)d.next();
      }
      if (d.overrun) break;
    }
  }
}

// The trial position of bead i, and its fixed-point mirror for the precision
// form's pair sweep.
__device__ __forceinline__ void put_trial(const DevParams& P, const DevBuffers& B, int b_lo, int i,
                                          double4_32a t) {
  B.trial[i] = t;
  if (P.form) B.ftrial[i - b_lo] = fix_point(P, t, B.type[i]);
}

// Generates the next step's trial move into `trial` (and the fixed-point
// mirror for the precision form); thread 0 consumes the draws, the block
// applies the geometry.
__device__ __forceinline__ void gen_move(const DevParams& P, const DevBuffers& B, DevState& S,
                                      Draws& d, long long wbase, GenPlan& plan, int* s_off,
                                      int* s_boff, double (*s_w)[kPivotMax],
                                      short (*jump)[kDrawWindow + 1],
                                      const unsigned* accbits) {
  DevState* const st = &S;
  // ----------------------------------------------------- generate next move
  if (threadIdx.x == 0) {
    plan.type = -1;
    plan.scan = 0;
    st->step_open = 1;
    (void)d.next();  // simulation.cc:221 (the GC draw)
    const int n_ch = P.n_chain_total, n_io = P.n_ion_total;
    if (P.n_mol - P.phantom > 0) {
      int wc = (int)floor(unit_draw(d.next()) * n_ch);
      int wi = (int)floor(unit_draw(d.next()) * n_io);
      if (wc == n_ch) wc--;
      if (wi == n_io) wi--;
      int chain_id = (wc >= 0 && wc < n_ch) ? B.chain_ids[wc] : -1;
      int ion_id = (wi >= 0 && wi < n_io) ? B.ion_ids[wi] : -1;
      int mt = 0;
      double u = unit_draw(d.next());
      double cur = P.move_prob[0];
      while (cur < u && mt < 4) {
        mt++;
        cur += P.move_prob[mt];
      }
      if (cur < u) mt++;
      if (mt > 4) mt = 4;
      int molid = -1;
      if (mt == 0 && n_io > 0)
        molid = ion_id;
      else if (n_ch > 0)
        molid = chain_id;
      const bool attempted = (mt == 0 && n_io > 0) || (mt > 0 && n_ch > 0);
      if (attempted && molid >= 0) {
        const int b0 = B.mol_start[molid], b1 = B.mol_start[molid + 1];
        const int len = b1 - b0;
        plan.mol = molid;
        plan.b0 = b0;
        plan.b1 = b1;
        plan.b_lo = b0;
        plan.b_hi = b1;
        plan.type = mt;
        if (mt == 0) {
          // Molecule::BeadTranslate (molecule.cc:103-133)
          double v[3];
          rand_sphere(d, v, accbits);
          double vl = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
          if (vl > 0) vl = 3 * P.move_size / vl;
          for (int a = 0; a < 3; a++) plan.vec[a] = vl * v[a];
          plan.b_hi = b0 + 1;
        } else if (mt == 1) {
          // Molecule::COMTranslate (molecule.cc:135-151). Here, and in the
          // pivot and crankshaft picks, the reference multiplies the word
          // before dividing, so these keep the division (unit_draw is the
          // quotient of the word alone).
          for (int a = 0; a < 3; a++) plan.vec[a] = 0.5 * P.move_size * (double)d.next() / kMtMax;
          for (int a = 0; a < 3; a++)
            if (d.next() % 2u == 0u) plan.vec[a] = -plan.vec[a];
        } else if (mt == 2) {
          // Molecule::Pivot (molecule.cc:153-237). Bead i's new position is
          // the previous one plus bl_i * unit(old_i - old_prev + s v_i): the
          // reference's running translation of the chain tail cancels out of
          // the bond direction. Thread 0 only locates each bead's draws; the
          // geometry and the running sum are done by the block below.
          int pivot = (int)floor(len * (double)d.next() / kMtMax);
          if (pivot == len) pivot--;
          double s = P.move_size * (double)d.next() / kMtMax;
          plan.s = s;
          plan.pivot = pivot;
          if (len <= kPivotMax) {
            // the block locates every bead's draws (pivot_draws)
            plan.scan = 1;
            plan.scan_rel = (int)(d.pos - wbase);
          } else {
            plan.pivot = -1;
            const double eq = P.bond_len;
            for (int dirn = 0; dirn < 2; dirn++) {
              double T[3] = {0.0, 0.0, 0.0};
              double4_32a pv = B.pos[b0 + pivot];
              double prev[3] = {pv.x, pv.y, pv.z};
              int i = dirn == 0 ? pivot + 1 : pivot - 1;
              for (; dirn == 0 ? i < len : i >= 0; i += dirn == 0 ? 1 : -1) {
                double v[3];
                rand_sphere(d, v, accbits);
                double4_32a o = B.pos[b0 + i];
                double p[3] = {o.x + T[0], o.y + T[1], o.z + T[2]};
                double dx = (p[0] + s * v[0]) - prev[0];
                double dy = (p[1] + s * v[1]) - prev[1];
                double dz = (p[2] + s * v[2]) - prev[2];
                double bl = eq;
                if (P.vary_bond) bl += (eq / 5.0) * (unit_draw(d.next()) - 0.5);
                double norm = bl / sqrt(dx * dx + dy * dy + dz * dz);
                double c[3] = {norm * dx + prev[0], norm * dy + prev[1], norm * dz + prev[2]};
                for (int a = 0; a < 3; a++) {
                  T[a] += c[a] - p[a];
                  prev[a] = c[a];
                }
                B.trial[b0 + i] = make_double4_32a(c[0], c[1], c[2], o.w);
                if (d.overrun) break;
              }
            }
          }
        } else if (mt == 3) {
          // Molecule::Crankshaft (molecule.cc:239-265); Rodrigues rotation in
          // the per-entry grouping of Eigen's AngleAxis::toRotationMatrix.
          int first = (int)floor((len - 2) * (double)d.next() / kMtMax);
          int last = (int)floor((len - first) * (double)d.next() / kMtMax) + first;
          if (last > len - 1) last = len - 1;  // the reference reads past the chain here
          double4_32a pf = B.pos[b0 + first], pl = B.pos[b0 + last];
          double ax[3] = {pl.x - pf.x, pl.y - pf.y, pl.z - pf.z};
          double z2 = ax[0] * ax[0] + ax[1] * ax[1] + ax[2] * ax[2];
          if (z2 > 0) {
            double n = sqrt(z2);
            for (int a = 0; a < 3; a++) ax[a] /= n;
          }
          const double pi_libm = 3.14159265358979323846;
          double ang = P.move_size * (unit_draw(d.next()) * 2 * pi_libm - pi_libm);
          double sn, cs;
          sincos(ang, &sn, &cs);
          double sa[3] = {sn * ax[0], sn * ax[1], sn * ax[2]};
          double ca[3] = {(1.0 - cs) * ax[0], (1.0 - cs) * ax[1], (1.0 - cs) * ax[2]};
          double t = ca[0] * ax[1];
          plan.R[1] = t - sa[2];
          plan.R[3] = t + sa[2];
          t = ca[0] * ax[2];
          plan.R[2] = t + sa[1];
          plan.R[6] = t - sa[1];
          t = ca[1] * ax[2];
          plan.R[5] = t - sa[0];
          plan.R[7] = t + sa[0];
          for (int a = 0; a < 3; a++) plan.R[4 * a] = ca[a] * ax[a] + cs;
          plan.first = first;
          plan.b_lo = b0 + first + 1;
          plan.b_hi = b0 + (last > first + 1 ? last : first + 1);
        } else {
          // Molecule::RandomReptation (molecule.cc:267-312)
          double bl = P.bond_len;
          if (P.vary_bond) bl += (P.bond_len / 5.0) * (unit_draw(d.next()) - 0.5);
          int dir = 1, end = len - 1;
          if (d.next() % 2u == 0u) {
            dir = -1;
            end = 0;
          }
          double v[3];
          rand_sphere(d, v, accbits);
          double vl = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
          for (int a = 0; a < 3; a++) plan.vec[a] = bl * v[a] / vl;
          plan.dir = dir;
          plan.end = end;
        }
      }
    }
    if (!plan.scan) gen_tail(st, B, d, plan);
  }
  __syncthreads();
  if (plan.scan) {
    pivot_draws(P, d.wlen, plan, s_off, s_boff, jump, accbits);
    if (threadIdx.x == 0) {
      if (plan.scan_ok) {
        d.pos = wbase + plan.scan_end;
      } else {
        d.pos = wbase + plan.scan_rel;
        pivot_draws_seq(P, d, wbase, plan.b1 - plan.b0, plan.pivot, s_off, s_boff, accbits);
      }
      gen_tail(st, B, d, plan);
    }
    __syncthreads();
  }
  // Apply the plan in parallel (the sequential pivot of a long chain already
  // wrote its trial positions).
  const GenPlan g = plan;
  if (g.type == 0 || g.type == 1) {
    for (int i = g.b_lo + threadIdx.x; i < g.b_hi; i += blockDim.x) {
      double4_32a o = B.pos[i];
      put_trial(P, B, g.b_lo, i,
                make_double4_32a(o.x + g.vec[0], o.y + g.vec[1], o.z + g.vec[2], o.w));
    }
  } else if (g.type == 3) {
    const double4_32a pf = B.pos[g.b0 + g.first];
    for (int i = g.b_lo + threadIdx.x; i < g.b_hi; i += blockDim.x) {
      double4_32a o = B.pos[i];
      double v[3] = {o.x - pf.x, o.y - pf.y, o.z - pf.z};
      double r[3];
      for (int a = 0; a < 3; a++)
        r[a] = ((g.R[3 * a] * v[0] + g.R[3 * a + 1] * v[1]) + g.R[3 * a + 2] * v[2]);
      put_trial(P, B, g.b_lo, i, make_double4_32a(r[0] + pf.x, r[1] + pf.y, r[2] + pf.z, o.w));
    }
  } else if (g.type == 2 && g.pivot >= 0) {
    const int len = g.b1 - g.b0, pv = g.pivot;
    const double eq = P.bond_len;
    for (int i = threadIdx.x; i < len; i += blockDim.x) {
      if (i == pv) continue;
      const int j = i > pv ? i - 1 : i + 1;
      double v[3];
      sphere_vec(d.at(wbase + s_off[i]), d.at(wbase + s_off[i] + 1), v);
      double bl = eq;
      if (P.vary_bond) bl += (eq / 5.0) * (unit_draw(d.at(wbase + s_boff[i])) - 0.5);
      const double4_32a oi = B.pos[g.b0 + i], oj = B.pos[g.b0 + j];
      double dx = (oi.x - oj.x) + g.s * v[0];
      double dy = (oi.y - oj.y) + g.s * v[1];
      double dz = (oi.z - oj.z) + g.s * v[2];
      double norm = bl / sqrt(dx * dx + dy * dy + dz * dz);
      // scan slot: forward beads first (pivot+1 ..), then backward (pivot-1 ..)
      const int k = i > pv ? i - pv - 1 : (len - 1 - pv) + (pv - 1 - i);
      s_w[0][k] = norm * dx;
      s_w[1][k] = norm * dy;
      s_w[2][k] = norm * dz;
    }
    // Inclusive running sums within the two segments (Hillis-Steele).
    const int nf = len - 1 - pv, n = len - 1;
    for (int off = 1; off < n; off <<= 1) {
      __syncthreads();
      double add[3][2];
      for (int r = 0; r < 2; r++) {
        int k = threadIdx.x + r * blockDim.x;
        bool ok = k < n && (k < nf ? k - off >= 0 : k - off >= nf);
        for (int a = 0; a < 3; a++) add[a][r] = ok ? s_w[a][k - off] : 0.0;
      }
      __syncthreads();
      for (int r = 0; r < 2; r++) {
        int k = threadIdx.x + r * blockDim.x;
        if (k < n)
          for (int a = 0; a < 3; a++) s_w[a][k] += add[a][r];
      }
    }
    __syncthreads();
    const double4_32a pp = B.pos[g.b0 + pv];
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
      const int i = k < nf ? pv + 1 + k : pv - 1 - (k - nf);
      const double q = B.pos[g.b0 + i].w;
      put_trial(P, B, g.b_lo, g.b0 + i,
                make_double4_32a(pp.x + s_w[0][k], pp.y + s_w[1][k], pp.z + s_w[2][k], q));
    }
    // the pivot bead stays where it is (its trial entry equals its position)
    if (P.form && threadIdx.x == 0)
      B.ftrial[g.b0 + pv - g.b_lo] = fix_point(P, B.trial[g.b0 + pv], B.type[g.b0 + pv]);
  } else if (g.type == 4) {
    const int len = g.b1 - g.b0;
    for (int i = threadIdx.x; i < len; i += blockDim.x) {
      double4_32a nw;
      if (i == g.end) {
        double4_32a o = B.pos[g.b0 + i];
        nw = make_double4_32a(o.x + g.vec[0], o.y + g.vec[1], o.z + g.vec[2], o.w);
      } else {
        double4_32a o = B.pos[g.b0 + i + g.dir];
        nw = make_double4_32a(o.x, o.y, o.z, B.pos[g.b0 + i].w);
      }
      put_trial(P, B, g.b_lo, g.b0 + i, nw);
    }
  }
  if (P.form && g.type == 2 && g.pivot < 0) {
    // fixed-point trial coordinates of the sequential pivot
    __syncthreads();
    for (int i = g.b_lo + threadIdx.x; i < g.b_hi; i += blockDim.x)
      B.ftrial[i - g.b_lo] = fix_point(P, B.trial[i], B.type[i]);
  }
  // surrogate move: its descriptor is accumulated from zero by the next launch
  const bool surr = g.type >= 2 && B.desc_acc && B.desc_fine && (st->da_on || B.log_desc);
  if (surr)
    for (int k = threadIdx.x; k < mlp::kFineAll; k += blockDim.x) B.desc_fine[k] = 0u;
  if (threadIdx.x == 0) {
    st->da_active = surr ? 1 : 0;
    st->da_skip = 0;
    if (g.type >= 0) {
      st->pending = 1;
      st->mol = g.mol;
      st->b_lo = g.b_lo;
      st->b_hi = g.b_hi;
      st->move_type = g.type;
    } else {
      st->pending = 0;
    }
  }
}

// Shared memory of one serial step.
struct SerialSmem {
  uint32_t win[kDrawWindow];
  unsigned accbits[kDrawWindow / 32];  // randSphere acceptance per position
  double red[3 * (kSerialThreads / 32)];
  GenPlan plan;
  int s_accept, s_ext_bad;
  int s_off[kPivotMax], s_boff[kPivotMax];  // draw offsets per bead
  union {
    short jump[kJumpLevels][kDrawWindow + 1];  // pivot draws: 2^l beads on
    double s_w[3][kPivotMax];                  // pivot bond steps (used after)
  };
  // The state lives in shared memory for the step: thread 0's chain of
  // decisions then never waits on global memory for it.
  DevState S;
};

// Batched replicas: the pending move's sums are per-item slots of the batch
// delta kernel, added here in item order.
struct SlotSums {
  const double* slots;  // [items][2]
  int pair_off, n_pair, k_off, n_k;
};

__device__ __forceinline__ void serial_body(const DevParams& P, const DevBuffers& B, int mode,
                                            SerialSmem& sm, const SlotSums* slots) {
  uint32_t* const win = sm.win;
  unsigned* const accbits = sm.accbits;
  double* const red = sm.red;
  GenPlan& plan = sm.plan;
  int& s_accept = sm.s_accept;
  int& s_ext_bad = sm.s_ext_bad;
  int* const s_off = sm.s_off;
  int* const s_boff = sm.s_boff;
  double(*const s_w)[kPivotMax] = sm.s_w;
  short(*const jump)[kDrawWindow + 1] = sm.jump;
  DevState& S = sm.S;
  {
    const int nw = (int)(sizeof(DevState) / sizeof(int));
    const int* src = reinterpret_cast<const int*>(B.state);
    int* dst = reinterpret_cast<int*>(&S);
    for (int i = threadIdx.x; i < nw; i += blockDim.x) dst[i] = src[i];
  }
  __syncthreads();
  if (S.error) return;
  if (slots && (mode & kModeFinish) && S.pending) {
    double a = 0.0, b = 0.0, c = 0.0;
    for (int i = threadIdx.x; i < slots->n_pair; i += blockDim.x) {
      a += slots->slots[2 * (slots->pair_off + i)];
      b += slots->slots[2 * (slots->pair_off + i) + 1];
    }
    for (int i = threadIdx.x; i < slots->n_k; i += blockDim.x)
      c += slots->slots[2 * (slots->k_off + i)];
    bsum3<kSerialThreads>(a, b, c, red);
    if (threadIdx.x == 0) {
      S.red_lj = a;
      S.red_re = b;
      S.red_k = c;
    }
    __syncthreads();
  }

  // Stage the next stream words.
  const long long wbase = S.stream_pos;
  int wlen = 0;
  if (mode & (kModeDecide | kModeGen)) {
    long long avail = S.stream_len - wbase;
    wlen = (int)(avail < kDrawWindow ? (avail > 0 ? avail : 0) : kDrawWindow);
    for (int i = threadIdx.x; i < wlen; i += blockDim.x) win[i] = B.stream[wbase + i];
  }
  __syncthreads();
  if (mode & kModeGen) {
    // every window position's randSphere test, one position per thread; a
    // warp's ballot makes the word of its 32 positions
    for (int p0 = threadIdx.x & ~31; p0 < kDrawWindow; p0 += blockDim.x) {
      const int p = p0 + (threadIdx.x & 31);
      const bool ok = p + 1 < wlen && !sphere_reject(win[p], win[p + 1]);
      const unsigned bits = __ballot_sync(0xFFFFFFFFu, ok);
      if ((threadIdx.x & 31) == 0) accbits[p0 >> 5] = bits;
    }
    __syncthreads();
  }
  Draws d{B.stream, win, wbase, S.stream_len, wbase, wlen, 0};

  const int pending = S.pending;
  const int b_lo = S.b_lo, b_hi = S.b_hi, mol = S.mol;

  if ((mode & kModeFinish) && pending && S.da_skip) {
    // Stage one rejected the move: no exact change was computed, and no
    // delta kernel applied the S(k) change of the last accepted move.
    if (P.use_ewald && S.sk_pending) {
      const double2* add = B.dsk + (size_t)S.sk_buf * P.n_k;
      for (int k = threadIdx.x; k < P.n_k; k += blockDim.x) {
        const double2 a = add[k];
        double2 v = B.sk[k];
        v.x += a.x;
        v.y += a.y;
        B.sk[k] = v;
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      S.sk_pending = 0;
      S.de = 0.0;
    }
    __syncthreads();
  } else if ((mode & kModeFinish) && pending) {
    // walls of the moved beads, sum q dz
    if (threadIdx.x == 0) s_ext_bad = 0;
    __syncthreads();
    double ext = 0.0, dmz = 0.0;
    for (int i = b_lo + threadIdx.x; i < b_hi; i += blockDim.x) {
      double4_32a t = B.trial[i], p = B.pos[i];
      if (P.use_ext) {
        int ty = B.type[i];
        double en = wall64(P, t.z, ty);
        if (en >= kVeryLarge) s_ext_bad = 1;
        ext += en - wall64(P, p.z, ty);
      }
      dmz += t.w * (t.z - p.z);
    }
    // bonds of the moved molecule at trial positions
    const int m0 = B.mol_start[mol], m1 = B.mol_start[mol + 1];
    double bt = 0.0;
    if (P.use_bond && m1 - m0 > 1)
      for (int i = m0 + threadIdx.x; i < m1 - 1; i += blockDim.x) {
        double4_32a p = B.trial[i], q = B.trial[i + 1];
        double dx = p.x - q.x, dy = p.y - q.y, dz = p.z - q.z;
        double r = sqrt(dx * dx + dy * dy + dz * dz);
        bt += 0.5 * P.k_bond * (r - P.r0) * (r - P.r0);
      }
    bsum3<kSerialThreads>(ext, dmz, bt, red);
    if (threadIdx.x == 0) {
      // the delta kernel applied any pending S(k) commit if it ran k tiles
      if (P.use_ewald && b_hi > b_lo) S.sk_pending = 0;
      const double de_lj = S.red_lj, de_re = S.red_re, de_k = b_hi > b_lo ? S.red_k : 0.0;
      double de = 0.0, dp = 0.0, dx = 0.0, dw = 0.0, db = 0.0;
      double dip_t = S.dipl_cur;
      bool done = false;
      if (P.use_pair) {
        dp = de_lj;
        de += dp;
        done = de >= kVeryLarge;
      }
      if (!done && P.use_ext) {
        dx = s_ext_bad ? kVeryLarge : ext;
        de += dx;
        done = de >= kVeryLarge;
      }
      if (!done && P.use_ewald) {
        dw = de_re + P.kpref * de_k;
        if (P.dipole) {
          dip_t = P.dip_coef * S.mz * S.mz;
          dw += dip_t - S.dipl_cur;
        }
        de += dw;
      }
      if (!done && P.use_bond && m1 - m0 > 1) {
        db = bt - B.bond_mol[mol];
        de += db;
      }
      if (!isfinite(de)) S.n_nonfinite++;  // flagged, rejected as the reference does
      S.de = de;
      S.de_pair = dp;
      S.de_ext = dx;
      S.de_ewald = dw;
      S.de_bond = db;
      S.bond_trial = bt;
      S.dipl_trial = dip_t;
      S.dmz = dmz;
    }
    __syncthreads();
    // training log: (descriptor, exact dE) of a surrogate move
    if (S.da_active && B.log_desc && S.log_n < S.log_cap) {
      const long long row = S.log_n;  // rows of mlp::kIn values
      for (int k = threadIdx.x; k < mlp::kIn; k += blockDim.x)
        B.log_desc[row * mlp::kIn + k] = (float)B.desc_acc[k] * mlp::kDescUnit;
      if (threadIdx.x == 0) {
        B.log_de[row] = S.de;
        S.log_n++;
      }
      __syncthreads();
    }
  }

  // Metropolis (simulation.cc:324-332) or the host's decision.
  if ((mode & (kModeDecide | kModeCommit)) && pending) {
    if (threadIdx.x == 0) {
      int acc = 0;
      if (mode & kModeDecide) {
        if (S.da_active && S.da_on) {
          // Delayed acceptance, stage two: with the stage-one probability
          // min(1, exp(-beta s)) and s antisymmetric under reversing the
          // move, min(1, exp(-beta (dE - s))) gives the same ratio
          // exp(-beta dE) of forward to reverse acceptance as Metropolis.
          if (!S.da_skip && !(S.de >= kVeryLarge))
            acc = metropolis(d.u(), P.beta * (S.de - S.da_s));
          S.da_n_moves++;
          S.da_n_pass += S.da_skip ? 0 : 1;
          S.da_n_accept += acc;
        } else if (!(S.de >= kVeryLarge)) {
          acc = metropolis(d.u(), P.beta * S.de);  // a NaN dE still draws
        }
        if (d.overrun) S.error = PLUM_ERR_STREAM_DEV;
      } else {
        acc = S.last_accept;
      }
      s_accept = acc;
    }
    __syncthreads();
    const int acc = s_accept;
    if (acc) {
      for (int i = b_lo + threadIdx.x; i < b_hi; i += blockDim.x) {
        const int4 old_f = P.form ? B.fpos[i] : make_int4(0, 0, 0, 0);
        B.pos[i] = B.trial[i];
        if (B.fpos64) B.fpos64[i] = fix64x4(P, B.trial[i]);
        if (P.form) B.fpos[i] = B.ftrial[i - b_lo];
        if (P.cell_cap && B.cell_key) {
          // the bead's entry follows it: rewritten in place while it stays in
          // its cell (or already is in the extra list), else marked dead and
          // the bead appended to the extra list
          const int4 f = B.ftrial[i - b_lo];
          const int4 ent = make_int4(f.x, f.y, f.z, (i << 3) | f.w);
          const int key = B.cell_key[i];
          if (key >= 0 && cell_index(P, old_f) == cell_index(P, f)) {
            B.cell_ent[key] = ent;
          } else if (key <= -2) {
            B.cell_extra[-2 - key] = ent;
          } else {
            if (key >= 0) B.cell_ent[key] = make_int4(0, 0, 0, -1);
            const int nc = P.cell_nc[0] * P.cell_nc[1] * P.cell_nc[2];
            const int e = atomicAdd(&B.cell_n[nc], 1);
            if (e < P.cell_cap) {
              B.cell_extra[e] = ent;
              B.cell_key[i] = -2 - e;
            } else {
              B.cell_key[i] = -1;
              S.cell_ok = 0;  // every writer stores the same value
            }
          }
        }
      }
    } else {
      for (int i = b_lo + threadIdx.x; i < b_hi; i += blockDim.x) B.trial[i] = B.pos[i];
    }
    if (threadIdx.x == 0) {
      if (acc) {
        S.e_pair += S.de_pair;
        S.e_ext += S.de_ext;
        S.e_ewald += S.de_ewald;
        S.e_bond += S.de_bond;
        S.mz += S.dmz;
        if (P.dipole) S.dipl_cur = S.dipl_trial;
        if (P.use_bond && B.mol_start[mol + 1] - B.mol_start[mol] > 1)
          B.bond_mol[mol] = S.bond_trial;
        if (P.use_ewald && b_hi > b_lo) {
          // the next delta kernel adds dsk[cur_buf] into S(k)
          S.sk_pending = 1;
          S.sk_buf = S.cur_buf;
          S.cur_buf ^= 1;
        }
        S.n_accept++;
      }
      S.last_accept = acc;
      S.pending = 0;
    }
  }
  // Per-step log (also for steps where nothing was attempted).
  if ((mode & kModeDecide) && S.step_open && threadIdx.x == 0) {
    int sidx = S.step;
    if (B.log_type) B.log_type[sidx] = pending ? S.move_type : -1;
    if (B.log_accept) B.log_accept[sidx] = pending ? S.last_accept : 0;
    if (B.log_etot) B.log_etot[sidx] = S.e_pair + S.e_ewald + S.e_bond + S.e_ext;
    if (B.log_step_de) B.log_step_de[sidx] = pending ? S.de : __longlong_as_double(0x7ff8000000000000LL);
    S.step = sidx + 1;
    S.step_open = 0;
  }
  __syncthreads();

  if ((mode & kModeGen) && !S.error)
    gen_move(P, B, S, d, wbase, plan, s_off, s_boff, s_w, jump, accbits);

  // write the state back
  if (threadIdx.x == 0) S.stream_pos = S.stream_pos > d.pos ? S.stream_pos : d.pos;
  __syncthreads();
  {
    const int nw = (int)(sizeof(DevState) / sizeof(int));
    int* dst = reinterpret_cast<int*>(B.state);
    const int* src = reinterpret_cast<const int*>(&S);
    for (int i = threadIdx.x; i < nw; i += blockDim.x) dst[i] = src[i];
  }
}

__global__ void __launch_bounds__(kSerialThreads)
    k_serial64(const DevParams P, const DevBuffers B, int mode) {
  __shared__ SerialSmem sm;
  serial_body(P, B, mode, sm, nullptr);
}

// One block per replica: the replica's parameters and buffers are staged in
// shared memory, then the same serial step runs on them.
__global__ void __launch_bounds__(kSerialThreads)
    k_batch_serial(const DevParams* __restrict__ rp, const DevBuffers* __restrict__ rb,
                   const int* __restrict__ item_off, const double* __restrict__ slots, int mode) {
  __shared__ SerialSmem sm;
  __shared__ DevParams P;
  __shared__ DevBuffers B;
  const int r = blockIdx.x;
  {
    const int* src = reinterpret_cast<const int*>(rp + r);
    int* dst = reinterpret_cast<int*>(&P);
    for (int i = threadIdx.x; i < (int)(sizeof(DevParams) / sizeof(int)); i += blockDim.x)
      dst[i] = src[i];
    const long long* bs = reinterpret_cast<const long long*>(rb + r);
    long long* bd = reinterpret_cast<long long*>(&B);
    for (int i = threadIdx.x; i < (int)(sizeof(DevBuffers) / sizeof(long long)); i += blockDim.x)
      bd[i] = bs[i];
  }
  __syncthreads();
  SlotSums ss{slots, item_off[4 * r], item_off[4 * r + 1], item_off[4 * r + 2],
              item_off[4 * r + 3]};
  serial_body(P, B, mode, sm, &ss);
}

void launch_batch_serial(const DevParams* rp, const DevBuffers* rb, const int* item_off,
                         const double* slots, int n_rep, int mode, cudaStream_t s) {
  k_batch_serial<<<n_rep, kSerialThreads, 0, s>>>(rp, rb, item_off, slots, mode);
}

void launch_serial64(const DevParams& P, const DevBuffers& B, int mode, cudaStream_t s) {
  k_serial64<<<1, kSerialThreads, 0, s>>>(P, B, mode);
}

__global__ void k_set_move(DevState* st, int mol, int b_lo, int b_hi) {
  st->pending = 1;
  st->mol = mol;
  st->b_lo = b_lo;
  st->b_hi = b_hi;
  st->move_type = -1;
}

void launch_set_move(const DevBuffers& B, int mol, int b_lo, int b_hi, cudaStream_t s) {
  k_set_move<<<1, 1, 0, s>>>(B.state, mol, b_lo, b_hi);
}

// ------------------------------------------------------------ mt19937 fill
// One block regenerates the 624-word state in the three data-independent
// phases of the MT19937 recurrence (i < 227 reads only old words; i < 454
// reads new words of phase one; the rest reads phase-two words), then
// tempers. state[624] holds the output index as in std::mt19937.
__device__ __forceinline__ uint32_t mt_twist(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t y = (a & 0x80000000u) | (b & 0x7fffffffu);
  uint32_t v = c ^ (y >> 1);
  if (y & 1u) v ^= 0x9908b0dfu;
  return v;
}

__device__ __forceinline__ void mt_fill_body(uint32_t* state, uint32_t* out, long long n) {
  __shared__ uint32_t mt[624], old[624];
  for (int i = threadIdx.x; i < 624; i += blockDim.x) mt[i] = state[i];
  __shared__ int idx;
  if (threadIdx.x == 0) idx = (int)state[624];
  __syncthreads();
  long long w = 0;
  while (w < n) {
    if (idx >= 624) {
      for (int i = threadIdx.x; i < 624; i += blockDim.x) old[i] = mt[i];
      __syncthreads();
      for (int i = threadIdx.x; i < 227; i += blockDim.x)
        mt[i] = mt_twist(old[i], old[i + 1], old[i + 397]);
      __syncthreads();
      for (int i = 227 + threadIdx.x; i < 454; i += blockDim.x)
        mt[i] = mt_twist(old[i], old[i + 1], mt[i - 227]);
      __syncthreads();
      for (int i = 454 + threadIdx.x; i < 623; i += blockDim.x)
        mt[i] = mt_twist(old[i], old[i + 1], mt[i - 227]);
      __syncthreads();
      if (threadIdx.x == 0) {
        mt[623] = mt_twist(old[623], mt[0], mt[396]);
        idx = 0;
      }
      __syncthreads();
    }
    long long take = 624 - idx;
    if (take > n - w) take = n - w;
    for (int i = threadIdx.x; i < take; i += blockDim.x) {
      uint32_t y = mt[idx + i];
      y ^= y >> 11;
      y ^= (y << 7) & 0x9d2c5680u;
      y ^= (y << 15) & 0xefc60000u;
      y ^= y >> 18;
      out[w + i] = y;
    }
    __syncthreads();
    if (threadIdx.x == 0) idx += (int)take;
    w += take;
    __syncthreads();
  }
  for (int i = threadIdx.x; i < 624; i += blockDim.x) state[i] = mt[i];
  if (threadIdx.x == 0) state[624] = (uint32_t)idx;
}

__global__ void __launch_bounds__(1024) k_mt_fill(uint32_t* state, uint32_t* out,
                                                  long long n) {
  mt_fill_body(state, out, n);
}

__global__ void __launch_bounds__(1024)
    k_mt_fill_batch(uint32_t* const* states, uint32_t* const* outs, const long long* pos,
                    const long long* len, const long long* cap, const int* need,
                    DevState* const* sts) {
  const int r = blockIdx.x;
  if (!need[r]) return;
  uint32_t* out = outs[r];
  const long long p = pos[r], l = len[r];
  const long long tail = l > p ? l - p : 0;
  // move the unread words to the front (forward copy; source is ahead)
  for (long long i0 = 0; i0 < tail; i0 += blockDim.x) {
    long long i = i0 + threadIdx.x;
    uint32_t v = i < tail ? out[p + i] : 0u;
    __syncthreads();
    if (i < tail) out[i] = v;
    __syncthreads();
  }
  mt_fill_body(states[r], out + tail, cap[r] - tail);
  if (threadIdx.x == 0) {
    sts[r]->stream_pos = 0;
    sts[r]->stream_len = cap[r];
  }
}

// Compact copy of every replica's stream cursor, counters and error flag:
// out[r] = {stream_pos, stream_len, error, n_accept, n_nonfinite, 0}.
__global__ void k_gather_states(DevState* const* sts, int n_rep, long long* out) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n_rep; r += gridDim.x * blockDim.x) {
    const DevState* st = sts[r];
    out[6 * r] = st->stream_pos;
    out[6 * r + 1] = st->stream_len;
    out[6 * r + 2] = st->error;
    out[6 * r + 3] = st->n_accept;
    out[6 * r + 4] = st->n_nonfinite;
    out[6 * r + 5] = st->cell_ok;
  }
}

void launch_gather_states(DevState* const* sts, int n_rep, long long* out, cudaStream_t s) {
  k_gather_states<<<(n_rep + 255) / 256, 256, 0, s>>>(sts, n_rep, out);
}

// Running totals {pair, ewald, bond, ext} of every replica into out[4 r + q].
__global__ void k_gather_energies(DevState* const* sts, int n_rep, double* out) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n_rep; r += gridDim.x * blockDim.x) {
    const DevState* st = sts[r];
    out[4 * r] = st->e_pair;
    out[4 * r + 1] = st->e_ewald;
    out[4 * r + 2] = st->e_bond;
    out[4 * r + 3] = st->e_ext;
  }
}

void launch_gather_energies(DevState* const* sts, int n_rep, double* out, cudaStream_t s) {
  k_gather_energies<<<(n_rep + 255) / 256, 256, 0, s>>>(sts, n_rep, out);
}

void launch_mt_fill_batch(uint32_t* const* states, uint32_t* const* outs, const long long* pos,
                          const long long* len, const long long* cap, const int* need,
                          DevState* const* sts, int n_rep, cudaStream_t s) {
  k_mt_fill_batch<<<n_rep, 1024, 0, s>>>(states, outs, pos, len, cap, need, sts);
}

void launch_mt_fill(uint32_t* state, uint32_t* out, long long n, cudaStream_t s) {
  if (n > 0) k_mt_fill<<<1, 1024, 0, s>>>(state, out, n);
}

}  // namespace plum
