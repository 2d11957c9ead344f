// Wall-force pressure of slit systems (ForceField::CalcPressureForceLJELSlit,
// pressure.cc:404-488) on the device: the per-item arithmetic of
// slit_pressure.h in three launches.
//
//  k_slit_pairs  (site, bead) pair items -- LJ and real-space Ewald z forces --
//                then the wall items (the external force of every system
//                bead), dealt grid-stride; each block writes six partial sums
//  k_slit_recip  one thread per half-space k vector: the five group structure
//                factors over all beads (staged through shared memory in tiles
//                of 256) and the k vector's reciprocal z forces; each block
//                writes three partial sums
//  k_slit_sum    one block adds the partials in a fixed order: the result is
//                run-to-run identical
//
// Cost: pairs are sites x (beads of the second wall and the system), each
// with the real-space image loop; the k part is n_k x n_bead sincos, in place
// of the reference's sites x beads x n_k.
#include "engine.h"
#include "slit_pressure.h"

namespace plum {

namespace {

constexpr int kSlitThreads = 256;

template <int NQ>
__device__ __forceinline__ void block_sums(double* v, double* out) {
  __shared__ double red[NQ][kSlitThreads / 32];
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
#pragma unroll
  for (int q = 0; q < NQ; q++) {
    double x = v[q];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if (l == 0) red[q][w] = x;
  }
  __syncthreads();
  if (threadIdx.x < NQ) {
    double t = 0.0;
    for (int i = 0; i < kSlitThreads / 32; i++) t += red[threadIdx.x][i];
    out[threadIdx.x] = t;
  }
}

__global__ void __launch_bounds__(kSlitThreads)
    k_slit_pairs(const SlitPressParams S, const double* xyzq, const int* type,
                 const int* mol_start, long long n_pair, long long n_wall, int wall_b0,
                 double* part) {
  double acc[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  const long long n = n_pair + n_wall;
  const long long stride = (long long)gridDim.x * kSlitThreads;
  for (long long it = (long long)blockIdx.x * kSlitThreads + threadIdx.x; it < n; it += stride) {
    if (it < n_pair)
      slit_pair_item(S, xyzq, type, mol_start, it, acc);
    else
      slit_wall_item(S, xyzq, type, mol_start, wall_b0 + (int)(it - n_pair), acc);
  }
  block_sums<6>(acc, part + 6 * (size_t)blockIdx.x);
}

__global__ void __launch_bounds__(kSlitThreads)
    k_slit_recip(const SlitPressParams S, const double* xyzq, const int* mol_start,
                 const short4* kn, const double* kw, int n_k, double3 kunit, double* part) {
  __shared__ double4_32a s_p[kSlitThreads];
  __shared__ int s_g[kSlitThreads];
  const int k = blockIdx.x * kSlitThreads + threadIdx.x;
  const bool on = k < n_k;
  double kx = 0.0, ky = 0.0, kz = 0.0, w = 0.0;
  if (on) {
    const short4 v = kn[k];
    kx = v.x * kunit.x;
    ky = v.y * kunit.y;
    kz = v.z * kunit.z;
    w = kw[k];
  }
  double re[5] = {0.0, 0.0, 0.0, 0.0, 0.0}, im[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  for (int t0 = 0; t0 < S.n_bead; t0 += kSlitThreads) {
    const int b = t0 + threadIdx.x;
    __syncthreads();  // the previous tile is consumed
    if (b < S.n_bead) {
      const double* p = xyzq + 4 * (size_t)b;
      double x = p[0], y = p[1], z = p[2];
      // the periodic axes into the primary cell (e^{i k.r} is periodic there)
      if (S.npbc > 0) x -= S.ebox[0] * floor(x / S.ebox[0]);
      if (S.npbc > 1) y -= S.ebox[1] * floor(y / S.ebox[1]);
      if (S.npbc > 2) z -= S.ebox[2] * floor(z / S.ebox[2]);
      s_p[threadIdx.x] = make_double4_32a(x, y, z, p[3]);
      s_g[threadIdx.x] = p[3] != 0.0 ? slit_bead_groups(S, mol_start, b) : 0;
    } else {
      s_g[threadIdx.x] = 0;
    }
    __syncthreads();
    const int nt = min(kSlitThreads, S.n_bead - t0);
    if (on)
      for (int u = 0; u < nt; u++) {
        const int g = s_g[u];  // the same for every thread: no divergence
        if (!g) continue;
        const double4_32a p = s_p[u];
        double s, c;
        sincos(kx * p.x + ky * p.y + kz * p.z, &s, &c);
        s *= p.w;
        c *= p.w;
#pragma unroll
        for (int q = 0; q < 5; q++)
          if (g >> q & 1) {
            re[q] += c;
            im[q] += s;
          }
      }
  }
  double o[3] = {0.0, 0.0, 0.0};
  if (on) slit_k_terms(kz, w, re, im, o);
  const double pre = slit_recip_prefactor(S);
  for (int q = 0; q < 3; q++) o[q] *= pre;
  block_sums<3>(o, part + 3 * (size_t)blockIdx.x);
}

// out6 = {LJ ion, LJ polymer, LJ wall-wall, Ewald ion, Ewald polymer, Ewald
// wall-wall}: the increments of p_tensor[6..11] before the reference's
// wall-wall guard.
__global__ void __launch_bounds__(kSlitThreads)
    k_slit_sum(const double* part, int n1, const double* part3, int n2, double* out6) {
  double v[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  for (int i = threadIdx.x; i < n1; i += kSlitThreads)
    for (int q = 0; q < 6; q++) v[q] += part[6 * (size_t)i + q];
  for (int i = threadIdx.x; i < n2; i += kSlitThreads)
    for (int q = 0; q < 3; q++) v[3 + q] += part3[3 * (size_t)i + q];
  block_sums<6>(v, out6);
}

}  // namespace

int slit_partials_count(long long n_items, int n_k, int* n1, int* n2) {
  const long long blocks = (n_items + kSlitThreads - 1) / kSlitThreads;
  *n1 = (int)(blocks < 1 ? 1 : (blocks > 152 * 8 ? 152 * 8 : blocks));
  *n2 = (n_k + kSlitThreads - 1) / kSlitThreads;
  return 6 * *n1 + 3 * *n2 + 6;
}

void launch_slit_pressure(const SlitPressParams& S, const DevBuffers& B, long long n_pair,
                          long long n_wall, int wall_b0, int n_k, const double* kunit,
                          double* scratch, int n1, int n2, cudaStream_t s) {
  const double* xyzq = reinterpret_cast<const double*>(B.pos);
  double* part = scratch;
  double* part3 = scratch + 6 * (size_t)n1;
  double* out6 = part3 + 3 * (size_t)n2;
  k_slit_pairs<<<n1, kSlitThreads, 0, s>>>(S, xyzq, B.type, B.mol_start, n_pair, n_wall,
                                           wall_b0, part);
  if (n2 > 0)
    k_slit_recip<<<n2, kSlitThreads, 0, s>>>(S, xyzq, B.mol_start, B.kn, B.kw, n_k,
                                             make_double3(kunit[0], kunit[1], kunit[2]),
                                             part3);
  k_slit_sum<<<1, kSlitThreads, 0, s>>>(part, n1, part3, n2, out6);
}

}  // namespace plum
