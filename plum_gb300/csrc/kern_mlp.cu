// Surrogate network kernels on the 5th-generation tensor cores (tcgen05):
// BF16 operands staged in shared memory, FP32 accumulators in tensor memory,
// one elected thread issuing the MMAs, an mbarrier signalled by
// tcgen05.commit, and tcgen05.ld for the epilogues. One CTA of 128 threads
// owns a tile of 128 rows (64 samples as given, then the same 64 with the
// before/after channels swapped), so the antisymmetric output
// s = y_scale (f(x) - f(swap x)) and its gradient stay inside the CTA.
//
//   k_mlp_infer   forward on 512 threads (four per tile row, one 32-column
//                 slice each): s per sample; with DaArgs, the
//                 delayed-acceptance stage one of each replica's pending move
//   k_mlp<true>   forward + backward of the mean squared error against the
//                 targets; per-tile gradients of every parameter
//   k_mlp_reduce  per-tile gradients summed in tile order (deterministic)
//   k_mlp_adam    Adam on the fp32 master parameters, bf16 copies refreshed
//   k_desc        descriptor of pending moves (integer Gaussian-bin sums)
//
// Shared-memory operands use the no-swizzle K-major layout: 8x8 core
// matrices of 128 contiguous bytes, core (row/8, k/8) at
// (row/8) * K*16 + (k/8) * 128 bytes, so a descriptor has leading-dimension
// offset 128 B (next core along K) and stride offset K*16 B (next 8 rows),
// and the k-th 16-wide slice starts 256*k bytes further.
//
// Tensor memory (512 columns while training, 256 for inference), lane = row:
//   [0,128) z1 = W1 x'        later dW1 (96 columns)
//   [128,256) z2 = W2 h1
//   [256,384) dh1 = dz2 W2    [384,512) dW2 = dz2^T h1
// Every wait on the mbarrier gives up after one second; the kernel then
// records an error, issues no further MMA and still frees its tensor memory.
#include <cstdio>
#include <type_traits>

#include "device_common.cuh"
#include "mlp.h"

namespace plum {

using namespace mlp;

namespace {

__host__ __device__ constexpr uint32_t op_off(int row, int k, int K) {
  return (uint32_t)((row >> 3) * (K * 16) + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

// tcgen05 instruction descriptor, kind::f16: D f32, A and B bf16, both
// K-major, M x N.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) |
         ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// shared-memory matrix descriptor (no swizzle, K-major, version 1)
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, int K) {
  const uint32_t lbo = 128, sbo = (uint32_t)K * 16;
  uint64_t d = (uint64_t)((addr & 0x3FFFFu) >> 4);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

__device__ __forceinline__ void mma_bf16(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc,
                                         uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d),
      "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

// D[128 x N] (+)= A[128 x K] B[N x K]^T, operands at shared addresses a, b
__device__ __forceinline__ void mma_tile(uint32_t d, uint32_t a, uint32_t b, int K,
                                         uint32_t idesc) {
  for (int k = 0; k < K / 16; k++)
    mma_bf16(d, sdesc(a + 256u * k, K), sdesc(b + 256u * k, K), idesc, k > 0 ? 1u : 0u);
}

__device__ __forceinline__ void mma_commit(uint32_t mbar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
      : "memory");
}

__device__ __forceinline__ void tc_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void proxy_fence() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ uint64_t gtime() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ bool mbar_try(uint32_t mbar, uint32_t phase) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(mbar), "r"(phase)
      : "memory");
  return ok != 0;
}

// bounded wait: false after one second
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t phase) {
  const uint64_t t0 = gtime();
  while (!mbar_try(mbar, phase))
    if (gtime() - t0 > 1000000000ull) return false;
  return true;
}

// 32 consecutive fp32 columns of this thread's lane
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
      "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, "
      "[%32];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),
        "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),
        "=r"(r[31])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ float sigm(float z) { return 1.0f / (1.0f + expf(-z)); }

__device__ __forceinline__ void st_bf16x8(unsigned char* p, const float* v) {
  __align__(16) __nv_bfloat16 h[8];
#pragma unroll
  for (int e = 0; e < 8; e++) h[e] = __float2bfloat16_rn(v[e]);
  *reinterpret_cast<uint4*>(p) = *reinterpret_cast<const uint4*>(h);
}

__device__ __forceinline__ void st_bf16(unsigned char* p, float v) {
  *reinterpret_cast<__nv_bfloat16*>(p) = __float2bfloat16_rn(v);
}

// shared-memory map (bytes)
constexpr uint32_t kW1 = 0;            // B [128][96]
constexpr uint32_t kX = 24576;         // A [128][96]; W1+X later dZ2^T A [128][128]
constexpr uint32_t kW2 = 49152;        // B [128][128]; later dZ1^T A [128][128]
constexpr uint32_t kH1 = 81920;        // A [128][128]; later dZ2 A [128][128]
// training only
constexpr uint32_t kW2T = 114688;      // B [128 a][128 b]
constexpr uint32_t kXT = 147456;       // B [96 c][128 i]
constexpr uint32_t kH1T = 172032;      // B [128 a][128 i]
constexpr uint32_t kRed = 204800;      // f32 [128][33]
constexpr uint32_t kMiscT = 221696;
constexpr uint32_t kMiscI = 114688;
// misc block: y[128], dy[128], tmp[128], db1[128], db2[128], dw3[128] (f32),
// mbarrier, tensor-memory address, flag
constexpr uint32_t kMiscBytes = 6 * 512 + 16;
constexpr uint32_t kSmemTrain = kMiscT + kMiscBytes;
constexpr uint32_t kSmemInfer = kMiscI + kMiscBytes;
static_assert(kSmemTrain <= 232448, "shared memory per CTA");
static_assert(kW1 + 49152 >= 32768 && kX == kW1 + 24576, "dZ2^T fits over W1 and X");

// column sums over the 128 rows of red[row][33] (first 32 columns), in a
// fixed order; result in out[0..31]
__device__ __forceinline__ void col_sum32(const float* red, float* tmp, float* out) {
  const int t = threadIdx.x, c = t & 31, q = t >> 5;
  __syncthreads();
  float s = 0.0f;
  for (int r = q * 32; r < q * 32 + 32; r++) s += red[r * 33 + c];
  tmp[q * 32 + c] = s;
  __syncthreads();
  if (t < 32) out[t] = ((tmp[t] + tmp[32 + t]) + tmp[64 + t]) + tmp[96 + t];
  __syncthreads();
}

template <bool kTrain, typename TIn>
__global__ void __launch_bounds__(kThreads, 1)
    k_mlp(const MlpNet* __restrict__ net, const TIn* __restrict__ x, float xscale, int n,
          const float* __restrict__ tgt, float* __restrict__ s_out, float* __restrict__ part,
          float inv_n, DaArgs da, int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char sm[];
  const int t = threadIdx.x, warp = t >> 5;
  const uint32_t misc = kTrain ? kMiscT : kMiscI;
  float* ys = reinterpret_cast<float*>(sm + misc);
  float* dys = ys + 128;
  float* tmp = ys + 256;
  float* db1s = ys + 384;
  float* db2s = ys + 512;
  float* dw3s = ys + 640;
  uint64_t* mbar = reinterpret_cast<uint64_t*>(sm + misc + 3072);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(sm + misc + 3080);
  int* sflag = reinterpret_cast<int*>(sm + misc + 3084);
  const uint32_t base = smem_u32(sm);
  const uint32_t mb = smem_u32(mbar);
  constexpr uint32_t kCols = kTrain ? 512u : 256u;

  if (warp == 0) {
    asm volatile(
        "tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n\t"
        "tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::"r"(smem_u32(tslot)),
        "r"(kCols)
        : "memory");
  }
  if (t == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mb) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    *sflag = 0;
  }

  // ---- operands: weights and the input tile
  const __nv_bfloat16* w1 = net->w1;
  const __nv_bfloat16* w2 = net->w2;
#pragma unroll 4
  for (int c = t; c < kHid * (kIn / 8); c += kThreads) {
    const int row = c / (kIn / 8), k8 = c % (kIn / 8);
    *reinterpret_cast<uint4*>(sm + kW1 + op_off(row, k8 * 8, kIn)) =
        *reinterpret_cast<const uint4*>(w1 + row * kIn + k8 * 8);
  }
#pragma unroll 4
  for (int c = t; c < kHid * (kHid / 8); c += kThreads) {
    const int row = c / (kHid / 8), k8 = c % (kHid / 8);
    *reinterpret_cast<uint4*>(sm + kW2 + op_off(row, k8 * 8, kHid)) =
        *reinterpret_cast<const uint4*>(w2 + row * kHid + k8 * 8);
  }
  if (kTrain)
    for (int e = t; e < kHid * kHid; e += kThreads) {
      const int a = e % kHid, b = e / kHid;  // W2^T (a, b) = W2[b][a]
      *reinterpret_cast<__nv_bfloat16*>(sm + kW2T + op_off(a, b, kHid)) = w2[b * kHid + a];
    }
  const int sample = blockIdx.x * kSamp + (t & (kSamp - 1));
  const bool swapped = t >= kSamp;
  const bool valid = sample < n;
  // Launched as a dependent of the previous kernel, the weights above were
  // staged while it ran; its results are visible after this wait (a no-op
  // for an ordinary launch).
  asm volatile("griddepcontrol.wait;" ::: "memory");
  {
    // the tile's input rows, staged with coalesced 16-byte loads (rows are
    // 384 bytes, so every row starts 16-byte aligned) into the H1 region
    float* xs = reinterpret_cast<float*>(sm + kH1);
    const int s0 = blockIdx.x * kSamp;
    constexpr int kVec = kSamp * kIn / 4;
#pragma unroll 4
    for (int e = t; e < kVec; e += kThreads) {
      const int row = e / (kIn / 4);
      float4 v = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      if (s0 + row < n) {
        const uint4 raw = reinterpret_cast<const uint4*>(x + (size_t)s0 * kIn)[e];
        if constexpr (std::is_same<TIn, float>::value) {
          v = make_float4(__uint_as_float(raw.x), __uint_as_float(raw.y), __uint_as_float(raw.z),
                          __uint_as_float(raw.w));
        } else {  // integer descriptor sums
          v = make_float4((float)raw.x, (float)raw.y, (float)raw.z, (float)raw.w);
        }
      }
      reinterpret_cast<float4*>(xs)[e] = make_float4(v.x * xscale, v.y * xscale, v.z * xscale,
                                                     v.w * xscale);
    }
  }
  __syncthreads();
  const float* xrow = reinterpret_cast<const float*>(sm + kH1) + (t & (kSamp - 1)) * kIn;
  for (int k8 = 0; k8 < kIn / 8; k8++) {
    float v[8];
#pragma unroll
    for (int e = 0; e < 8; e++) {
      const int f = k8 * 8 + e;
      const int src = swapped ? (f + kIn / 2) % kIn : f;
      v[e] = valid ? (xrow[src] - net->mu[f]) * net->isd[f] : 0.0f;
    }
    st_bf16x8(sm + kX + op_off(t, k8 * 8, kIn), v);
    if (kTrain)
#pragma unroll
      for (int e = 0; e < 8; e++) st_bf16(sm + kXT + op_off(k8 * 8 + e, t, kHid), v[e]);
  }
  proxy_fence();
  tc_before();
  __syncthreads();
  tc_after();
  const uint32_t tmem = *tslot;
  const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
  uint32_t phase = 0;
  bool ok = true;
  auto step = [&](bool issue) {
    // wait for the MMAs committed by thread 0, then agree on the outcome
    bool got = !issue || mbar_wait(mb, phase);
    phase ^= 1u;
    if (!got) atomicOr(sflag, 1);
    tc_before();
    __syncthreads();
    tc_after();
    ok = *sflag == 0;
  };

  // ---- layer 1: z1 = x' W1^T
  if (t == 0) {
    mma_tile(tmem, base + kX, base + kW1, kIn, idesc_bf16(128, 128));
    mma_commit(mb);
  }
  step(true);
  for (int q = 0; q < 4; q++) {
    float v[32];
    tmem_ld32(trow + 32 * q, v);
#pragma unroll
    for (int c = 0; c < 32; c++) {
      const float z = v[c] + net->b1[32 * q + c];
      v[c] = z * sigm(z);
    }
#pragma unroll
    for (int j = 0; j < 4; j++) st_bf16x8(sm + kH1 + op_off(t, 32 * q + 8 * j, kHid), v + 8 * j);
    if (kTrain)
#pragma unroll
      for (int c = 0; c < 32; c++) st_bf16(sm + kH1T + op_off(32 * q + c, t, kHid), v[c]);
  }
  proxy_fence();
  tc_before();
  __syncthreads();
  tc_after();

  // ---- layer 2: z2 = h1 W2^T, then f = w3 . SiLU(z2) + b3
  if (t == 0 && ok) {
    mma_tile(tmem + 128, base + kH1, base + kW2, kHid, idesc_bf16(128, 128));
    mma_commit(mb);
  }
  step(ok);
  float y = net->b3;
  for (int q = 0; q < 4; q++) {
    float v[32];
    tmem_ld32(trow + 128 + 32 * q, v);
#pragma unroll
    for (int c = 0; c < 32; c++) {
      const float z = v[c] + net->b2[32 * q + c];
      y += __bfloat162float(net->w3[32 * q + c]) * (z * sigm(z));
    }
  }
  ys[t] = y;
  __syncthreads();
  float s = 0.0f;
  if (t < kSamp) {
    s = net->y_scale * (ys[t] - ys[t + kSamp]);
    if (valid && s_out) s_out[sample] = s;
    if (!kTrain && valid && da.sts) {
      DevState* st = da.sts[sample];
      if (st->pending && st->da_active) {
        const double u1 = st->da_u1;
        const float m = net->da_margin;
        const float sd = s > m ? s - m : (s < -m ? s + m : 0.0f);
        st->da_s = (double)sd;
        st->da_skip = !(u1 < exp(-da.rp[sample].beta * (double)sd));
      }
    }
  }

  if (kTrain) {
    float* red = reinterpret_cast<float*>(sm + kRed);
    float* gp = part + (size_t)blockIdx.x * kGradStride;
    float lossv = 0.0f;
    if (t < kSamp) {
      float g = 0.0f;
      if (valid) {
        const float d = s - tgt[sample];
        g = 2.0f * d * net->y_scale * inv_n;
        lossv = d * d * inv_n;
      }
      dys[t] = g;
      dys[t + kSamp] = -g;
    }
    __syncthreads();
    const float dyt = dys[t];
    // loss and db3 (zero by construction: the two orientations cancel)
    red[t * 33] = lossv;
    red[t * 33 + 1] = dyt;
    for (int c = 2; c < 32; c++) red[t * 33 + c] = 0.0f;
    col_sum32(red, tmp, db1s);  // db1s is scratch here
    if (t == 0) {
      gp[kNParam] = db1s[0];
      gp[kOffB3] = db1s[1];
    }
    __syncthreads();
    // dz2 = dy w3 SiLU'(z2); dW3 and db2 column sums; dz2 in both layouts
    for (int q = 0; q < 4; q++) {
      float v[32], dz[32];
      tmem_ld32(trow + 128 + 32 * q, v);
#pragma unroll
      for (int c = 0; c < 32; c++) {
        const int b = 32 * q + c;
        const float z = v[c] + net->b2[b];
        const float sg = sigm(z);
        red[t * 33 + c] = dyt * (z * sg);
        dz[c] = dyt * __bfloat162float(net->w3[b]) * sg * (1.0f + z * (1.0f - sg));
      }
      col_sum32(red, tmp, dw3s + 32 * q);
#pragma unroll
      for (int c = 0; c < 32; c++) red[t * 33 + c] = dz[c];
      col_sum32(red, tmp, db2s + 32 * q);
#pragma unroll
      for (int j = 0; j < 4; j++) st_bf16x8(sm + kH1 + op_off(t, 32 * q + 8 * j, kHid), dz + 8 * j);
#pragma unroll
      for (int c = 0; c < 32; c++) st_bf16(sm + kW1 + op_off(32 * q + c, t, kHid), dz[c]);
    }
    proxy_fence();
    tc_before();
    __syncthreads();
    tc_after();
    // dh1 = dz2 W2 (B = W2^T as [a][b]);  dW2 = dz2^T h1 (A = dz2^T, B = h1^T)
    if (t == 0 && ok) {
      mma_tile(tmem + 256, base + kH1, base + kW2T, kHid, idesc_bf16(128, 128));
      mma_tile(tmem + 384, base + kW1, base + kH1T, kHid, idesc_bf16(128, 128));
      mma_commit(mb);
    }
    step(ok);
    for (int q = 0; q < 4; q++) {
      float dh[32], z1[32];
      tmem_ld32(trow + 256 + 32 * q, dh);
      tmem_ld32(trow + 32 * q, z1);
#pragma unroll
      for (int c = 0; c < 32; c++) {
        const float z = z1[c] + net->b1[32 * q + c];
        const float sg = sigm(z);
        dh[c] = dh[c] * sg * (1.0f + z * (1.0f - sg));
        red[t * 33 + c] = dh[c];
      }
      col_sum32(red, tmp, db1s + 32 * q);
#pragma unroll
      for (int c = 0; c < 32; c++) st_bf16(sm + kW2 + op_off(32 * q + c, t, kHid), dh[c]);
    }
    for (int q = 0; q < 4; q++) {
      float v[32];
      tmem_ld32(trow + 384 + 32 * q, v);
#pragma unroll
      for (int c = 0; c < 32; c++) gp[kOffW2 + t * kHid + 32 * q + c] = v[c];
    }
    proxy_fence();
    tc_before();
    __syncthreads();
    tc_after();
    // dW1 = dz1^T x' (A = dz1^T [a][i], B = x'^T [c][i])
    if (t == 0 && ok) {
      mma_tile(tmem, base + kW2, base + kXT, kHid, idesc_bf16(128, 96));
      mma_commit(mb);
    }
    step(ok);
    for (int q = 0; q < 3; q++) {
      float v[32];
      tmem_ld32(trow + 32 * q, v);
#pragma unroll
      for (int c = 0; c < 32; c++) gp[kOffW1 + t * kIn + 32 * q + c] = v[c];
    }
    gp[kOffB1 + t] = db1s[t];
    gp[kOffB2 + t] = db2s[t];
    gp[kOffW3 + t] = dw3s[t];
  }

  tc_before();
  __syncthreads();
  if (t == 0 && !ok && err) atomicExch(err, 1);
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kCols)
                 : "memory");
}

// Inference on 512 threads: thread t takes tile row (TMEM lane) t % 128 and
// the 32-column slice t / 128 of every 128-column epilogue, so each lane
// quarter's rows are shared by four warps (a warp reads only its own lane
// quarter, 32 (warp % 4) .. +31). The per-slice partial outputs are added in
// slice order. Same operands, layout and MMAs as k_mlp; SiLU with the fast
// exponential and divide (relative error ~1e-6, far below the bf16 rounding
// of the operands).
constexpr int kInferThreads = 512;

__device__ __forceinline__ float silu_fast(float z) {
  return __fdividef(z, 1.0f + __expf(-z));  // 0 once exp(-z) passes 2^126
}

template <typename TIn>
__global__ void __launch_bounds__(kInferThreads, 1)
    k_mlp_infer(const MlpNet* __restrict__ net, const TIn* __restrict__ x, float xscale, int n,
                float* __restrict__ s_out, DaArgs da, int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char sm[];
  const int t = threadIdx.x, warp = t >> 5;
  const int row = t & 127, cq = t >> 7;
  float* ypart = reinterpret_cast<float*>(sm + kMiscI);  // [4 slices][128 rows]
  uint64_t* mbar = reinterpret_cast<uint64_t*>(sm + kMiscI + 3072);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(sm + kMiscI + 3080);
  int* sflag = reinterpret_cast<int*>(sm + kMiscI + 3084);
  const uint32_t base = smem_u32(sm);
  const uint32_t mb = smem_u32(mbar);
  constexpr uint32_t kCols = 256u;

  if (warp == 0) {
    asm volatile(
        "tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n\t"
        "tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::"r"(smem_u32(tslot)),
        "r"(kCols)
        : "memory");
  }
  if (t == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mb) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    *sflag = 0;
  }
  const __nv_bfloat16* w1 = net->w1;
  const __nv_bfloat16* w2 = net->w2;
  for (int c = t; c < kHid * (kIn / 8); c += kInferThreads) {
    const int r = c / (kIn / 8), k8 = c % (kIn / 8);
    *reinterpret_cast<uint4*>(sm + kW1 + op_off(r, k8 * 8, kIn)) =
        *reinterpret_cast<const uint4*>(w1 + r * kIn + k8 * 8);
  }
  for (int c = t; c < kHid * (kHid / 8); c += kInferThreads) {
    const int r = c / (kHid / 8), k8 = c % (kHid / 8);
    *reinterpret_cast<uint4*>(sm + kW2 + op_off(r, k8 * 8, kHid)) =
        *reinterpret_cast<const uint4*>(w2 + r * kHid + k8 * 8);
  }
  const int sample = blockIdx.x * kSamp + (row & (kSamp - 1));
  const bool swapped = row >= kSamp;
  const bool valid = sample < n;
  // launched as a dependent of the previous kernel: the weights above were
  // staged while it ran; its results are visible after this wait
  asm volatile("griddepcontrol.wait;" ::: "memory");
  {
    float* xs = reinterpret_cast<float*>(sm + kH1);
    const int s0 = blockIdx.x * kSamp;
    constexpr int kVec = kSamp * kIn / 4;
    for (int e = t; e < kVec; e += kInferThreads) {
      const int r = e / (kIn / 4);
      float4 v = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      if (s0 + r < n) {
        const uint4 raw = reinterpret_cast<const uint4*>(x + (size_t)s0 * kIn)[e];
        if constexpr (std::is_same<TIn, float>::value) {
          v = make_float4(__uint_as_float(raw.x), __uint_as_float(raw.y), __uint_as_float(raw.z),
                          __uint_as_float(raw.w));
        } else {  // integer descriptor sums
          v = make_float4((float)raw.x, (float)raw.y, (float)raw.z, (float)raw.w);
        }
      }
      reinterpret_cast<float4*>(xs)[e] = make_float4(v.x * xscale, v.y * xscale, v.z * xscale,
                                                     v.w * xscale);
    }
  }
  __syncthreads();
  const float* xrow = reinterpret_cast<const float*>(sm + kH1) + (row & (kSamp - 1)) * kIn;
  for (int k8 = cq; k8 < kIn / 8; k8 += 4) {
    float v[8];
#pragma unroll
    for (int e = 0; e < 8; e++) {
      const int f = k8 * 8 + e;
      const int src = swapped ? (f + kIn / 2) % kIn : f;
      v[e] = valid ? (xrow[src] - net->mu[f]) * net->isd[f] : 0.0f;
    }
    st_bf16x8(sm + kX + op_off(row, k8 * 8, kIn), v);
  }
  proxy_fence();
  tc_before();
  __syncthreads();
  tc_after();
  const uint32_t tmem = *tslot;
  const uint32_t trow = tmem + ((uint32_t)((warp & 3) * 32) << 16);
  uint32_t phase = 0;
  bool ok = true;
  auto step = [&](bool issue) {
    bool got = !issue || mbar_wait(mb, phase);
    phase ^= 1u;
    if (!got) atomicOr(sflag, 1);
    tc_before();
    __syncthreads();
    tc_after();
    ok = *sflag == 0;
  };

  // layer 1: z1 = x' W1^T; this thread's 32 columns through SiLU into H1
  if (t == 0) {
    mma_tile(tmem, base + kX, base + kW1, kIn, idesc_bf16(128, 128));
    mma_commit(mb);
  }
  step(true);
  {
    float v[32];
    tmem_ld32(trow + 32 * cq, v);
#pragma unroll
    for (int c = 0; c < 32; c++) v[c] = silu_fast(v[c] + net->b1[32 * cq + c]);
#pragma unroll
    for (int j = 0; j < 4; j++) st_bf16x8(sm + kH1 + op_off(row, 32 * cq + 8 * j, kHid), v + 8 * j);
  }
  proxy_fence();
  tc_before();
  __syncthreads();
  tc_after();

  // layer 2: z2 = h1 W2^T; partial w3 . SiLU(z2) over this thread's columns
  if (t == 0 && ok) {
    mma_tile(tmem + 128, base + kH1, base + kW2, kHid, idesc_bf16(128, 128));
    mma_commit(mb);
  }
  step(ok);
  {
    float v[32];
    tmem_ld32(trow + 128 + 32 * cq, v);
    float y = 0.0f;
#pragma unroll
    for (int c = 0; c < 32; c++)
      y = fmaf(__bfloat162float(net->w3[32 * cq + c]), silu_fast(v[c] + net->b2[32 * cq + c]), y);
    ypart[cq * 128 + row] = y;
  }
  __syncthreads();
  if (t < kSamp) {
    auto yrow = [&](int r) {
      return net->b3 + (((ypart[r] + ypart[128 + r]) + ypart[256 + r]) + ypart[384 + r]);
    };
    const float s = net->y_scale * (yrow(t) - yrow(t + kSamp));
    if (valid && s_out) s_out[sample] = s;
    if (valid && da.sts) {
      DevState* st = da.sts[sample];
      if (st->pending && st->da_active) {
        const double u1 = st->da_u1;
        const float m = net->da_margin;
        const float sd = s > m ? s - m : (s < -m ? s + m : 0.0f);
        st->da_s = (double)sd;
        st->da_skip = !(u1 < exp(-da.rp[sample].beta * (double)sd));
      }
    }
  }
  tc_before();
  __syncthreads();
  if (t == 0 && !ok && err) atomicExch(err, 1);
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kCols)
                 : "memory");
}

__global__ void k_mlp_reduce(const float* __restrict__ part, int tiles, float* __restrict__ grad) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p > kNParam) return;
  float s = 0.0f;
  for (int i = 0; i < tiles; i++) s += part[(size_t)i * kGradStride + p];
  grad[p] = s;
}

__device__ __forceinline__ void put_param(MlpNet* net, int p, float w) {
  if (p < kOffB1) net->w1[p] = __float2bfloat16_rn(w);
  else if (p < kOffW2) net->b1[p - kOffB1] = w;
  else if (p < kOffB2) net->w2[p - kOffW2] = __float2bfloat16_rn(w);
  else if (p < kOffW3) net->b2[p - kOffB2] = w;
  else if (p < kOffB3) net->w3[p - kOffW3] = __float2bfloat16_rn(w);
  else net->b3 = w;
}

__global__ void k_mlp_adam(float* __restrict__ param, float* __restrict__ m, float* __restrict__ v,
                           const float* __restrict__ g, float lr, float c1, float c2,
                           MlpNet* __restrict__ net) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= kNParam) return;
  const float gi = g[p];
  const float mi = 0.9f * m[p] + 0.1f * gi;
  const float vi = 0.999f * v[p] + 0.001f * gi * gi;
  m[p] = mi;
  v[p] = vi;
  const float w = param[p] - lr * (mi * c1) / (sqrtf(vi * c2) + 1e-8f);
  param[p] = w;
  put_param(net, p, w);
}

__global__ void k_mlp_pack(const float* __restrict__ param, MlpNet* __restrict__ net) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < kNParam) put_param(net, p, param[p]);
}

// ------------------------------------------------------------ descriptor
// k_desc counts pairs in fine distance bins. A work item is (replica, 256
// other beads, up to 32 moved beads): one other bead per thread, run against
// the item's moved beads, whose current and trial positions sit in shared
// memory (all of a replica's, loaded once per replica a block visits), in a
// loop with no barrier; items of equal size keep the blocks balanced. A pair within
// the cut adds one to the block's count of its (channel, fine bin) in shared
// memory; the counts go to the replica's desc_fine when the block moves on.
// k_desc_fin smears them into the 96 descriptor bins with integer weights.
// Integer counts and sums make both independent of the order.
constexpr int kDescThreads = 256;
constexpr int kDescMaxMoved = 512;  // longest molecule (the pivot move's limit)
constexpr int kDescSlab = 32;       // moved beads per work item

// FP64 positions: one FP64 subtraction per axis, the periodic wrap in FP32
// (the descriptor only uses pairs within 7.5 sigma, far from the half-box
// distance where the two roundings could pick different images)
__device__ __forceinline__ float wrap32(double d, float L, float invL, bool periodic) {
  const float f = (float)d;
  return periodic ? f - L * rintf(f * invL) : f;
}

// Squared distance of two fixed-point positions (b - a, minimum image by
// integer wraparound) with every rounding pinned (no contraction), so the
// all-pairs and the cell-list kernels give the same bins bit for bit.
__device__ __forceinline__ float desc_r2_fix(const DevParams& P, int4 a, int4 b) {
  const float dx = __fmul_rn((float)(int)((unsigned)b.x - (unsigned)a.x), P.f_scale[0]);
  const float dy = __fmul_rn((float)(int)((unsigned)b.y - (unsigned)a.y), P.f_scale[1]);
  const float dz = __fmul_rn((float)(int)((unsigned)b.z - (unsigned)a.z), P.f_scale[2]);
  return __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
}

// Fine distance bin floor(32 r + 1/2) of a squared distance within the cut.
__device__ __forceinline__ int fine_bin(float r2) {
  return __float2int_rz(__fadd_rn(__fmul_rn(sqrtf(r2), (float)kFinePerSigma), 0.5f));
}

// A bead position as the descriptor kernel keeps it: form 1 the fixed-point
// mirror (x, y, z, type); form 0 FP64 (x, y, z) and the type.
template <int kForm>
struct DPos;
template <>
struct DPos<1> {
  int4 f;
};
template <>
struct DPos<0> {
  double x, y, z;
  int type;
};

template <int kForm>
__device__ __forceinline__ DPos<kForm> load_pos(const DevBuffers& B, int i, int ii, bool trial) {
  DPos<kForm> p;
  if constexpr (kForm == 1) {
    p.f = trial ? B.ftrial[ii] : B.fpos[i];
  } else {
    const double4_32a q = trial ? B.trial[i] : B.pos[i];
    p.x = q.x;
    p.y = q.y;
    p.z = q.z;
    p.type = B.type[i];
  }
  return p;
}

template <int kForm>
__device__ __forceinline__ int ptype(const DPos<kForm>& p) {
  if constexpr (kForm == 1) return p.f.w;
  else return p.type;
}

template <int kForm>
__device__ __forceinline__ float dist2(const DevParams& P, const DPos<kForm>& a,
                                       const DPos<kForm>& b) {
  if constexpr (kForm == 1) {
    return desc_r2_fix(P, a.f, b.f);
  } else {
    const float dx = wrap32(b.x - a.x, (float)P.box[0], (float)P.inv_box[0], P.npbc > 0);
    const float dy = wrap32(b.y - a.y, (float)P.box[1], (float)P.inv_box[1], P.npbc > 1);
    const float dz = wrap32(b.z - a.z, (float)P.box[2], (float)P.inv_box[2], P.npbc > 2);
    return dx * dx + dy * dy + dz * dz;
  }
}

// Per-axis pre-test: a pair can only be within the cut when every axis
// difference is; in fixed point that is one integer subtraction and compare
// per axis (no conversion), and most pairs fail on the first axis. The
// integer bound is one unit above the cut; boxes shorter than twice the cut
// get no bound on that axis.
template <int kForm>
__device__ __forceinline__ bool near_axis(const DPos<kForm>& a, const DPos<kForm>& b, int axis,
                                          const int* icut, const float* fcut,
                                          const DevParams& P) {
  if constexpr (kForm == 1) {
    const unsigned ua = axis == 0 ? a.f.x : (axis == 1 ? a.f.y : a.f.z);
    const unsigned ub = axis == 0 ? b.f.x : (axis == 1 ? b.f.y : b.f.z);
    const int d = (int)(ub - ua);
    return abs(d) <= icut[axis];
  } else {
    const double da = axis == 0 ? b.x - a.x : (axis == 1 ? b.y - a.y : b.z - a.z);
    const float f = wrap32(da, (float)P.box[axis], (float)P.inv_box[axis], P.npbc > axis);
    return fabsf(f) <= fcut[axis];
  }
}

template <int kForm>
__global__ void __launch_bounds__(kDescThreads)
    k_desc(const DevParams* __restrict__ rp, const DevBuffers* __restrict__ rb, int n_rep) {
  // the delayed-acceptance inference may start staging its weights now
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  __shared__ int s_icut[3];
  __shared__ float s_fcut[3];
  __shared__ unsigned fh[kFineAll];
  __shared__ DPos<kForm> mcur[kDescMaxMoved], mtri[kDescMaxMoved];  // the moved beads
  __shared__ int s_pref[kMaxReplicas + 1];
  __shared__ DevParams P;
  __shared__ DevBuffers B;
  __shared__ int s_bl[2];
  for (int r = threadIdx.x; r < n_rep; r += blockDim.x) {
    const DevState* st = rb[r].state;
    const bool cells = rp[r].cell_cap && rb[r].cell_key && st->cell_ok;  // k_desc_cells
    const int m = (st->pending && st->da_active && !cells)
                      ? min(st->b_hi - st->b_lo, kDescMaxMoved) : 0;
    s_pref[r + 1] = ((rp[r].n_bead + kDescThreads - 1) / kDescThreads) *
                    ((m + kDescSlab - 1) / kDescSlab);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    s_pref[0] = 0;
    for (int r = 0; r < n_rep; r++) s_pref[r + 1] += s_pref[r];
  }
  __syncthreads();
  const int T = s_pref[n_rep];
  const int it0 = (int)((long long)T * blockIdx.x / gridDim.x);
  const int it1 = (int)((long long)T * (blockIdx.x + 1) / gridDim.x);
  int cur = -1;
  // the block's counts go to a replica's desc_fine when the block moves on
  // to the next replica and at the end
  auto flush = [&]() {
    for (int k = threadIdx.x; k < kFineAll; k += blockDim.x)
      if (fh[k]) atomicAdd(&B.desc_fine[k], fh[k]);
  };
  for (int item = it0; item < it1; item++) {
    int lo = 0, hi = n_rep - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (s_pref[mid] <= item) lo = mid; else hi = mid - 1;
    }
    const int r = lo;
    if (r != cur) {
      __syncthreads();
      if (cur >= 0) flush();
      __syncthreads();
      const int* src = reinterpret_cast<const int*>(rp + r);
      int* dst = reinterpret_cast<int*>(&P);
      for (int i = threadIdx.x; i < (int)(sizeof(DevParams) / sizeof(int)); i += blockDim.x)
        dst[i] = src[i];
      const long long* bs = reinterpret_cast<const long long*>(rb + r);
      long long* bd = reinterpret_cast<long long*>(&B);
      for (int i = threadIdx.x; i < (int)(sizeof(DevBuffers) / sizeof(long long)); i += blockDim.x)
        bd[i] = bs[i];
      if (threadIdx.x == 0) {
        s_bl[0] = rb[r].state->b_lo;
        s_bl[1] = rb[r].state->b_hi;
      }
      if (threadIdx.x < 3) {
        const int a = threadIdx.x;
        const double unit = rp[r].ebox[a] / 4294967296.0;
        const double lim = kDescCut / unit + 1.0;
        s_icut[a] = lim < 2147483000.0 ? (int)lim : 2147483647;
        s_fcut[a] = kDescCut * 1.0001f;
      }
      for (int k = threadIdx.x; k < kFineAll; k += blockDim.x) fh[k] = 0u;
      __syncthreads();
      const int m = min(s_bl[1] - s_bl[0], kDescMaxMoved);
      for (int q = threadIdx.x; q < m; q += blockDim.x) {
        mcur[q] = load_pos<kForm>(B, s_bl[0] + q, q, false);
        mtri[q] = load_pos<kForm>(B, s_bl[0] + q, q, true);
      }
      __syncthreads();
      cur = r;
    }
    const int b_lo = s_bl[0], m = min(s_bl[1] - b_lo, kDescMaxMoved), N = P.n_bead;
    const int n_chunks = (N + kDescThreads - 1) / kDescThreads;
    const int local = item - s_pref[r];
    const int q0 = (local / n_chunks) * kDescSlab, q1 = min(m, q0 + kDescSlab);
    const int j = (local % n_chunks) * kDescThreads + threadIdx.x;
    if (j < N) {
      const bool jm = j >= b_lo && j < b_lo + m;
      const DPos<kForm> jc = load_pos<kForm>(B, j, 0, false);
      const DPos<kForm> jt = jm ? load_pos<kForm>(B, j, j - b_lo, true) : jc;
      const int tj = ptype<kForm>(jc);
      // moved pairs count once: j moved pairs only with moved i < j
      const int q_end = jm ? min(q1, j - b_lo) : q1;
      for (int q = q0; q < q_end; q++) {
        const DPos<kForm> ic = mcur[q];
        const DPos<kForm> it = mtri[q];
        bool nb = near_axis<kForm>(ic, jc, 0, s_icut, s_fcut, P);
        bool na = near_axis<kForm>(it, jt, 0, s_icut, s_fcut, P);
        if (!(nb || na)) continue;
        nb = nb && near_axis<kForm>(ic, jc, 1, s_icut, s_fcut, P);
        na = na && near_axis<kForm>(it, jt, 1, s_icut, s_fcut, P);
        if (!(nb || na)) continue;
        const int cls = ptype<kForm>(ic) == tj ? 0 : 1;
        if (nb) {
          const float r0 = dist2<kForm>(P, ic, jc);
          if (r0 < kDescCut * kDescCut) atomicAdd(&fh[cls * kFine + fine_bin(r0)], 1u);
        }
        if (na) {
          const float r1 = dist2<kForm>(P, it, jt);
          if (r1 < kDescCut * kDescCut) atomicAdd(&fh[(2 + cls) * kFine + fine_bin(r1)], 1u);
        }
      }
    }
  }
  __syncthreads();
  if (cur >= 0) flush();
}

// ------------------------------------------------- descriptor cell list
// Replicas with a cell list (precision form, periodic on every axis, cells at
// least the cut wide) take the descriptor from k_desc_cells: the pairs
// within the cut of a moved bead lie in the 27 cells around it, about
// 27 x N / cells candidates instead of N. The list is rebuilt at the start of
// every batch of steps by a counting sort (reset, count, scan, scatter) and
// kept up to date by the serial step (kern_moves.cu): beads that leave their
// cell go to a short cell-less list that every descriptor scans in full.
__global__ void k_cell_reset(const DevParams* __restrict__ rp, const DevBuffers* __restrict__ rb) {
  const DevParams& P = rp[blockIdx.x];
  const DevBuffers& B = rb[blockIdx.x];
  if (!P.cell_cap || !B.cell_key) return;
  const int cells = P.cell_nc[0] * P.cell_nc[1] * P.cell_nc[2];
  for (int c = threadIdx.x; c <= cells; c += blockDim.x) B.cell_n[c] = 0;
  if (threadIdx.x == 0) B.state->cell_ok = 1;
}

__global__ void k_cell_count(const DevParams* __restrict__ rp, const DevBuffers* __restrict__ rb) {
  const DevParams& P = rp[blockIdx.y];
  const DevBuffers& B = rb[blockIdx.y];
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (!P.cell_cap || !B.cell_key || j >= P.n_bead) return;
  atomicAdd(&B.cell_n[cell_index(P, B.fpos[j])], 1);
}

// One block per replica: cell_start = exclusive prefix of the counts, and
// the counts become the scatter cursors (cell_n[c] = cell_start[c]).
__global__ void __launch_bounds__(1024)
    k_cell_scan(const DevParams* __restrict__ rp, const DevBuffers* __restrict__ rb) {
  const DevParams& P = rp[blockIdx.x];
  const DevBuffers& B = rb[blockIdx.x];
  if (!P.cell_cap || !B.cell_key) return;
  const int cells = P.cell_nc[0] * P.cell_nc[1] * P.cell_nc[2];
  __shared__ int warp_sum[32];
  __shared__ int carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int base = 0; base < cells; base += blockDim.x) {
    const int c = base + threadIdx.x;
    const int v = c < cells ? B.cell_n[c] : 0;
    int x = v;  // inclusive scan within the warp
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += t;
    }
    if (lane == 31) warp_sum[w] = x;
    __syncthreads();
    if (w == 0) {
      int y = lane < (int)(blockDim.x >> 5) ? warp_sum[lane] : 0;
      for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, y, o);
        if (lane >= o) y += t;
      }
      warp_sum[lane] = y;  // inclusive prefix of the warp totals
    }
    __syncthreads();
    const int ex = carry + (w ? warp_sum[w - 1] : 0) + x - v;
    if (c < cells) {
      B.cell_start[c] = ex;
      B.cell_n[c] = ex;
    }
    __syncthreads();
    if (threadIdx.x == 0) carry += warp_sum[(blockDim.x >> 5) - 1];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    B.cell_start[cells] = carry;
    B.cell_n[cells] = 0;  // extra list empty
  }
}

__global__ void k_cell_scatter(const DevParams* __restrict__ rp,
                               const DevBuffers* __restrict__ rb) {
  const DevParams& P = rp[blockIdx.y];
  const DevBuffers& B = rb[blockIdx.y];
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (!P.cell_cap || !B.cell_key || j >= P.n_bead) return;
  const int4 f = B.fpos[j];
  const int k = atomicAdd(&B.cell_n[cell_index(P, f)], 1);
  B.cell_ent[k] = make_int4(f.x, f.y, f.z, (j << 3) | f.w);
  B.cell_key[j] = k;
}

// moved beads per block: a warp per (bead, before / after); many beads per
// block keep the per-block histogram flush (global atomics) few
constexpr int kCellBeads = 16;
constexpr int kCellSplit = 1;  // warps per (bead, before / after), each a part of its entries
constexpr int kCellWarps = 2 * kCellBeads * kCellSplit;

// Block (x, r): moved beads [4x, 4x + 4) of replica r's pending surrogate
// move. Warp (bead, channel pair): before the move (channels 0, 1) the
// entries of the 27 cells around the bead's current position, after it
// (channels 2, 3) around its trial position, then the cell-less list of
// beads that changed cell, skipping the moved beads (their pairs, each
// once, at the end). Entries carry the positions, so a candidate costs one
// load, and the 27 cells' entries form one list spread over the lanes. The
// same pairs, distances and bins as k_desc.
// A replica without a valid list (none built, or one that overflowed since
// the last rebuild) takes every other bead instead of the cells' entries:
// the same pairs, so the same counts, at all-pairs cost, in this launch.
__global__ void __launch_bounds__(kCellWarps * 32, 1)
    k_desc_cells(const DevParams* __restrict__ rp, const DevBuffers* __restrict__ rb) {
  const DevParams& P = rp[blockIdx.y];
  const DevBuffers& B = rb[blockIdx.y];
  const DevState* st = B.state;
  if (!(st->pending && st->da_active)) return;
  const bool cells = P.cell_cap && B.cell_key && st->cell_ok;
  const int b_lo = st->b_lo, m = min(st->b_hi - b_lo, kDescMaxMoved);
  if ((int)blockIdx.x * kCellBeads >= m) return;
  __shared__ unsigned fh[kFineAll];
  __shared__ int s_pre[kCellWarps][32], s_base[kCellWarps][32];
  for (int k = threadIdx.x; k < kFineAll; k += blockDim.x) fh[k] = 0u;
  __syncthreads();
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int part = w % kCellSplit, pc = w / kCellSplit;
  const int q = blockIdx.x * kCellBeads + (pc >> 1), ch = pc & 1;
  if (q < m) {
    const int tq = B.fpos[b_lo + q].w;
    const int4 p = ch ? B.ftrial[q] : B.fpos[b_lo + q];
    const int nx = P.cell_nc[0], ny = P.cell_nc[1], nz = P.cell_nc[2];
    const float cut2 = kDescCut * kDescCut;
    unsigned* hist = fh + 2 * ch * kFine;
    // lane l < 27: neighbour cell l (offsets -1..1 per axis): its first
    // entry and count
    int cbase = 0, cn = 0;
    if (cells && lane < 27) {
      const int ox = lane % 3 - 1, oy = (lane / 3) % 3 - 1, oz = lane / 9 - 1;
      int x = cell_axis((unsigned)p.x, nx) + ox, y = cell_axis((unsigned)p.y, ny) + oy,
          z = cell_axis((unsigned)p.z, nz) + oz;
      x += x < 0 ? nx : (x >= nx ? -nx : 0);
      y += y < 0 ? ny : (y >= ny ? -ny : 0);
      z += z < 0 ? nz : (z >= nz ? -nz : 0);
      const int c = x + nx * (y + ny * z);
      cbase = B.cell_start[c];
      cn = B.cell_start[c + 1] - cbase;
    }
    auto visit = [&](int4 ent) {
      if (ent.w < 0) return;  // dead: the bead left this cell
      const int j = ent.w >> 3;
      if (j >= b_lo && j < b_lo + m) return;  // moved pairs below
      const float r2 = desc_r2_fix(P, p, ent);
      if (r2 < cut2) atomicAdd(&hist[((ent.w & 7) == tq ? 0 : 1) * kFine + fine_bin(r2)], 1u);
    };
    // the 27 cells' entries as one list, split in kCellSplit contiguous
    // parts (one per warp of this bead and channel): lane e of a part takes
    // its entries e, e + 32, ..., finding the cell by binary search in the
    // inclusive prefix of the counts
    int pre = cn;
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, pre, o);
      if (lane >= o) pre += t;
    }
    const int total = __shfl_sync(0xffffffffu, pre, 26);
    s_pre[w][lane] = pre;
    s_base[w][lane] = cbase;
    __syncwarp();
    if (cells) {
      const int e_lo = part * total / kCellSplit, e_hi = (part + 1) * total / kCellSplit;
#pragma unroll 4
      for (int e = e_lo + lane; e < e_hi; e += 32) {
        int lo = 0, hi = 26;
        while (lo < hi) {
          const int mid = (lo + hi) >> 1;
          if (s_pre[w][mid] > e) hi = mid; else lo = mid + 1;
        }
        visit(B.cell_ent[s_base[w][lo] + e - (lo ? s_pre[w][lo - 1] : 0)]);
      }
      const int n_extra = min(B.cell_n[nx * ny * nz], P.cell_cap);
      for (int e = part * 32 + lane; e < n_extra; e += 32 * kCellSplit) visit(B.cell_extra[e]);
    } else {
#pragma unroll 4
      for (int j = part * 32 + lane; j < P.n_bead; j += 32 * kCellSplit) {
        const int4 f = B.fpos[j];
        visit(make_int4(f.x, f.y, f.z, (j << 3) | f.w));
      }
    }
    for (int q2 = q + 1 + part * 32 + lane; q2 < m; q2 += 32 * kCellSplit) {
      const int4 o = ch ? B.ftrial[q2] : B.fpos[b_lo + q2];
      const float r2 = desc_r2_fix(P, p, o);
      if (r2 < cut2)
        atomicAdd(&hist[(B.fpos[b_lo + q2].w == tq ? 0 : 1) * kFine + fine_bin(r2)], 1u);
    }
  }
  __syncthreads();
  for (int k = threadIdx.x; k < kFineAll; k += blockDim.x)
    if (fh[k]) atomicAdd(&B.desc_fine[k], fh[k]);
}

// One block per replica: bin k of channel c = sum_f count[c][f] *
// round(4096 exp(-(r_f - c_k)^2 / (2 w^2))) over the fine bins within
// 1.2 sigma (where the weight rounds to zero beyond).
__global__ void __launch_bounds__(128) k_desc_fin(const DevBuffers* __restrict__ rb) {
  // launched as a dependent of k_desc: let the inference start staging, then
  // wait for the counts
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  asm volatile("griddepcontrol.wait;" ::: "memory");
  const DevBuffers& B = rb[blockIdx.x];
  const DevState* st = B.state;
  if (!(st->pending && st->da_active)) return;
  const int k = threadIdx.x;
  if (k >= kIn) return;
  const int ch = k / kBins, kb = k % kBins;
  const float c = (kb + 0.5f) * kBinW;
  const int f0 = max(0, (int)((c - 1.2f) * kFinePerSigma));
  const int f1 = min(kFine - 1, (int)((c + 1.2f) * kFinePerSigma) + 1);
  unsigned v = 0u;
  for (int f = f0; f <= f1; f++) {
    const unsigned n = B.desc_fine[ch * kFine + f];
    if (!n) continue;
    const float d = f * (1.0f / kFinePerSigma) - c;
    v += n * __float2uint_rn(4096.0f * expf(-0.5f / (kBinW * kBinW) * d * d));
  }
  B.desc_acc[k] = v;
}

}  // namespace

// ------------------------------------------------------------ launches
static void smem_attr(const void* f, int bytes) {
  cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

void launch_mlp_infer_f(const MlpNet* net, const float* x, int n, float* s_out, int* err,
                        cudaStream_t st) {
  if (n <= 0) return;
  static bool attr = false;
  if (!attr) {
    smem_attr((const void*)k_mlp_infer<float>, kSmemInfer);
    attr = true;
  }
  k_mlp_infer<float><<<(n + kSamp - 1) / kSamp, kInferThreads, kSmemInfer, st>>>(
      net, x, 1.0f, n, s_out, DaArgs{nullptr, nullptr}, err);
}

void launch_mlp_infer_i(const MlpNet* net, const unsigned* x, int n, float* s_out, DaArgs da,
                        int* err, cudaStream_t st) {
  if (n <= 0) return;
  static bool attr = false;
  if (!attr) {
    smem_attr((const void*)k_mlp_infer<unsigned>, kSmemInfer);
    attr = true;
  }
  // programmatic dependent launch: may start while the preceding kernel on
  // the stream (the descriptor kernel) still runs
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((n + kSamp - 1) / kSamp);
  cfg.blockDim = dim3(kInferThreads);
  cfg.dynamicSmemBytes = kSmemInfer;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, k_mlp_infer<unsigned>, net, x, kDescUnit, n, s_out, da, err);
}

void launch_mlp_grad(const MlpNet* net, const float* x, const float* t, int n, float* part,
                     float* grad, int* err, cudaStream_t st) {
  if (n <= 0) return;
  static bool attr = false;
  if (!attr) {
    smem_attr((const void*)k_mlp<true, float>, kSmemTrain);
    attr = true;
  }
  const int tiles = (n + kSamp - 1) / kSamp;
  k_mlp<true, float><<<tiles, kThreads, kSmemTrain, st>>>(net, x, 1.0f, n, t, nullptr, part,
                                                          1.0f / n, DaArgs{nullptr, nullptr}, err);
  k_mlp_reduce<<<(kNParam + 1 + 255) / 256, 256, 0, st>>>(part, tiles, grad);
}

void launch_mlp_adam(float* param, float* m, float* v, const float* grad, int step, float lr,
                     MlpNet* net, cudaStream_t st) {
  const float c1 = 1.0f / (1.0f - powf(0.9f, (float)step));
  const float c2 = 1.0f / (1.0f - powf(0.999f, (float)step));
  k_mlp_adam<<<(kNParam + 255) / 256, 256, 0, st>>>(param, m, v, grad, lr, c1, c2, net);
}

void launch_mlp_pack(const float* param, MlpNet* net, cudaStream_t st) {
  k_mlp_pack<<<(kNParam + 255) / 256, 256, 0, st>>>(param, net);
}

void launch_desc_counts(const DevParams* rp, const DevBuffers* rb, int n_rep, int form,
                        cudaStream_t st) {
  if (form) k_desc<1><<<4 * 152, kDescThreads, 0, st>>>(rp, rb, n_rep);
  else k_desc<0><<<4 * 152, kDescThreads, 0, st>>>(rp, rb, n_rep);
}

__global__ void k_cell_off(const DevBuffers* __restrict__ rb) {
  if (threadIdx.x == 0) rb[blockIdx.x].state->cell_ok = 0;
}

void launch_cell_rebuild(const DevParams* rp, const DevBuffers* rb, int n_rep, int max_bead,
                         int on, cudaStream_t st) {
  if (!on) {
    k_cell_off<<<n_rep, 32, 0, st>>>(rb);
    return;
  }
  k_cell_reset<<<n_rep, 256, 0, st>>>(rp, rb);
  k_cell_count<<<dim3((max_bead + 255) / 256, n_rep), 256, 0, st>>>(rp, rb);
  k_cell_scan<<<n_rep, 1024, 0, st>>>(rp, rb);
  k_cell_scatter<<<dim3((max_bead + 255) / 256, n_rep), 256, 0, st>>>(rp, rb);
}

void launch_desc_batch(const DevParams* rp, const DevBuffers* rb, int n_rep, unsigned* acc,
                       int form, int cell_moved, cudaStream_t st) {
  (void)acc;
  if (cell_moved > 0)
    k_desc_cells<<<dim3((std::min(cell_moved, kDescMaxMoved) + kCellBeads - 1) / kCellBeads,
                        n_rep), kCellWarps * 32, 0, st>>>(rp, rb);
  // with cell lists the cell kernel also takes the replicas whose list is
  // not valid (all pairs); else the all-pairs kernel takes every replica
  if (!(cell_moved > 0 && form)) launch_desc_counts(rp, rb, n_rep, form, st);
  // programmatic dependent of k_desc (it waits for the counts itself)
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(n_rep);
  cfg.blockDim = dim3(128);
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, k_desc_fin, rb);
}

}  // namespace plum
