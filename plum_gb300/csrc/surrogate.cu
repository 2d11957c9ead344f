// Host side of the learned surrogate (include/plum_gpu.h, plum_surrogate_*):
// parameters, Adam state and the training loop over device-resident data,
// all arithmetic in the kernels of kern_mlp.cu. No counterpart in the
// reference.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/plum_gpu.h"
#include "mlp.h"
#include "surrogate.h"

using namespace plum;

namespace plum {
int fail_msg(int code, const std::string& msg);  // capi.cu
}

namespace {

#define SCK(x)                                                                  \
  do {                                                                          \
    cudaError_t e_ = (x);                                                       \
    if (e_ != cudaSuccess) return plum::fail_msg(PLUM_ERR_CUDA, cudaGetErrorString(e_)); \
  } while (0)

template <typename T>
int salloc(T** p, size_t n) {
  cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), sizeof(T) * std::max<size_t>(n, 1));
  if (e != cudaSuccess) return plum::fail_msg(PLUM_ERR_CUDA, cudaGetErrorString(e));
  return 0;
}

// splitmix64: portable seeded uniforms for the initial weights
double unif(uint64_t& s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

int ensure_cap(plum_surrogate* g, long n) {
  if (n <= g->cap) return 0;
  cudaFree(g->d_x);
  cudaFree(g->d_t);
  cudaFree(g->d_s);
  cudaFree(g->part);
  g->d_x = g->d_t = g->d_s = g->part = nullptr;
  const long tiles = (n + mlp::kSamp - 1) / mlp::kSamp;
  int rc = salloc(&g->d_x, (size_t)n * mlp::kIn) | salloc(&g->d_t, (size_t)n) |
           salloc(&g->d_s, (size_t)n) | salloc(&g->part, (size_t)tiles * mlp::kGradStride);
  if (rc) return PLUM_ERR_CUDA;
  g->cap = n;
  return 0;
}

int check_err(plum_surrogate* g) {
  int e = 0;
  SCK(cudaMemcpyAsync(&e, g->d_err, sizeof(int), cudaMemcpyDeviceToHost, g->s));
  SCK(cudaStreamSynchronize(g->s));
  if (e) return plum::fail_msg(PLUM_ERR_TIMEOUT, "tensor-core wait timed out in the surrogate");
  return 0;
}

__global__ void k_gather_rows(const float* __restrict__ x, const float* __restrict__ t,
                              const int* __restrict__ idx, int n, float* __restrict__ xo,
                              float* __restrict__ to) {
  const int r = blockIdx.x;
  if (r >= n) return;
  const int src = idx[r];
  for (int k = threadIdx.x; k < mlp::kIn; k += blockDim.x)
    xo[(size_t)r * mlp::kIn + k] = x[(size_t)src * mlp::kIn + k];
  if (threadIdx.x == 0) to[r] = t[src];
}

__global__ void k_add_loss(const float* __restrict__ grad, double* __restrict__ acc) {
  acc[0] += (double)grad[mlp::kNParam];
}

}  // namespace

extern "C" {

int plum_surrogate_nparams(void) { return mlp::kNParam; }

int plum_surrogate_create(int device, unsigned long long seed, plum_surrogate** out) {
  if (!out) return plum::fail_msg(PLUM_ERR_INPUT, "null argument");
  *out = nullptr;
  if (cudaSetDevice(device) != cudaSuccess)
    return plum::fail_msg(PLUM_ERR_CUDA, "cannot select the device");
  plum_surrogate* g = new plum_surrogate();
  g->device = device;
  if (cudaStreamCreateWithFlags(&g->s, cudaStreamNonBlocking) != cudaSuccess) {
    g->s = nullptr;
    plum_surrogate_destroy(g);
    return plum::fail_msg(PLUM_ERR_CUDA, "cannot create the surrogate's stream");
  }
  int rc = salloc(&g->net, 1) | salloc(&g->param, mlp::kNParam) | salloc(&g->m, mlp::kNParam) |
           salloc(&g->v, mlp::kNParam) | salloc(&g->grad, mlp::kNParam + 1) |
           salloc(&g->d_err, 1) | salloc(&g->d_loss, 1);
  if (rc) {
    plum_surrogate_destroy(g);
    return PLUM_ERR_CUDA;
  }
  // Glorot-uniform weights, zero biases
  std::vector<float> p(mlp::kNParam, 0.0f);
  uint64_t st = seed;
  auto fill = [&](int off, int count, int fan_in, int fan_out) {
    const double a = std::sqrt(6.0 / (fan_in + fan_out));
    for (int i = 0; i < count; i++) p[off + i] = (float)((2.0 * unif(st) - 1.0) * a);
  };
  fill(mlp::kOffW1, mlp::kNW1, mlp::kIn, mlp::kHid);
  fill(mlp::kOffW2, mlp::kNW2, mlp::kHid, mlp::kHid);
  fill(mlp::kOffW3, mlp::kHid, mlp::kHid, 1);
  // on the surrogate's own (non-blocking) stream, ordered before the copies below
  cudaMemsetAsync(g->m, 0, sizeof(float) * mlp::kNParam, g->s);
  cudaMemsetAsync(g->v, 0, sizeof(float) * mlp::kNParam, g->s);
  cudaMemsetAsync(g->d_err, 0, sizeof(int), g->s);
  cudaMemsetAsync(g->net, 0, sizeof(MlpNet), g->s);
  std::vector<float> mu(mlp::kIn, 0.0f), isd(mlp::kIn, 1.0f);
  rc = plum_surrogate_set_norm(g, mu.data(), isd.data(), 1.0f);
  if (!rc) rc = plum_surrogate_set_params(g, p.data());
  if (rc) {
    plum_surrogate_destroy(g);
    return rc;
  }
  *out = g;
  return PLUM_OK;
}

int plum_surrogate_destroy(plum_surrogate* g) {
  if (!g) return PLUM_OK;
  cudaSetDevice(g->device);
  if (g->s) cudaStreamSynchronize(g->s);
  void* ptrs[] = {g->net, g->param, g->m,   g->v,    g->grad, g->d_err,
                  g->d_loss, g->d_x, g->d_t, g->d_s, g->part, g->d_idx};
  for (void* q : ptrs)
    if (q) cudaFree(q);
  if (g->s) cudaStreamDestroy(g->s);
  delete g;
  return PLUM_OK;
}

int plum_surrogate_set_params(plum_surrogate* g, const float* params) {
  if (!g || !params) return plum::fail_msg(PLUM_ERR_INPUT, "null argument");
  cudaSetDevice(g->device);
  SCK(cudaMemcpyAsync(g->param, params, sizeof(float) * mlp::kNParam, cudaMemcpyHostToDevice,
                      g->s));
  launch_mlp_pack(g->param, g->net, g->s);
  SCK(cudaGetLastError());
  SCK(cudaStreamSynchronize(g->s));
  return PLUM_OK;
}

int plum_surrogate_get_params(const plum_surrogate* g, float* params) {
  if (!g || !params) return plum::fail_msg(PLUM_ERR_INPUT, "null argument");
  cudaSetDevice(g->device);
  SCK(cudaMemcpyAsync(params, g->param, sizeof(float) * mlp::kNParam, cudaMemcpyDeviceToHost,
                      g->s));
  SCK(cudaStreamSynchronize(g->s));
  return PLUM_OK;
}

int plum_surrogate_set_norm(plum_surrogate* g, const float* mu, const float* isd, float y_scale) {
  if (!g || !mu || !isd || !(y_scale > 0.0f)) return plum::fail_msg(PLUM_ERR_INPUT, "bad argument");
  cudaSetDevice(g->device);
  for (int k = 0; k < mlp::kIn; k++)
    if (!std::isfinite(mu[k]) || !std::isfinite(isd[k]))
      return plum::fail_msg(PLUM_ERR_INPUT, "non-finite normalisation");
  SCK(cudaMemcpyAsync(reinterpret_cast<char*>(g->net) + offsetof(MlpNet, mu), mu,
                      sizeof(float) * mlp::kIn, cudaMemcpyHostToDevice, g->s));
  SCK(cudaMemcpyAsync(reinterpret_cast<char*>(g->net) + offsetof(MlpNet, isd), isd,
                      sizeof(float) * mlp::kIn, cudaMemcpyHostToDevice, g->s));
  SCK(cudaMemcpyAsync(reinterpret_cast<char*>(g->net) + offsetof(MlpNet, y_scale), &y_scale,
                      sizeof(float), cudaMemcpyHostToDevice, g->s));
  SCK(cudaStreamSynchronize(g->s));
  g->y_scale = y_scale;
  return PLUM_OK;
}

int plum_surrogate_set_margin(plum_surrogate* g, float margin) {
  if (!g || !(margin >= 0.0f)) return plum::fail_msg(PLUM_ERR_INPUT, "bad argument");
  cudaSetDevice(g->device);
  SCK(cudaMemcpyAsync(reinterpret_cast<char*>(g->net) + offsetof(MlpNet, da_margin), &margin,
                      sizeof(float), cudaMemcpyHostToDevice, g->s));
  SCK(cudaStreamSynchronize(g->s));
  return PLUM_OK;
}

int plum_surrogate_predict(plum_surrogate* g, const float* x, long n, float* s_out) {
  if (!g || n < 0 || (n > 0 && (!x || !s_out))) return plum::fail_msg(PLUM_ERR_INPUT, "bad argument");
  if (n == 0) return PLUM_OK;
  if (n > (1L << 30) / mlp::kIn) return plum::fail_msg(PLUM_ERR_INPUT, "too many samples");
  cudaSetDevice(g->device);
  if (ensure_cap(g, n)) return PLUM_ERR_CUDA;
  SCK(cudaMemcpyAsync(g->d_x, x, sizeof(float) * mlp::kIn * n, cudaMemcpyHostToDevice, g->s));
  launch_mlp_infer_f(g->net, g->d_x, (int)n, g->d_s, g->d_err, g->s);
  SCK(cudaGetLastError());
  SCK(cudaMemcpyAsync(s_out, g->d_s, sizeof(float) * n, cudaMemcpyDeviceToHost, g->s));
  return check_err(g);
}

int plum_surrogate_predict_device(plum_surrogate* g, const float* d_x, long n, float* d_s) {
  if (!g || n < 0 || (n > 0 && (!d_x || !d_s))) return plum::fail_msg(PLUM_ERR_INPUT, "bad argument");
  if (n == 0) return PLUM_OK;
  if (n > (1L << 30) / mlp::kIn) return plum::fail_msg(PLUM_ERR_INPUT, "too many samples");
  cudaSetDevice(g->device);
  launch_mlp_infer_f(g->net, d_x, (int)n, d_s, g->d_err, g->s);
  SCK(cudaGetLastError());
  return check_err(g);
}

int plum_surrogate_grad(plum_surrogate* g, const float* x, const float* t, long n,
                        float* grad_out) {
  if (!g || n <= 0 || !x || !t || !grad_out) return plum::fail_msg(PLUM_ERR_INPUT, "bad argument");
  if (n > (1L << 30) / mlp::kIn) return plum::fail_msg(PLUM_ERR_INPUT, "too many samples");
  cudaSetDevice(g->device);
  if (ensure_cap(g, n)) return PLUM_ERR_CUDA;
  SCK(cudaMemcpyAsync(g->d_x, x, sizeof(float) * mlp::kIn * n, cudaMemcpyHostToDevice, g->s));
  SCK(cudaMemcpyAsync(g->d_t, t, sizeof(float) * n, cudaMemcpyHostToDevice, g->s));
  launch_mlp_grad(g->net, g->d_x, g->d_t, (int)n, g->part, g->grad, g->d_err, g->s);
  SCK(cudaGetLastError());
  SCK(cudaMemcpyAsync(grad_out, g->grad, sizeof(float) * (mlp::kNParam + 1),
                      cudaMemcpyDeviceToHost, g->s));
  return check_err(g);
}

int plum_surrogate_train(plum_surrogate* g, const float* d_x, const float* d_t, long n, int batch,
                         int epochs, float lr, unsigned long long seed, double* loss_out) {
  if (!g || !d_x || !d_t || n <= 0 || batch <= 0 || epochs < 0 || !(lr > 0.0f))
    return plum::fail_msg(PLUM_ERR_INPUT, "bad argument");
  if (n > (1L << 31) - 1 || batch > (1 << 20)) return plum::fail_msg(PLUM_ERR_INPUT, "too large");
  cudaSetDevice(g->device);
  const long b = std::min<long>(batch, n);
  if (ensure_cap(g, b)) return PLUM_ERR_CUDA;
  if (g->idx_cap < n) {
    cudaFree(g->d_idx);
    g->d_idx = nullptr;
    if (salloc(&g->d_idx, (size_t)n)) return PLUM_ERR_CUDA;
    g->idx_cap = n;
  }
  std::vector<int> idx(n);
  std::iota(idx.begin(), idx.end(), 0);
  uint64_t st = seed;
  const long steps = n / b;
  for (int ep = 0; ep < epochs; ep++) {
    for (long i = n - 1; i > 0; i--) {  // Fisher-Yates
      const long j = (long)(unif(st) * (double)(i + 1));
      std::swap(idx[i], idx[j < i ? j : i]);
    }
    SCK(cudaMemcpyAsync(g->d_idx, idx.data(), sizeof(int) * n, cudaMemcpyHostToDevice, g->s));
    SCK(cudaMemsetAsync(g->d_loss, 0, sizeof(double), g->s));
    for (long k = 0; k < steps; k++) {
      k_gather_rows<<<(unsigned)b, 128, 0, g->s>>>(d_x, d_t, g->d_idx + k * b, (int)b, g->d_x,
                                                   g->d_t);
      launch_mlp_grad(g->net, g->d_x, g->d_t, (int)b, g->part, g->grad, g->d_err, g->s);
      k_add_loss<<<1, 1, 0, g->s>>>(g->grad, g->d_loss);
      launch_mlp_adam(g->param, g->m, g->v, g->grad, ++g->step, lr, g->net, g->s);
    }
    SCK(cudaGetLastError());
    double l = 0.0;
    SCK(cudaMemcpyAsync(&l, g->d_loss, sizeof(double), cudaMemcpyDeviceToHost, g->s));
    int rc = check_err(g);
    if (rc) return rc;
    if (loss_out) loss_out[ep] = steps > 0 ? l / steps : 0.0;
  }
  return PLUM_OK;
}

int plum_surrogate_adam_step(plum_surrogate* g, const float* grad, float lr) {
  if (!g || !grad || !(lr > 0.0f)) return plum::fail_msg(PLUM_ERR_INPUT, "bad argument");
  cudaSetDevice(g->device);
  SCK(cudaMemcpyAsync(g->grad, grad, sizeof(float) * mlp::kNParam, cudaMemcpyHostToDevice, g->s));
  launch_mlp_adam(g->param, g->m, g->v, g->grad, ++g->step, lr, g->net, g->s);
  SCK(cudaGetLastError());
  SCK(cudaStreamSynchronize(g->s));
  return PLUM_OK;
}

}  // extern "C"
