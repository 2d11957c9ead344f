// The surrogate object behind the C ABI's plum_surrogate handle (internal).
#pragma once

#include <cuda_runtime.h>

#include "mlp.h"

struct plum_surrogate {
  int device = 0;
  cudaStream_t s = nullptr;
  plum::MlpNet* net = nullptr;  // bf16 weights, fp32 biases and normalisation
  float* param = nullptr;       // fp32 master parameters [kNParam]
  float* m = nullptr;           // Adam moments
  float* v = nullptr;
  float* grad = nullptr;        // [kNParam + 1]: gradient, then the loss
  int* d_err = nullptr;         // set by a kernel whose tensor-core wait timed out
  double* d_loss = nullptr;     // epoch loss accumulator
  float y_scale = 1.0f;
  int step = 0;                 // Adam steps taken
  // staging of host data and training batches
  float *d_x = nullptr, *d_t = nullptr, *d_s = nullptr, *part = nullptr;
  long cap = 0;
  int* d_idx = nullptr;
  long idx_cap = 0;
};
