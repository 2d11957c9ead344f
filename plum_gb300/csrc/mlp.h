// Learned surrogate for the energy change of chain moves (pivot, crankshaft,
// reptation) and the delayed-acceptance step built on it. No counterpart in
// the reference: this is an addition that leaves the stationary distribution
// of the reference's Metropolis step unchanged.
//
// Descriptor (96 = 4 channels x 24 radial bins): for a move of beads
// [b_lo, b_hi), the pairs (i moved, j any other bead; moved pairs once) with
// r < 7.5 sigma are counted in fine distance bins f = floor(32 r + 1/2)
// (centred on multiples of 1/32 sigma, so the common bond length 1 sigma is
// mid-bin) per channel
//   0: j of the moved bead's type, before the move   1: other types, before
//   2: j of the moved bead's type, after the move    3: other types, after
// and bin k = 0..23 of a channel is sum_f count_f * round(4096 G(r_f - c_k)),
// G(d) = exp(-d^2 / (2 w^2)), r_f = f / 32, c_k = (k + 1/2) w,
// w = 0.25 sigma (0-6 sigma): a Gaussian-smeared radial histogram in integer
// units of 2^-12. Integer sums make it exact and independent of summation
// order, and the descriptor of the reverse move is exactly the forward one
// with channels (0,1) and (2,3) swapped.
//
// Network: x' = bf16((x - mu) * isd); h1 = bf16(SiLU(W1 x' + b1));
// h2 = SiLU(W2 h1 + b2); f = w3 . h2 + b3 (96 -> 128 -> 128 -> 1, BF16
// weights, FP32 accumulation). The surrogate energy change is antisymmetric
// by construction:  s = y_scale * (f(x) - f(swap(x))).
#pragma once

#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "engine.h"

namespace plum {
namespace mlp {
constexpr int kIn = 96;
constexpr int kBins = 24;
constexpr int kHid = 128;
constexpr int kRows = 128;     // rows of one tile (MMA M)
constexpr int kSamp = 64;      // samples per tile: rows [0,64) as given, [64,128) swapped
constexpr int kThreads = 128;  // one thread per row
constexpr float kBinW = 0.25f;
constexpr float kDescCut = 7.5f;
constexpr float kDescUnit = 1.0f / 4096.0f;  // integer descriptor unit
constexpr int kFinePerSigma = 32;            // fine distance bins per sigma
constexpr int kFine = 241;                   // fine bins per channel (0 - 7.5 sigma)
constexpr int kFineAll = 4 * kFine;
constexpr int kNW1 = kHid * kIn, kNW2 = kHid * kHid;
// fp32 parameter vector: W1 [out][in] | b1 | W2 [out][in] | b2 | w3 | b3
constexpr int kOffW1 = 0, kOffB1 = kNW1, kOffW2 = kOffB1 + kHid, kOffB2 = kOffW2 + kNW2,
              kOffW3 = kOffB2 + kHid, kOffB3 = kOffW3 + kHid, kNParam = kOffB3 + 1;
constexpr int kGradStride = 29184;  // per-tile gradient slot: kNParam values + the loss
static_assert(kGradStride >= kNParam + 1, "gradient slot");
}  // namespace mlp

// The network as the kernels read it (one device copy per surrogate).
struct MlpNet {
  __nv_bfloat16 w1[mlp::kNW1];  // [out][in]
  __nv_bfloat16 w2[mlp::kNW2];  // [out][in]
  __nv_bfloat16 w3[mlp::kHid];
  float b1[mlp::kHid], b2[mlp::kHid];
  float mu[mlp::kIn], isd[mlp::kIn];
  float b3, y_scale;
  // delayed acceptance uses s' = sign(s) max(|s| - da_margin, 0): odd in s,
  // so still antisymmetric; stage one then rejects only moves predicted to
  // cost more than da_margin k_BT
  float da_margin;
};

// Delayed-acceptance hook of the inference kernel: when sts is set, sample r
// is replica r; for a replica whose pending move is a surrogate move
// (DevState::da_active) the kernel stores s and the stage-one outcome.
struct DaArgs {
  DevState* const* sts;
  const DevParams* rp;
};

// y_out[n] = s of each sample (may be null); x: [n][96] floats (scale 1) or
// integer descriptor sums (scale kDescUnit).
void launch_mlp_infer_f(const MlpNet* net, const float* x, int n, float* s_out, int* err,
                        cudaStream_t st);
void launch_mlp_infer_i(const MlpNet* net, const unsigned* x, int n, float* s_out, DaArgs da,
                        int* err, cudaStream_t st);
// One forward + backward pass over n samples with targets t[n]:
// loss = mean (s - t)^2. Writes per-tile gradients into part
// [ceil(n/64)][kGradStride], then reduces them in tile order into grad
// [kNParam + 1] (the last entry is the loss).
void launch_mlp_grad(const MlpNet* net, const float* x, const float* t, int n, float* part,
                     float* grad, int* err, cudaStream_t st);
// Adam step on the fp32 master parameters; refreshes the bf16 copies in net.
void launch_mlp_adam(float* param, float* m, float* v, const float* grad, int step, float lr,
                     MlpNet* net, cudaStream_t st);
// fp32 parameters -> net (bf16 weights, fp32 biases).
void launch_mlp_pack(const float* param, MlpNet* net, cudaStream_t st);

// Descriptor of each replica's pending move into its desc_acc [96] (its
// desc_fine counts must be zero on entry; only replicas with da_active are
// processed). form 1 reads the fixed-point mirrors, form 0 the FP64
// positions. acc is the base of the batch's contiguous desc_acc rows.
// cell_moved > 0 (the longest molecule of replicas that have a cell list)
// first runs the cell-list kernel for the replicas whose list is valid; the
// all-pairs kernel takes the others.
void launch_desc_batch(const DevParams* rp, const DevBuffers* rb, int n_rep, unsigned* acc,
                       int form, int cell_moved, cudaStream_t st);
// Rebuilds the replicas' descriptor cell lists from their fixed-point
// positions (replicas without one are skipped); max_bead = largest n_bead.
// on = 0 marks every list invalid instead (the all-pairs kernel takes all).
void launch_cell_rebuild(const DevParams* rp, const DevBuffers* rb, int n_rep, int max_bead,
                         int on, cudaStream_t st);
// The fine counts only (k_desc).
void launch_desc_counts(const DevParams* rp, const DevBuffers* rb, int n_rep, int form,
                        cudaStream_t st);

}  // namespace plum
