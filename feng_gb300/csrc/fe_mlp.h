// Per-node MLP of the learned Newton initial guess: 16 inputs, two tanh
// hidden layers of 64, 4 outputs (the last is padding), FP32 throughout.
// Forward, back-propagation and Adam are hand-written kernels (fe_mlp.cu);
// there is no counterpart in the reference.
//
// Parameter packing: W1 [64 x 16] row-major, b1 [64], W2 [64 x 64], b2 [64],
// W3 [4 x 64], b3 [4].  Loss of a batch of n samples with a 0/1 mask per
// output: L = sum mask (y - t)^2 / (4 n).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace feng {

struct MLPDims {
  static constexpr int NIN = 16, H = 64, NOUT = 4;
  static constexpr int OW1 = 0, OB1 = OW1 + H * NIN, OW2 = OB1 + H, OB2 = OW2 + H * H, OW3 = OB2 + H,
                       OB3 = OW3 + NOUT * H, P = OB3 + NOUT;
  static constexpr int TILE = 128;  // samples per block
};

class MLPDevice {
 public:
  ~MLPDevice();
  // Glorot-uniform weights from SplitMix64(seed), zero biases, the output
  // layer scaled by outScale (a small start keeps the first corrections near 0).
  int init(uint64_t seed, int64_t maxBatch, cudaStream_t s, float outScale = 0.1f);
  int setParams(const float *hostParams);
  int getParams(float *hostParams) const;
  // Y [n x 4] = MLP(X [n x 16]); device pointers.
  int forward(const float *X, int64_t n, float *Y);
  // Block partial gradients of the loss over a batch: sample i is row idx[i]
  // of X/T/M (idx == nullptr: row i), i < nb.  nb <= maxBatch.
  int gradient(const float *X, const float *T, const float *M, const int32_t *idx, int64_t nb);
  // Sums the partial gradients and applies one Adam step.  gradOut (device,
  // P floats) receives the summed gradient when not null; lossOut (device,
  // one float) the batch loss.
  int adam(float lr, float beta1, float beta2, float eps, float *gradOut, float *lossOut);
  // Random minibatch rows (with replacement) of nRows, from a hash of
  // (seed, draw counter): writes idx [nb] on the device.
  int sample(int64_t nRows, int64_t nb, int32_t *idx);

  int step() const { return step_; }
  float *params() { return params_; }

 private:
  float *params_ = nullptr, *m_ = nullptr, *v_ = nullptr, *partial_ = nullptr, *lossPart_ = nullptr;
  int64_t maxBatch_ = 0;
  int maxBlocks_ = 0, lastBlocks_ = 0;
  int step_ = 0;
  uint64_t seed_ = 0, draws_ = 0;
  cudaStream_t s_ = nullptr;
};

}  // namespace feng
