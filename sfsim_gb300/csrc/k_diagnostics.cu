// k_diagnostics.cu -- SFU throughput probe used for roofline fractions.
#include "atmo_device.cuh"
#include "kernels.h"

namespace sfsim {

// Eight independent chains x <- 2^(-x) per thread keep every value in
// [0.5, 1] and the SFU pipe busy; the FP32 pipe only carries the negation.
__global__ void __launch_bounds__(256) k_sfu_probe(int iters, float* sink) {
  float a[8];
#pragma unroll
  for (int c = 0; c < 8; c++) a[c] = 0.5f + 0.01f * c + 1e-6f * threadIdx.x;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int c = 0; c < 8; c++) a[c] = Bulk<float>::exp2(-a[c]);
  }
  float s = 0;
#pragma unroll
  for (int c = 0; c < 8; c++) s += a[c];
  if (s == 123.0f) sink[blockIdx.x] = s;  // keeps the chains alive
}

void launch_sfu_probe(int blocks, int threads, int iters, float* sink, cudaStream_t st) {
  k_sfu_probe<<<blocks, threads, 0, st>>>(iters, sink);
}

}  // namespace sfsim
