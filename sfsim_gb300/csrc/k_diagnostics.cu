// k_diagnostics.cu -- SFU and shared-memory throughput probes used for
// roofline fractions.
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

// Shared-memory read bandwidth: every thread reads 16-byte words, a warp 512
// contiguous bytes per request (4 wavefronts, no bank conflict), 8
// independent accumulators per thread.  Bytes read = blocks x threads x
// iters x 8 x 16.
constexpr int kSmemProbeWords = 8192;  // 128 KB of float4
__global__ void __launch_bounds__(1024) k_smem_probe(int iters, float* sink) {
  extern __shared__ float4 words[];
  for (int t = threadIdx.x; t < kSmemProbeWords; t += blockDim.x)
    words[t] = make_float4(1e-7f * t, 0.0f, 0.0f, 0.0f);
  __syncthreads();
  float4 acc[8];
#pragma unroll
  for (int c = 0; c < 8; c++) acc[c] = make_float4(0, 0, 0, 0);
  int base = threadIdx.x;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int c = 0; c < 8; c++) {
      const float4 v = words[(base + c * 1024) & (kSmemProbeWords - 1)];
      acc[c].x += v.x;
      acc[c].y += v.y;
      acc[c].z += v.z;
      acc[c].w += v.w;
    }
    base = (base + 32) & (kSmemProbeWords - 1);
  }
  float s = 0;
#pragma unroll
  for (int c = 0; c < 8; c++) s += acc[c].x + acc[c].y + acc[c].z + acc[c].w;
  if (s == 123.0f) sink[blockIdx.x] = s;  // keeps the loads alive
}

int launch_smem_probe(int blocks, int iters, float* sink, cudaStream_t st) {
  const int smem = kSmemProbeWords * 16;
  if (cudaFuncSetAttribute(k_smem_probe, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess) return -1;
  k_smem_probe<<<blocks, 1024, smem, st>>>(iters, sink);
  return 0;
}

}  // namespace sfsim
