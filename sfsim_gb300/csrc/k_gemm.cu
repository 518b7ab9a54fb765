// k_gemm.cu -- BF16 GEMM on the fifth-generation tensor cores (tcgen05) with
// FP32 accumulation in tensor memory, and the epilogues the surrogate MLP
// needs.  C[m][n] = sum_k A[m][k] B[n][k] ("TN": both operands row-major with
// K contiguous).
//
// One CTA of 128 threads computes a 128 x N tile (N <= 256, N % 16 == 0) over
// a K range.  Per K chunk of 64 the threads copy A (128 x 64) and B (N x 64)
// from global memory into shared memory in the canonical no-swizzle K-major
// layout of the tensor cores (8-row x 16-byte core matrices; core matrices
// adjacent in K 128 B apart, adjacent in M/N 1024 B apart), then one thread
// issues four tcgen05.mma (K = 16 each) into the TMEM accumulator and commits
// them to an mbarrier that every thread waits on before the buffers are
// refilled.  The epilogue reads the accumulator with tcgen05.ld (warp w owns
// rows 32w..32w+31).  Every wait is bounded; on timeout the CTA records an
// error, releases its tensor memory and returns.
#include <cuda_bf16.h>
#include <stdint.h>

#include "atmo_device.cuh"
#include "kernels.h"
#include "tc.cuh"

namespace sfsim {



constexpr int kGemmBK = 64;
constexpr int kWaitLimit = 1 << 22;

// Copies rows [0, nrows) x K columns [k0, k0 + 64) of a row-major bf16 matrix
// (leading dimension ld) into a K-major core-matrix tile; rows >= valid read 0.
__device__ __forceinline__ void load_tile(const __nv_bfloat16* src, long long ld, int nrows, int valid, long long k0,
                                          unsigned char* tile) {
  for (int c = threadIdx.x; c < nrows * 8; c += blockDim.x) {
    const int row = c >> 3, kc = c & 7;
    uint4 v = make_uint4(0, 0, 0, 0);
    if (row < valid) v = *reinterpret_cast<const uint4*>(src + (long long)row * ld + k0 + kc * 8);
    *reinterpret_cast<uint4*>(tile + tc::tile_offset(row, kc * 8)) = v;
  }
}

__device__ __forceinline__ float silu(float z) { return z / (1.0f + __expf(-z)); }
__device__ __forceinline__ float dsilu(float z) {
  const float s = 1.0f / (1.0f + __expf(-z));
  return s * (1.0f + z * (1.0f - s));
}

template <int N>
__global__ void __launch_bounds__(128) k_gemm_tn(GemmArgs g) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ uint64_t mbar;
  __shared__ uint32_t tmem_slot;
  unsigned char* tileA = smem;
  unsigned char* tileB = smem + 128 * kGemmBK * 2;
  const int m0 = blockIdx.x * 128;
  const int split = blockIdx.y;
  const long long kper = g.K / gridDim.y;
  const long long kbeg = (long long)split * kper;
  constexpr uint32_t ncols = N <= 32 ? 32 : N <= 64 ? 64 : N <= 128 ? 128 : 256;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (warp == 0) tc::tmem_alloc(&tmem_slot, ncols);
  if (threadIdx.x == 0) tc::mbar_init(&mbar, 1);
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = tmem_slot;
  const uint32_t idesc = tc::idesc_bf16(128, N);
  bool ok = true;
  uint32_t parity = 0;
  const int validA = min(128, g.M - m0);
  for (long long k = 0; k < kper && ok; k += kGemmBK) {
    load_tile(g.A + (long long)m0 * g.lda, g.lda, 128, validA, kbeg + k, tileA);
    load_tile(g.B, g.ldb, N, g.N, kbeg + k, tileB);
    tc::fence_async_smem();
    __syncthreads();
    if (threadIdx.x == 0) {
      tc::fence_after();
      const uint32_t a0 = tc::smem_u32(tileA), b0 = tc::smem_u32(tileB);
#pragma unroll
      for (int ks = 0; ks < kGemmBK / 16; ks++) {
        const uint64_t da = tc::smem_desc(a0 + ks * 256, 128, 1024);
        const uint64_t db = tc::smem_desc(b0 + ks * 256, 128, 1024);
        tc::mma(tmem, da, db, idesc, (k > 0 || ks > 0) ? 1u : 0u);
      }
      tc::commit(&mbar);
    }
    bool done = tc::mbar_wait(&mbar, parity, kWaitLimit);
    if (!done) done = tc::mbar_wait(&mbar, parity, kWaitLimit);  // in-flight MMAs get a second window
    parity ^= 1;
    tc::fence_after();
    ok = __syncthreads_and(done) != 0;  // one decision for the whole CTA
  }

  if (ok) {
    // epilogue: warp w owns accumulator rows 32w..32w+31
    const int m = m0 + warp * 32 + lane;
    const bool row_ok = m < g.M;
    for (int n0 = 0; n0 < N; n0 += 8) {
      float v[8];
      tc::tmem_ld8(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)n0, v);
      if (!row_ok) continue;
#pragma unroll
      for (int i = 0; i < 8; i++) {
        const int n = n0 + i;
        if (n >= g.N) continue;
        float z = v[i] * g.alpha;
        if (g.bias) z += g.bias[n];
        if (g.dact) z *= g.dact[(long long)m * g.N + n];
        if (g.Cf32) g.Cf32[(long long)m * g.ldc + n] = z;
        if (g.Cacc) atomicAdd(g.Cacc + (long long)m * g.ldc + n, z);
        if (g.Dsilu) g.Dsilu[(long long)m * g.N + n] = dsilu(z);
        const float h = g.silu ? silu(z) : z;
        if (g.Hbf16) g.Hbf16[(long long)m * g.ldh + n] = __float2bfloat16(h);
        if (g.HTbf16) g.HTbf16[(long long)n * g.ldht + m] = __float2bfloat16(h);
      }
    }
  } else if (threadIdx.x == 0 && g.error) {
    atomicExch(g.error, 1);
  }
  tc::fence_before();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, ncols);
}

template <int N>
static int launch_n(const GemmArgs& g, int splits, cudaStream_t st) {
  const size_t smem = (size_t)(128 + N) * kGemmBK * 2;
  if (cudaFuncSetAttribute(k_gemm_tn<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return -1;
  dim3 grid((unsigned)((g.M + 127) / 128), splits);
  k_gemm_tn<N><<<grid, 128, smem, st>>>(g);
  return 0;
}

int launch_gemm_tn(const GemmArgs& g, int splits, cudaStream_t st) {
  // the B tile holds N rows rounded up to a multiple of 16
  if (g.K % (kGemmBK * splits) != 0) return -1;
  if (g.N <= 16) return launch_n<16>(g, splits, st);
  if (g.N <= 32) return launch_n<32>(g, splits, st);
  if (g.N <= 64) return launch_n<64>(g, splits, st);
  if (g.N <= 128) return launch_n<128>(g, splits, st);
  if (g.N <= 256) return launch_n<256>(g, splits, st);
  return -1;
}

}  // namespace sfsim
