// k_gemm.cu -- BF16 GEMM on the fifth-generation tensor cores (tcgen05) with
// FP32 accumulation in tensor memory, and the epilogues the surrogate MLP
// needs.  C[m][n] = sum_k A[m][k] B[n][k] ("TN": both operands row-major with
// K contiguous).
//
// A persistent, warp-specialised kernel.  Work items are output tiles of
// 128 x Nt (Nt = N rounded up to 16, at most 256) times split-K slices of the
// K range, dealt round-robin to one CTA per SM.  Warp 0 is the producer: one thread loads K chunks of 64 of A
// (128 x 64) and B (Nt x 64) with TMA tensor copies (128-byte swizzle) into a
// ring of shared-memory stages.  Warp 1 issues the tcgen05.mma (K = 16 each,
// 128-byte-swizzled K-major descriptors) into one of two tensor-memory
// accumulators and releases each stage with tcgen05.commit.  Warps 2-9 are the
// epilogue, two per group of 32 tensor-memory lanes (one per half of the
// columns): they read the finished accumulator (tcgen05.ld, the next 32
// columns in flight while the current ones are written) and apply the
// epilogue while the MMAs of the next tile run into the other accumulator;
// full 32 x 32 blocks pass their row-major input and outputs through a
// per-warp shared-memory tile so that global accesses are row-contiguous.
// Every wait is bounded by a poll limit set at run time
// (sfsim_atmo_set_wait_limit); on timeout the CTA records an error, tells its
// other roles through a shared-memory flag (their waits give up when they see
// it), waits for its copies and MMAs in flight, frees its tensor memory and
// returns.  A self-test mode (stall_polls > 0) makes the epilogue first wait
// on a barrier that nothing arrives on, so that exactly that path runs.
#include <cuda.h>
#include <cuda_bf16.h>
#include <stdint.h>

#include <algorithm>
#include <mutex>

#include "atmo_device.cuh"
#include "kernels.h"
#include "tc.cuh"

namespace sfsim {

constexpr int kGemmBK = 64;                 // K per stage: one 128-byte swizzle atom of bf16
constexpr int kGemmThreads = 320;  // producer, MMA, 8 epilogue warps
constexpr int kGemmEpilogueThreads = 256;
constexpr int kGemmSmemBudget = 192 * 1024;  // stages
constexpr int kGemmTileA = 128 * kGemmBK * 2;

// K-major operand with 128-byte swizzle: rows of 128 B, 16-byte chunks XOR
// (row % 8), 8-row groups 1024 B apart (SBO); the descriptor of the K = 16
// step ks starts 32 * ks bytes into the atom.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)1 << 16;                 // leading byte offset (unused with swizzling)
  d |= (uint64_t)(1024 >> 4) << 32;       // stride byte offset
  d |= (uint64_t)1 << 46;                 // descriptor version
  d |= (uint64_t)2 << 61;                 // layout: 128-byte swizzle
  return d;
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* mbar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
      "[%4];" ::"r"(tc::smem_u32(dst)),
      "l"(map), "r"(x), "r"(y), "r"(tc::smem_u32(mbar))
      : "memory");
}

__device__ __forceinline__ float silu(float z) { return z / (1.0f + __expf(-z)); }
__device__ __forceinline__ float dsilu(float z) {
  const float s = 1.0f / (1.0f + __expf(-z));
  return s * (1.0f + z * (1.0f - s));
}

struct GemmKernelArgs {
  GemmArgs g;
  int nt;          // N rounded up to 16: the MMA's N and the B box height
  int stages;
  int tiles_m, splits;
  long long kper;  // K per split, a multiple of kGemmBK
  int wait_limit;  // polls per mbarrier wait
};

// Per epilogue warp: a 32 x 32 staging tile (row stride 33 words) that turns
// the lane-per-row layout of the tensor-memory loads into row-contiguous
// global accesses.
constexpr int kGemmStageWords = 32 * 33;

// The 32 x 32 block of rows m0 .. m0 + 31 (lane = row), columns n0 .. n0 + 31,
// with every row and column inside the output and 16-byte aligned rows: the
// SiLU' input is read, and the SiLU' and BF16 row-major outputs written, a
// whole row segment at a time through the warp's staging tile.  Returns
// false (nothing done) when the block does not qualify.
template <bool ROWB>
__device__ __forceinline__ bool gemm_epilogue32_staged(const GemmArgs& g, const uint32_t* r, int m0, int n0,
                                                       float* sg) {
  const int lane = threadIdx.x & 31;
  const bool fits = m0 + 32 <= g.M && n0 + 32 <= g.N && (g.N % 4) == 0 && !g.Cacc && !g.Cf32 &&
                    (!g.dact || (reinterpret_cast<uintptr_t>(g.dact) & 15) == 0) &&
                    (!g.Dsilu || (reinterpret_cast<uintptr_t>(g.Dsilu) & 15) == 0) &&
                    (!g.row_bias || (reinterpret_cast<uintptr_t>(g.row_bias) & 15) == 0) &&
                    (!g.Hbf16 || ((g.ldh % 8) == 0 && (reinterpret_cast<uintptr_t>(g.Hbf16) & 15) == 0));
  if (!fits) return false;
  float z[32];
#pragma unroll
  for (int i = 0; i < 32; i++) z[i] = __uint_as_float(r[i]) * g.alpha;
  if (g.bias) {
#pragma unroll
    for (int i = 0; i < 32; i++) z[i] += g.bias[n0 + i];
  }
  if (ROWB) {
    const float4* rb = reinterpret_cast<const float4*>(g.row_bias + (long long)g.row_group[m0 + lane] * g.N + n0);
#pragma unroll
    for (int i = 0; i < 8; i++) {
      const float4 b = rb[i];
      z[4 * i] += b.x, z[4 * i + 1] += b.y, z[4 * i + 2] += b.z, z[4 * i + 3] += b.w;
    }
  }
  // row segments of 32 floats: lane l moves 16 bytes of row 4k + l / 8
  const int rq = lane >> 3, c4 = 4 * (lane & 7);
  if (g.dact) {
#pragma unroll
    for (int k = 0; k < 8; k++) {
      const int row = 4 * k + rq;
      const float4 v = *reinterpret_cast<const float4*>(g.dact + (long long)(m0 + row) * g.N + n0 + c4);
      float* d = sg + row * 33 + c4;
      d[0] = v.x, d[1] = v.y, d[2] = v.z, d[3] = v.w;
    }
    __syncwarp();
#pragma unroll
    for (int i = 0; i < 32; i++) z[i] *= sg[lane * 33 + i];
    __syncwarp();
  }
  // with SiLU' requested, the logistic s of each z serves both SiLU' and
  // SiLU (z s): one exponential and one reciprocal per element
  const bool silu_done = g.Dsilu && g.silu;
  if (g.Dsilu) {
#pragma unroll
    for (int i = 0; i < 32; i++) {
      const float sgm = 1.0f / (1.0f + __expf(-z[i]));
      sg[lane * 33 + i] = sgm * (1.0f + z[i] * (1.0f - sgm));
      if (g.silu) z[i] *= sgm;
    }
    __syncwarp();
#pragma unroll
    for (int k = 0; k < 8; k++) {
      const int row = 4 * k + rq;
      const float* d = sg + row * 33 + c4;
      *reinterpret_cast<float4*>(g.Dsilu + (long long)(m0 + row) * g.N + n0 + c4) = make_float4(d[0], d[1], d[2], d[3]);
    }
    __syncwarp();
  }
  if (g.Hbf16 || g.HTbf16) {
    __nv_bfloat16 h[32];
#pragma unroll
    for (int i = 0; i < 32; i++) h[i] = __float2bfloat16(g.silu && !silu_done ? silu(z[i]) : z[i]);
    if (g.Hbf16) {
      // 16 packed pairs per row; lane l moves 16 bytes of row 8k + l / 4
      uint32_t* s32 = reinterpret_cast<uint32_t*>(sg);
      const uint32_t* hp = reinterpret_cast<const uint32_t*>(h);
#pragma unroll
      for (int i = 0; i < 16; i++) s32[lane * 17 + i] = hp[i];
      __syncwarp();
      const int rr = lane >> 2, q4 = 4 * (lane & 3);
#pragma unroll
      for (int k = 0; k < 4; k++) {
        const int row = 8 * k + rr;
        const uint32_t* d = s32 + row * 17 + q4;
        *reinterpret_cast<uint4*>(g.Hbf16 + (long long)(m0 + row) * g.ldh + n0 + 2 * q4) =
            make_uint4(d[0], d[1], d[2], d[3]);
      }
      __syncwarp();
    }
    if (g.HTbf16) {
      const int m = m0 + lane;
#pragma unroll
      for (int i = 0; i < 32; i++) g.HTbf16[(long long)(n0 + i) * g.ldht + m] = h[i];
    }
  }
  return true;
}

// 32 columns of the epilogue for row m, columns n0 .. n0 + 31.
template <bool ROWB>
__device__ __forceinline__ void gemm_epilogue32(const GemmArgs& g, const uint32_t* r, int m, int n0) {
  const bool row_ok = m < g.M;
  if (!row_ok) return;
#pragma unroll
  for (int i8 = 0; i8 < 4; i8++) {
    const int nb = n0 + 8 * i8;
    if (nb >= g.N) break;
    float z[8];
#pragma unroll
    for (int i = 0; i < 8; i++) z[i] = __uint_as_float(r[8 * i8 + i]) * g.alpha;
    const bool full8 = nb + 8 <= g.N;
    if (g.bias) {
#pragma unroll
      for (int i = 0; i < 8; i++)
        if (nb + i < g.N) z[i] += g.bias[nb + i];
    }
    if (ROWB) {
      const float* rb = g.row_bias + (long long)g.row_group[m] * g.N;
#pragma unroll
      for (int i = 0; i < 8; i++)
        if (nb + i < g.N) z[i] += rb[nb + i];
    }
    if (g.dact) {
      const float* src = g.dact + (long long)m * g.N + nb;
      if (full8 && (g.N % 4 == 0) && (reinterpret_cast<uintptr_t>(g.dact) & 15) == 0) {
        const float4 a = *reinterpret_cast<const float4*>(src), b = *reinterpret_cast<const float4*>(src + 4);
        z[0] *= a.x, z[1] *= a.y, z[2] *= a.z, z[3] *= a.w, z[4] *= b.x, z[5] *= b.y, z[6] *= b.z, z[7] *= b.w;
      } else {
#pragma unroll
        for (int i = 0; i < 8; i++)
          if (nb + i < g.N) z[i] *= src[i];
      }
    }
    if (g.Cacc && full8 && (g.ldc % 4 == 0) && (reinterpret_cast<uintptr_t>(g.Cacc) & 15) == 0) {
      // vector reductions: a quarter of the atomic operations
      float4* dst = reinterpret_cast<float4*>(g.Cacc + (long long)m * g.ldc + nb);
      atomicAdd(dst, make_float4(z[0], z[1], z[2], z[3]));
      atomicAdd(dst + 1, make_float4(z[4], z[5], z[6], z[7]));
    } else if (g.Cacc) {
#pragma unroll
      for (int i = 0; i < 8; i++)
        if (nb + i < g.N) atomicAdd(g.Cacc + (long long)m * g.ldc + nb + i, z[i]);
    }
    if (g.Cf32) {
#pragma unroll
      for (int i = 0; i < 8; i++)
        if (nb + i < g.N) g.Cf32[(long long)m * g.ldc + nb + i] = z[i];
    }
    const bool silu_done = g.Dsilu && g.silu;
    if (g.Dsilu) {
      float* dst = g.Dsilu + (long long)m * g.N + nb;
      float d[8];
#pragma unroll
      for (int i = 0; i < 8; i++) {
        const float sgm = 1.0f / (1.0f + __expf(-z[i]));
        d[i] = sgm * (1.0f + z[i] * (1.0f - sgm));
        if (g.silu) z[i] *= sgm;
      }
      if (full8 && (g.N % 4 == 0) && (reinterpret_cast<uintptr_t>(g.Dsilu) & 15) == 0) {
        *reinterpret_cast<float4*>(dst) = make_float4(d[0], d[1], d[2], d[3]);
        *reinterpret_cast<float4*>(dst + 4) = make_float4(d[4], d[5], d[6], d[7]);
      } else {
#pragma unroll
        for (int i = 0; i < 8; i++)
          if (nb + i < g.N) dst[i] = d[i];
      }
    }
    if (g.Hbf16 || g.HTbf16) {
      __nv_bfloat16 h[8];
#pragma unroll
      for (int i = 0; i < 8; i++) h[i] = __float2bfloat16(g.silu && !silu_done ? silu(z[i]) : z[i]);
      if (g.Hbf16) {
        __nv_bfloat16* dst = g.Hbf16 + (long long)m * g.ldh + nb;
        if (full8 && (g.ldh % 8 == 0) && (reinterpret_cast<uintptr_t>(g.Hbf16) & 15) == 0) {
          *reinterpret_cast<uint4*>(dst) = *reinterpret_cast<const uint4*>(h);
        } else {
#pragma unroll
          for (int i = 0; i < 8; i++)
            if (nb + i < g.N) dst[i] = h[i];
        }
      }
      if (g.HTbf16) {
#pragma unroll
        for (int i = 0; i < 8; i++)
          if (nb + i < g.N) g.HTbf16[(long long)(nb + i) * g.ldht + m] = h[i];
      }
    }
  }
}

// ROWB: the epilogue adds the per-row-group bias (the conditioned surrogate's
// first layer); a separate instantiation keeps the other GEMMs' registers.
template <bool ROWB>
__global__ void __launch_bounds__(kGemmThreads, 1)
    k_gemm_tn(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB, GemmKernelArgs a) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  // 1024-byte alignment for the swizzle atoms
  unsigned char* smem = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const int S = a.stages;
  const int stage_bytes = kGemmTileA + a.nt * kGemmBK * 2;
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + S * stage_bytes);
  uint64_t* empty = full + S;
  uint64_t* tfull = empty + S;   // [2] accumulator ready
  uint64_t* tempty = tfull + 2;  // [2] accumulator drained by the epilogue
  uint64_t* drain = tempty + 2;
  uint64_t* stall = drain + 1;   // self-test: nothing arrives on it
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(stall + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
  float* staging = reinterpret_cast<float*>(smem + S * stage_bytes + 1024);  // [8 epilogue warps][32 * 33]
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t ncols = a.nt <= 32 ? 32 : a.nt <= 64 ? 64 : a.nt <= 128 ? 128 : 256;  // per accumulator
  const long long ntiles = (long long)a.tiles_m * a.splits;
  const long long my_tiles = blockIdx.x < ntiles ? (ntiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
  const int kchunks = (int)(a.kper / kGemmBK);

  if (warp == 0) tc::tmem_alloc(tmem_slot, 2 * ncols);
  if (threadIdx.x == 32) {
    for (int s = 0; s < S; s++) {
      tc::mbar_init(&full[s], 1);
      tc::mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; b++) {
      tc::mbar_init(&tfull[b], 1);
      tc::mbar_init(&tempty[b], kGemmEpilogueThreads);
    }
    tc::mbar_init(drain, 1);
    tc::mbar_init(stall, 1);
    *abort_flag = 0;
    tc::fence_mbar_init();
  }
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      // producer
      long long issued = 0;
      bool ok = true;
      for (long long ti = 0; ti < my_tiles && ok; ti++) {
        const long long tile = blockIdx.x + ti * gridDim.x;
        const int tm = (int)(tile % a.tiles_m), split = (int)(tile / a.tiles_m);
        for (int kc = 0; kc < kchunks; kc++, issued++) {
          const int s = (int)(issued % S);
          if (*abort_flag ||
              (issued >= S &&
               !tc::mbar_wait_or_abort(&empty[s], (uint32_t)(((issued - S) / S) & 1), a.wait_limit, abort_flag))) {
            ok = false;
            break;
          }
          unsigned char* st = smem + s * stage_bytes;
          tc::mbar_expect_tx(&full[s], (uint32_t)stage_bytes);
          const int k = (int)(split * a.kper + (long long)kc * kGemmBK);
          tma_load_2d(st, &mapA, k, tm * 128, &full[s]);
          tma_load_2d(st + kGemmTileA, &mapB, k, 0, &full[s]);
        }
      }
      if (!ok) {
        *abort_flag = 1;
        if (a.g.error) atomicExch(a.g.error, 1);
      }
      // copies in flight land before the CTA leaves: wait for the last S
      // issued (under the full limit, whatever the flag says)
      for (long long k = issued > S ? issued - S : 0; k < issued; k++)
        tc::mbar_wait(&full[k % S], (uint32_t)((k / S) & 1), a.wait_limit);
    }
    __syncwarp();
  } else if (warp == 1) {
    if (lane == 0) {
      // MMA issuer
      const uint32_t idesc = tc::idesc_bf16(128, a.nt);
      const uint32_t base = tc::smem_u32(smem);
      long long c = 0;
      bool ok = true;
      for (long long ti = 0; ti < my_tiles && ok; ti++) {
        const int b = (int)(ti & 1);
        if (ti >= 2 &&
            !(ok = tc::mbar_wait_or_abort(&tempty[b], (uint32_t)(((ti - 2) >> 1) & 1), a.wait_limit, abort_flag) &&
                   !*abort_flag))
          break;
        tc::fence_after();
        const uint32_t d = tmem + (uint32_t)(b * ncols);
        for (int kc = 0; kc < kchunks; kc++, c++) {
          const int s = (int)(c % S);
          if (!(ok = tc::mbar_wait_or_abort(&full[s], (uint32_t)((c / S) & 1), a.wait_limit, abort_flag) &&
                     !*abort_flag))
            break;
          tc::fence_after();
          const uint32_t sa = base + s * stage_bytes, sb = sa + kGemmTileA;
#pragma unroll
          for (int ks = 0; ks < kGemmBK / 16; ks++)
            tc::mma(d, sw128_desc(sa + 32 * ks), sw128_desc(sb + 32 * ks), idesc, (kc > 0 || ks > 0) ? 1u : 0u);
          tc::commit(&empty[s]);
        }
        if (ok) tc::commit(&tfull[b]);
      }
      if (!ok) {
        *abort_flag = 1;
        if (a.g.error) atomicExch(a.g.error, 1);
      }
      // every MMA issued by this thread completes before the CTA leaves
      tc::commit(drain);
      tc::mbar_wait(drain, 0, a.wait_limit);
    }
    __syncwarp();
  } else {
    // epilogue: warp w reads tensor-memory lanes 32 (w % 4) .. + 31, columns
    // of its half
    const int q = warp & 3, half = (warp - 2) >> 2;
    bool ok = true;
    if (a.g.stall_polls > 0) {
      // self-test of the timeout path: a wait that cannot succeed
      const bool done = tc::mbar_wait(stall, 0, a.g.stall_polls);
      ok = __all_sync(0xffffffffu, done);
    }
    for (long long ti = 0; ti < my_tiles && ok; ti++) {
      const long long tile = blockIdx.x + ti * gridDim.x;
      const int tm = (int)(tile % a.tiles_m);
      const int b = (int)(ti & 1);
      bool done = tc::mbar_wait_or_abort(&tfull[b], (uint32_t)((ti >> 1) & 1), a.wait_limit, abort_flag);
      if (!__all_sync(0xffffffffu, done) || *abort_flag) {
        ok = false;
        break;
      }
      tc::fence_after();
      const int m = tm * 128 + q * 32 + lane;
      const int m0 = tm * 128 + q * 32;
      float* sg = staging + (warp - 2) * kGemmStageWords;
      auto epilogue = [&](const uint32_t* r, int n0) {
        if (!__all_sync(0xffffffffu, gemm_epilogue32_staged<ROWB>(a.g, r, m0, n0, sg)))
          gemm_epilogue32<ROWB>(a.g, r, m, n0);
      };
      const uint32_t trow = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(b * ncols);
      const int nall = (a.nt + 31) / 32, nh = (nall + 1) / 2;
      const int b0 = half * nh, b1 = min(nall, b0 + nh);
      if (b0 < b1) {
        uint32_t rb[2][32];
        tc::tmem_ld32_async(trow + (uint32_t)(32 * b0), rb[0]);
        tc::tmem_wait_ld(rb[0]);
        for (int blk = b0; blk < b1; blk += 2) {
          if (blk + 1 < b1) tc::tmem_ld32_async(trow + (uint32_t)(32 * (blk + 1)), rb[1]);
          epilogue(rb[0], 32 * blk);
          if (blk + 1 < b1) {
            tc::tmem_wait_ld(rb[1]);
            if (blk + 2 < b1) tc::tmem_ld32_async(trow + (uint32_t)(32 * (blk + 2)), rb[0]);
            epilogue(rb[1], 32 * (blk + 1));
            if (blk + 2 < b1) tc::tmem_wait_ld(rb[0]);
          }
        }
      }
      tc::fence_before();
      tc::mbar_arrive(&tempty[b]);
    }
    if (!ok) {
      *abort_flag = 1;
      if (lane == 0 && a.g.error) atomicExch(a.g.error, 1);
    }
  }
  tc::fence_before();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, 2 * ncols);
}

// ---------------------------------------------------------------------------
// Host side: tensor maps through the driver entry point (no link to libcuda)
// ---------------------------------------------------------------------------

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  });
  return fn;
}

// rows x cols bf16, row-major with leading dimension ld (elements); box
// box_rows x 64 with 128-byte swizzle; out-of-range rows read as zero.
static bool make_map(CUtensorMap* map, const void* base, long long rows, long long cols, long long ld, int box_rows) {
  EncodeTiledFn fn = encode_fn();
  if (!fn) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)(ld * 2)};
  const cuuint32_t box[2] = {(cuuint32_t)kGemmBK, (cuuint32_t)box_rows};
  const cuuint32_t estr[2] = {1, 1};
  return fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

int launch_gemm_tn(const GemmArgs& g, int splits, cudaStream_t st) {
  if (g.N < 1 || g.N > 256 || g.M < 1 || splits < 1) return -1;
  if (g.K % ((long long)kGemmBK * splits) != 0) return -1;
  // TMA: 16-byte aligned bases and row strides
  if ((reinterpret_cast<uintptr_t>(g.A) & 15) || (reinterpret_cast<uintptr_t>(g.B) & 15) || (g.lda % 8) ||
      (g.ldb % 8))
    return -1;
  GemmKernelArgs a;
  a.g = g;
  a.nt = (g.N + 15) / 16 * 16;
  a.splits = splits;
  a.tiles_m = (g.M + 127) / 128;
  a.kper = g.K / splits;
  a.wait_limit = g.wait_limit > 0 ? g.wait_limit : wait_limit();
  const int stage_bytes = kGemmTileA + a.nt * kGemmBK * 2;
  const long long kchunks = a.kper / kGemmBK;
  a.stages = (int)std::min<long long>(std::min(kGemmSmemBudget / stage_bytes, 8), std::max<long long>(kchunks, 2));
  // the epilogue warps' staging tiles after the stages and the barriers
  const size_t staging = (size_t)(kGemmEpilogueThreads / 32) * kGemmStageWords * sizeof(float);
  CUtensorMap mapA, mapB;
  if (!make_map(&mapA, g.A, g.M, g.K, g.lda, 128) || !make_map(&mapB, g.B, g.N, g.K, g.ldb, a.nt)) return -1;
  size_t smem = 1024 + (size_t)a.stages * stage_bytes + 1024 + staging;
  // two 256-column accumulators take all of an SM's tensor memory: one CTA per SM
  if (a.nt > 128) smem = std::max<size_t>(smem, 120 * 1024);
  if (g.row_bias && !g.row_group) return -1;
  auto* kernel = g.row_bias ? k_gemm_tn<true> : k_gemm_tn<false>;
  if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return -1;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return -1;
  const long long ntiles = (long long)a.tiles_m * splits;
  const unsigned grid = (unsigned)std::min<long long>(ntiles, sms);
  kernel<<<grid, kGemmThreads, smem, st>>>(mapA, mapB, a);
  return 0;
}

}  // namespace sfsim
