// k_mlp.cu -- CUDA-core kernels of the ray-scatter surrogate: a Fourier-
// feature MLP over ten coordinates of a query (the four table coordinates,
// the unclamped sun elevation, the table half and the four cell phases; each
// in [0, 1]) with 4 x 256 SiLU hidden layers and 4 outputs (three log-space
// corrections to the table lookup, the log of their expected squared error).
// The hidden-layer GEMMs run on the tensor cores (k_gemm.cu); these kernels
// do the features, the 256 -> 4 head, the loss, bias gradients, Adam, the
// sampling of training batches, and the conditioned network's atmosphere
// term.
#include <cuda_bf16.h>

#include "atmo_device.cuh"
#include "kernels.h"

namespace sfsim {

// F[i][32 d + 2 k] = sin(pi f_k u_d), F[i][32 d + 2 k + 1] = cos(pi f_k u_d);
// also the transpose FT[256][n] when requested.  A block computes the
// features of 32 rows into shared memory, then writes F row by row and FT
// as 32 consecutive entries (64 bytes) of each transposed row.
constexpr int kFeatTile = 32;
__global__ void k_features(long long n, const float* __restrict__ coords, __nv_bfloat16* __restrict__ F,
                           __nv_bfloat16* __restrict__ FT) {
  __shared__ __align__(16) __nv_bfloat16 tile[kFeatTile][kMlpIn + 8];
  const long long i0 = blockIdx.x * (long long)kFeatTile;
  const int rows = (int)min((long long)kFeatTile, n - i0);
  for (int e = threadIdx.x; e < rows * (kMlpIn / 2); e += blockDim.x) {
    const int r = e / (kMlpIn / 2), f = e % (kMlpIn / 2);
    const long long i = i0 + r;
    int d;
    float freq;
    feature_pair(f, &d, &freq);
    float sv, cv;
    sincospif(freq * coords[i * kMlpCoords + d], &sv, &cv);
    __nv_bfloat162 pr;
    pr.x = __float2bfloat16(sv);
    pr.y = __float2bfloat16(cv);
    *reinterpret_cast<__nv_bfloat162*>(&tile[r][2 * f]) = pr;
    *reinterpret_cast<__nv_bfloat162*>(F + i * kMlpIn + 2 * f) = pr;
  }
  if (!FT) return;
  __syncthreads();
  for (int c = threadIdx.x; c < kMlpIn; c += blockDim.x) {
    __nv_bfloat16* dst = FT + (long long)c * n + i0;
    if (rows == kFeatTile && (n & 7) == 0) {
      // i0 is a multiple of 32 and n of 8: the row segment is 16-byte aligned
#pragma unroll
      for (int q = 0; q < kFeatTile / 8; q++) {
        uint32_t w[4];
#pragma unroll
        for (int e = 0; e < 4; e++) {
          __nv_bfloat162 pr;
          pr.x = tile[8 * q + 2 * e][c];
          pr.y = tile[8 * q + 2 * e + 1][c];
          w[e] = *reinterpret_cast<const uint32_t*>(&pr);
        }
        reinterpret_cast<uint4*>(dst)[q] = make_uint4(w[0], w[1], w[2], w[3]);
      }
    } else {
      for (int r = 0; r < rows; r++) dst[r] = tile[r][c];
    }
  }
}

// out[i][c] = sum_j H[i][j] W5[c][j] + b5[c], c < kMlpOut; one warp per row,
// each lane one 16-byte load of eight BF16 (kMlpHidden == 256), W5 staged in
// shared memory.
static_assert(kMlpHidden == 256, "k_head_forward reads a row as 32 lanes x 8 BF16");
__global__ void k_head_forward(long long n, const __nv_bfloat16* __restrict__ H, const float* __restrict__ W5,
                               const float* __restrict__ b5, float* __restrict__ out) {
  __shared__ float sW[kMlpOut * kMlpHidden];
  for (int t = threadIdx.x; t < kMlpOut * kMlpHidden; t += blockDim.x) sW[t] = W5[t];
  __syncthreads();
  const long long row = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (row >= n) return;
  const uint4 q = *reinterpret_cast<const uint4*>(H + row * kMlpHidden + 8 * lane);
  const uint32_t wq[4] = {q.x, q.y, q.z, q.w};
  float h[8];
#pragma unroll
  for (int e = 0; e < 4; e++) {
    const float2 f = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&wq[e]));
    h[2 * e] = f.x;
    h[2 * e + 1] = f.y;
  }
  float acc[kMlpOut];
#pragma unroll
  for (int c = 0; c < kMlpOut; c++) {
    const float* w = sW + c * kMlpHidden + 8 * lane;
    float a = 0;
#pragma unroll
    for (int e = 0; e < 8; e++) a = fmaf(h[e], w[e], a);
    acc[c] = a;
  }
#pragma unroll
  for (int c = 0; c < kMlpOut; c++) {
    for (int o = 16; o > 0; o >>= 1) acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], o);
    if (lane == 0) out[row * kMlpOut + c] = acc[c] + b5[c];
  }
}

// Per row: e_c = out_c - target_c (c < 3), m = mean e_c^2, s = out_3.
// dout_c = 2 e_c / (3 n), with e_c clamped to [-huber, huber] when huber > 0
// (the Huber loss); dout_3 = var_weight (1 - m exp(-s)) / (2 n), the
// gradient of the Gaussian negative log-likelihood (m exp(-s) + s) / 2 of the
// squared error under the predicted variance exp(s), with m held fixed.
// loss += m / n.
__global__ void k_loss_grad(long long n, const float* __restrict__ out, const float* __restrict__ target,
                            float huber, float var_weight, float* __restrict__ dout, float* __restrict__ loss) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  float e2 = 0;
  if (t < n) {
    const float inv = 1.0f / (float)n;
    float m = 0;
#pragma unroll
    for (int c = 0; c < 3; c++) {
      const float e = out[t * kMlpOut + c] - target[t * 3 + c];
      const float ge = huber > 0 ? fminf(fmaxf(e, -huber), huber) : e;
      dout[t * kMlpOut + c] = 2.0f * ge * inv / 3.0f;
      m += e * e;
    }
    m *= 1.0f / 3.0f;
    const float s = fminf(fmaxf(out[t * kMlpOut + 3], -40.0f), 20.0f);
    dout[t * kMlpOut + 3] = var_weight * 0.5f * (1.0f - m * __expf(-s)) * inv;
    e2 = m * inv;
  }
  for (int o = 16; o > 0; o >>= 1) e2 += __shfl_xor_sync(0xffffffffu, e2, o);
  if ((threadIdx.x & 31) == 0 && e2 != 0.0f) atomicAdd(loss, e2);
}

static_assert(kMlpOut == 4, "the head kernels read rows of dout as float4");

// Backward of the head: dZ4[i][j] = (sum_c dout[i][c] W5[c][j]) * dsilu4[i][j]
// (BF16, also transposed), and dW5 += dout^T H4, db5 += sum dout.  Thread j
// of a block handles hidden unit j over the block's rows, 32 rows at a time:
// the tile of 32 x 256 BF16 gradients passes through shared memory so that
// each thread writes 32 consecutive entries of one transposed row (64 bytes)
// instead of 32 scattered 2-byte values.  The rows of a block start at a
// multiple of 32 (n is a multiple of 1024).
constexpr int kHeadTile = 32;
__global__ void k_head_backward(long long n, const float* __restrict__ dout, const __nv_bfloat16* __restrict__ H,
                                const float* __restrict__ W5, const float* __restrict__ dsilu,
                                __nv_bfloat16* __restrict__ dZ, __nv_bfloat16* __restrict__ dZT,
                                float* __restrict__ dW5, float* __restrict__ db5) {
  __shared__ float sW[kMlpOut * kMlpHidden];
  // [row][unit], 8 BF16 of padding a row: column reads hit 16 banks, one word per lane pair
  __shared__ __align__(16) __nv_bfloat16 tile[kHeadTile][kMlpHidden + 8];
  for (int t = threadIdx.x; t < kMlpOut * kMlpHidden; t += blockDim.x) sW[t] = W5[t];
  __syncthreads();
  const int j = threadIdx.x;  // blockDim.x == kMlpHidden
  const long long tiles = n / kHeadTile;
  const long long tiles_per_block = (tiles + gridDim.x - 1) / gridDim.x;
  const long long t0 = blockIdx.x * tiles_per_block, t1 = min(tiles, t0 + tiles_per_block);
  float gw[kMlpOut] = {}, gb[kMlpOut] = {};
  for (long long tl = t0; tl < t1; tl++) {
    const long long i0 = tl * kHeadTile;
#pragma unroll 8
    for (int ii = 0; ii < kHeadTile; ii++) {
      const long long i = i0 + ii;
      const float4 d = *reinterpret_cast<const float4*>(dout + i * kMlpOut);
      const float dd[kMlpOut] = {d.x, d.y, d.z, d.w};
      const float h = __bfloat162float(H[i * kMlpHidden + j]);
      float dh = 0;
#pragma unroll
      for (int c = 0; c < kMlpOut; c++) {
        gw[c] = fmaf(dd[c], h, gw[c]);
        gb[c] += dd[c];
        dh = fmaf(dd[c], sW[c * kMlpHidden + j], dh);
      }
      const __nv_bfloat16 dz = __float2bfloat16(dh * dsilu[i * kMlpHidden + j]);
      dZ[i * kMlpHidden + j] = dz;
      tile[ii][j] = dz;
    }
    __syncthreads();
    // transposed row j, entries i0 .. i0 + 31: four 16-byte stores
    uint4* dst = reinterpret_cast<uint4*>(dZT + (long long)j * n + i0);
#pragma unroll
    for (int q = 0; q < kHeadTile / 8; q++) {
      uint32_t w[4];
#pragma unroll
      for (int e = 0; e < 4; e++) {
        __nv_bfloat162 pr;
        pr.x = tile[8 * q + 2 * e][j];
        pr.y = tile[8 * q + 2 * e + 1][j];
        w[e] = *reinterpret_cast<const uint32_t*>(&pr);
      }
      dst[q] = make_uint4(w[0], w[1], w[2], w[3]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int c = 0; c < kMlpOut; c++) atomicAdd(dW5 + c * kMlpHidden + j, gw[c]);
  if (j == 0) {
#pragma unroll
    for (int c = 0; c < kMlpOut; c++) atomicAdd(db5 + c, gb[c]);
  }
}

// db[j] += sum_i dZT[j][i] (the transposed gradients make the rows
// contiguous); kBiasSplit blocks share a row, each reading 8 BF16 at a time,
// and add their partial sums atomically.  n is a multiple of 1024.
constexpr int kBiasSplit = 8;
__global__ void k_bias_grad(long long n, int width, const __nv_bfloat16* __restrict__ dZT, float* __restrict__ db) {
  const int j = blockIdx.x / kBiasSplit, part = blockIdx.x % kBiasSplit;
  const long long n8 = n / 8;
  const uint4* row = reinterpret_cast<const uint4*>(dZT + (long long)j * n);
  float s = 0;
  for (long long v = part * (long long)blockDim.x + threadIdx.x; v < n8; v += (long long)kBiasSplit * blockDim.x) {
    const uint4 q = row[v];
    const uint32_t w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
    for (int e = 0; e < 4; e++) {
      const float2 f = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&w[e]));
      s += f.x + f.y;
    }
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  __shared__ float red[32];
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    s = threadIdx.x < (int)(blockDim.x >> 5) ? red[threadIdx.x] : 0.0f;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) atomicAdd(db + j, s);
  }
  (void)width;
}

// Adam with bias correction over the whole parameter vector [0, count) in one
// launch; the elements of the weight matrices listed in `mats` also refresh
// their BF16 copy [rows][cols] and its transpose.
__global__ void k_adam_all(long long count, float* __restrict__ w, const float* __restrict__ g,
                           float* __restrict__ m, float* __restrict__ v, float lr, float beta1, float beta2, float eps,
                           float c1, float c2, AdamMatrices mats) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= count) return;
  const float gt = g[t];
  const float mt = beta1 * m[t] + (1 - beta1) * gt;
  const float vt = beta2 * v[t] + (1 - beta2) * gt * gt;
  m[t] = mt;
  v[t] = vt;
  const float mhat = mt / c1, vhat = vt / c2;
  const float wt = w[t] - lr * mhat / (sqrtf(vhat) + eps);
  w[t] = wt;
#pragma unroll
  for (int k = 0; k < AdamMatrices::kMax; k++) {
    if (k >= mats.n) break;
    const long long o = t - mats.start[k];
    if (o >= 0 && o < (long long)mats.rows[k] * mats.cols[k]) {
      const int r = (int)(o / mats.cols[k]), c = (int)(o % mats.cols[k]);
      mats.wb[k][o] = __float2bfloat16(wt);
      mats.wbt[k][(long long)c * mats.rows[k] + r] = __float2bfloat16(wt);
    }
  }
}

// Adam with bias correction on FP32 master weights; refreshes the BF16
// copy W_bf16 [rows][cols] and its transpose WT_bf16 [cols][rows] when given.
__global__ void k_adam(long long count, float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, float lr, float beta1, float beta2, float eps, float c1, float c2,
                       int rows, int cols, __nv_bfloat16* __restrict__ wb, __nv_bfloat16* __restrict__ wbt) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= count) return;
  const float gt = g[t];
  const float mt = beta1 * m[t] + (1 - beta1) * gt;
  const float vt = beta2 * v[t] + (1 - beta2) * gt * gt;
  m[t] = mt;
  v[t] = vt;
  const float mhat = mt / c1, vhat = vt / c2;
  const float wt = w[t] - lr * mhat / (sqrtf(vhat) + eps);
  w[t] = wt;
  if (wb) {
    const int r = (int)(t / cols), c = (int)(t % cols);
    wb[t] = __float2bfloat16(wt);
    if (wbt) wbt[(long long)c * rows + r] = __float2bfloat16(wt);
  }
}

__global__ void k_to_bf16(long long count, const float* __restrict__ w, int rows, int cols,
                          __nv_bfloat16* __restrict__ wb, __nv_bfloat16* __restrict__ wbt) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= count) return;
  const int r = (int)(t / cols), c = (int)(t % cols);
  wb[t] = __float2bfloat16(w[t]);
  if (wbt) wbt[(long long)c * rows + r] = __float2bfloat16(w[t]);
}

// SplitMix64 hash for reproducible sampling.
__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// Batch of n rows: a fraction `node_frac` drawn from pool A (na samples),
// the rest from pool B (nb samples); each sample is kMlpCoords coordinates and
// 3 targets.
__global__ void k_gather_batch(long long n, unsigned long long seed, float node_frac, const float* __restrict__ poolA,
                               long long na, const float* __restrict__ poolB, long long nb, float* __restrict__ coords,
                               float* __restrict__ target) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const unsigned long long h = mix64(seed ^ (unsigned long long)i * 0x2545F4914F6CDD1Dull);
  const bool fromA = nb == 0 || ((h >> 40) & 0xFFFFFF) < (unsigned long long)(node_frac * 16777216.0f);
  const float* src = fromA ? poolA + kPoolRow * (long long)(mix64(h) % (unsigned long long)na)
                           : poolB + kPoolRow * (long long)(mix64(h + 1) % (unsigned long long)nb);
#pragma unroll
  for (int c = 0; c < kMlpCoords; c++) coords[i * kMlpCoords + c] = src[c];
#pragma unroll
  for (int c = 0; c < 3; c++) target[i * 3 + c] = src[kMlpCoords + c];
}

// Conditioned batches: the group (atmosphere) of row i is drawn uniformly,
// then the row from that group's pool A (table nodes) or pool B (direct
// samples) as k_gather_batch does.
__global__ void k_gather_batch_groups(long long n, unsigned long long seed, float node_frac, int groups,
                                      const float* const* __restrict__ poolsA, long long na,
                                      const float* const* __restrict__ poolsB, long long nb,
                                      float* __restrict__ coords, float* __restrict__ target,
                                      int* __restrict__ group) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const unsigned long long h = mix64(seed ^ (unsigned long long)i * 0x2545F4914F6CDD1Dull);
  const int a = (int)(mix64(h + 2) % (unsigned long long)groups);
  const bool fromA = nb == 0 || ((h >> 40) & 0xFFFFFF) < (unsigned long long)(node_frac * 16777216.0f);
  const float* src = fromA ? poolsA[a] + kPoolRow * (long long)(mix64(h) % (unsigned long long)na)
                           : poolsB[a] + kPoolRow * (long long)(mix64(h + 1) % (unsigned long long)nb);
#pragma unroll
  for (int c = 0; c < kMlpCoords; c++) coords[i * kMlpCoords + c] = src[c];
#pragma unroll
  for (int c = 0; c < 3; c++) target[i * 3 + c] = src[kMlpCoords + c];
  group[i] = a;
}

// C[a][j] = b1[j] + sum_p U[j][p] G[a][p]: one thread per (a, j).
__global__ void k_cond_bias(int groups, const float* __restrict__ U, const float* __restrict__ G,
                            const float* __restrict__ b1, float* __restrict__ C) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= groups * kMlpHidden) return;
  const int a = t / kMlpHidden, j = t % kMlpHidden;
  float z = b1 ? b1[j] : 0.0f;
#pragma unroll
  for (int p = 0; p < kCondInputs; p++) z = fmaf(U[j * kCondInputs + p], G[a * kCondInputs + p], z);
  C[t] = z;
}

// dU[j][p] += sum_a s_a G[a][p] with s_a = sum over the rows i of group a of
// dZT[j][i]: one block per hidden unit j, the per-group sums in shared memory.
__global__ void k_cond_grad(long long n, const __nv_bfloat16* __restrict__ dZT, const int* __restrict__ group,
                            int groups, const float* __restrict__ G, float* __restrict__ dU) {
  __shared__ float acc[kMaxCondGroups];
  const int j = blockIdx.x;
  for (int a = threadIdx.x; a < groups; a += blockDim.x) acc[a] = 0.0f;
  __syncthreads();
  for (long long i = threadIdx.x; i < n; i += blockDim.x)
    atomicAdd(&acc[group[i]], __bfloat162float(dZT[(long long)j * n + i]));
  __syncthreads();
  if (threadIdx.x < kCondInputs) {
    const int p = threadIdx.x;
    float s = 0.0f;
    for (int a = 0; a < groups; a++) s = fmaf(acc[a], G[a * kCondInputs + p], s);
    dU[j * kCondInputs + p] += s;
  }
}

static inline unsigned grid_for(long long n, int blk) { return (unsigned)((n + blk - 1) / blk); }

void launch_features(long long n, const float* coords, __nv_bfloat16* F, __nv_bfloat16* FT, cudaStream_t st) {
  k_features<<<(unsigned)((n + kFeatTile - 1) / kFeatTile), 256, 0, st>>>(n, coords, F, FT);
}
void launch_head_forward(long long n, const __nv_bfloat16* H, const float* W5, const float* b5, float* out,
                         cudaStream_t st) {
  k_head_forward<<<grid_for(n * 32, 256), 256, 0, st>>>(n, H, W5, b5, out);
}
void launch_loss_grad(long long n, const float* out, const float* target, float huber, float var_weight, float* dout,
                      float* loss, cudaStream_t st) {
  k_loss_grad<<<grid_for(n, 256), 256, 0, st>>>(n, out, target, huber, var_weight, dout, loss);
}
void launch_head_backward(long long n, const float* dout, const __nv_bfloat16* H, const float* W5,
                          const float* dsilu, __nv_bfloat16* dZ, __nv_bfloat16* dZT, float* dW5, float* db5,
                          cudaStream_t st) {
  const int blocks = (int)min(1024LL, (n / kHeadTile + 1) / 2);
  k_head_backward<<<blocks, kMlpHidden, 0, st>>>(n, dout, H, W5, dsilu, dZ, dZT, dW5, db5);
}
void launch_bias_grad(long long n, int width, const __nv_bfloat16* dZT, float* db, cudaStream_t st) {
  k_bias_grad<<<width * kBiasSplit, 256, 0, st>>>(n, width, dZT, db);
}
void launch_adam(long long count, float* w, const float* g, float* m, float* v, float lr, float beta1, float beta2,
                 float eps, int step, int rows, int cols, __nv_bfloat16* wb, __nv_bfloat16* wbt, cudaStream_t st) {
  const float c1 = 1.0f - powf(beta1, (float)step), c2 = 1.0f - powf(beta2, (float)step);
  k_adam<<<grid_for(count, 256), 256, 0, st>>>(count, w, g, m, v, lr, beta1, beta2, eps, c1, c2, rows, cols, wb,
                                                wbt);
}
void launch_adam_all(long long count, float* w, const float* g, float* m, float* v, float lr, float beta1, float beta2,
                     float eps, int step, const AdamMatrices& mats, cudaStream_t st) {
  const float c1 = 1.0f - powf(beta1, (float)step), c2 = 1.0f - powf(beta2, (float)step);
  k_adam_all<<<grid_for(count, 256), 256, 0, st>>>(count, w, g, m, v, lr, beta1, beta2, eps, c1, c2, mats);
}
void launch_to_bf16(long long count, const float* w, int rows, int cols, __nv_bfloat16* wb, __nv_bfloat16* wbt,
                    cudaStream_t st) {
  k_to_bf16<<<grid_for(count, 256), 256, 0, st>>>(count, w, rows, cols, wb, wbt);
}
void launch_gather_batch(long long n, unsigned long long seed, float node_frac, const float* poolA, long long na,
                         const float* poolB, long long nb, float* coords, float* target, cudaStream_t st) {
  k_gather_batch<<<grid_for(n, 256), 256, 0, st>>>(n, seed, node_frac, poolA, na, poolB, nb, coords, target);
}

void launch_gather_batch_groups(long long n, unsigned long long seed, float node_frac, int groups,
                                const float* const* poolsA, long long na, const float* const* poolsB, long long nb,
                                float* coords, float* target, int* group, cudaStream_t st) {
  k_gather_batch_groups<<<grid_for(n, 256), 256, 0, st>>>(n, seed, node_frac, groups, poolsA, na, poolsB, nb, coords,
                                                          target, group);
}
void launch_cond_bias(int groups, const float* U, const float* G, const float* b1, float* C, cudaStream_t st) {
  k_cond_bias<<<grid_for((long long)groups * kMlpHidden, 256), 256, 0, st>>>(groups, U, G, b1, C);
}
void launch_cond_grad(long long n, const __nv_bfloat16* dZT, const int* group, int groups, const float* G, float* dU,
                      cudaStream_t st) {
  k_cond_grad<<<kMlpHidden, 256, 0, st>>>(n, dZT, group, groups, G, dU);
}

}  // namespace sfsim
