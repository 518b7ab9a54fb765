// k_noise.cu -- sfsim's cloud-noise table builders on the GPU:
//  * Worley noise (src/clj/sfsim/worley.clj:96-109): per voxel the distance to
//    the nearest random point of the 27 surrounding cells of a periodic grid,
//    scaled by the maximum and inverted;
//  * Perlin noise (src/clj/sfsim/perlin.clj:111-133): improved gradient noise
//    with the 12 edge gradients, scaled to [0, 1];
//  * blue noise (src/clj/sfsim/bluenoise.clj:112-172): Ulichney's void and
//    cluster dithering on an m x m torus.
// The random inputs (point grid, gradient indices, seed pixels) are
// arguments; the host draws them.  Worley and Perlin run in FP32 with the
// voxel-to-point differences formed exactly; blue noise runs in FP64 with
// the reference's order of operations per pixel, so its ranks agree exactly
// with the FP64 oracle for the same seed.
#include <math.h>
#include <stdint.h>

#include "kernels.h"

namespace sfsim {

// ---------------------------------------------------------------- Worley

// local[c] = point of cell c relative to the cell's lower corner (FP32)
__global__ void k_worley_local(int divisions, int size, const double* grid, float4* local) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = divisions * divisions * divisions;
  if (c >= n) return;
  const int cs = size / divisions;
  const int i = c % divisions, j = (c / divisions) % divisions, k = c / (divisions * divisions);
  local[c] = make_float4((float)(grid[3 * c] - (double)(i * cs)), (float)(grid[3 * c + 1] - (double)(j * cs)),
                         (float)(grid[3 * c + 2] - (double)(k * cs)), 0.0f);
}

// Distance to the nearest point; out[(k size + j) size + i] for the point
// (k + 0.5, j + 0.5, i + 0.5) as worley-noise orders it.  The cell origin of
// a neighbour one beyond the grid is its unwrapped index times the cell size
// (clipped-index-and-offset adds the texture size exactly there).
__global__ void k_worley_distance(int divisions, int size, const float4* __restrict__ local, float* out,
                                  unsigned int* max_bits) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long n = (long long)size * size * size;
  float d2min = INFINITY;
  if (t < n) {
    const int i = (int)(t % size), j = (int)((t / size) % size), k = (int)(t / ((long long)size * size));
    const int cs = size / divisions;
    const int cx = k / cs, cy = j / cs, cz = i / cs;  // cells of x = k + 0.5, y = j + 0.5, z = i + 0.5
    for (int dk = -1; dk <= 1; dk++) {
      const int nz = cz + dk, wz = nz < 0 ? nz + divisions : nz >= divisions ? nz - divisions : nz;
      const float rz = (float)(i - nz * cs) + 0.5f;
      for (int dj = -1; dj <= 1; dj++) {
        const int ny = cy + dj, wy = ny < 0 ? ny + divisions : ny >= divisions ? ny - divisions : ny;
        const float ry = (float)(j - ny * cs) + 0.5f;
        for (int di = -1; di <= 1; di++) {
          const int nx = cx + di, wx = nx < 0 ? nx + divisions : nx >= divisions ? nx - divisions : nx;
          const float rx = (float)(k - nx * cs) + 0.5f;
          const float4 p = local[(wz * divisions + wy) * divisions + wx];
          const float dx = rx - p.x, dy = ry - p.y, dz = rz - p.z;
          d2min = fminf(d2min, fmaf(dx, dx, fmaf(dy, dy, dz * dz)));
        }
      }
    }
    const float d = sqrtf(d2min);
    out[t] = d;
    d2min = d;
  } else {
    d2min = 0.0f;
  }
  // maximum over the block, then one atomic (non-negative floats order as their bits)
  for (int o = 16; o > 0; o >>= 1) d2min = fmaxf(d2min, __shfl_xor_sync(0xffffffffu, d2min, o));
  __shared__ float wmax[32];
  if ((threadIdx.x & 31) == 0) wmax[threadIdx.x >> 5] = d2min;
  __syncthreads();
  if (threadIdx.x < 32) {
    float v = threadIdx.x < (blockDim.x >> 5) ? wmax[threadIdx.x] : 0.0f;
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    if (threadIdx.x == 0) atomicMax(max_bits, __float_as_uint(v));
  }
}

__global__ void k_worley_finish(long long n, const unsigned int* max_bits, float* out) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= n) return;
  out[t] = 1.0f - out[t] / __uint_as_float(*max_bits);
}

// ---------------------------------------------------------------- Perlin

__constant__ signed char c_gradients[12][3] = {{1, 1, 0},  {-1, 1, 0},  {1, -1, 0}, {-1, -1, 0},
                                               {1, 0, 1},  {-1, 0, 1},  {1, 0, -1}, {-1, 0, -1},
                                               {0, 1, 1},  {0, -1, 1},  {0, 1, -1}, {0, -1, -1}};

__device__ __forceinline__ float ease(float t) { return (((t * 6.0f - 15.0f) * t + 10.0f) * t) * t * t; }

// Monotone map of floats to unsigned ints (for atomic min / max).
__device__ __forceinline__ unsigned int ordered(float f) {
  const unsigned int u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float unordered(unsigned int u) {
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u);
}

// perlin-noise-sample at the cell (i + 0.5, j + 0.5, k + 0.5) into
// out[(k size + j) size + i]; the minimum and maximum go to range[0..1].
__global__ void k_perlin_sample(int divisions, int size, const int* __restrict__ gradients, float* out,
                                unsigned int* range) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long n = (long long)size * size * size;
  float lo = INFINITY, hi = -INFINITY;
  if (t < n) {
    const int i = (int)(t % size), j = (int)((t / size) % size), k = (int)(t / ((long long)size * size));
    const float scale = (float)divisions / (float)size;
    const float p[3] = {((float)i + 0.5f) * scale, ((float)j + 0.5f) * scale, ((float)k + 0.5f) * scale};
    const int x = (int)floorf(p[0]), y = (int)floorf(p[1]), z = (int)floorf(p[2]);
    const int xs[2] = {x, (x + 1) % divisions}, ys[2] = {y, (y + 1) % divisions}, zs[2] = {z, (z + 1) % divisions};
    const float f[3] = {p[0] - (float)x, p[1] - (float)y, p[2] - (float)z};
    const float ex[2] = {ease(1.0f - f[0]), ease(f[0])}, ey[2] = {ease(1.0f - f[1]), ease(f[1])},
                ez[2] = {ease(1.0f - f[2]), ease(f[2])};
    float sum = 0.0f;
#pragma unroll
    for (int zc = 0; zc < 2; zc++)
#pragma unroll
      for (int yc = 0; yc < 2; yc++)
#pragma unroll
        for (int xc = 0; xc < 2; xc++) {
          const int gi = gradients[(zs[zc] * divisions + ys[yc]) * divisions + xs[xc]];
          const float vx = f[0] - (float)xc, vy = f[1] - (float)yc, vz = f[2] - (float)zc;
          const float infl = (float)c_gradients[gi][0] * vx + (float)c_gradients[gi][1] * vy +
                             (float)c_gradients[gi][2] * vz;
          sum = fmaf(ez[zc] * ey[yc] * ex[xc], infl, sum);
        }
    out[t] = sum;
    lo = hi = sum;
  }
  for (int o = 16; o > 0; o >>= 1) {
    lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  if ((threadIdx.x & 31) == 0 && lo <= hi) {
    atomicMin(range, ordered(lo));
    atomicMax(range + 1, ordered(hi));
  }
}

__global__ void k_perlin_finish(long long n, const unsigned int* range, float* out) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= n) return;
  const float lo = unordered(range[0]), hi = unordered(range[1]);
  out[t] = (out[t] - lo) / (hi - lo);
}

// ------------------------------------------------------------ blue noise

constexpr int kBlueThreads = 1024;

struct BlueArgs {
  int m;
  double sigma;
  const int* seed;  // n pixel indices
  int n;
  const double* table;  // Gauss weights [|dy|][|dx|], (m/2 + 1)^2
  double* density;      // m*m (shared memory when it fits, else this global array)
  double* density0;     // m*m global scratch
  unsigned char* mask;  // m*m global scratch (used when shared memory is too small)
  unsigned char* work;
  int* dither;          // m*m output
  int use_smem;
};

__device__ __forceinline__ int wrap_m(int x, int m) {
  const int offset = m >> 1;
  int r = (x + offset) % m;
  if (r < 0) r += m;
  return r - offset;
}

// Best (value, index) under "larger value wins, equal values: larger index"
// (max-key / min-key keep the last of equal elements); min searches negate.
struct Best {
  double v;
  int i;
};
__device__ __forceinline__ Best better(Best a, Best b) {
  if (b.i < 0) return a;
  if (a.i < 0) return b;
  if (b.v > a.v || (b.v == a.v && b.i > a.i)) return b;
  return a;
}

// Block-wide arg-extremum over pixels whose mask equals `want`: arg max of
// density (sign +1) or arg min (sign -1).  All threads get the index.
__device__ int block_arg(const double* density, const unsigned char* mask, int total, unsigned char want,
                         double sign, Best* red) {
  Best b{0.0, -1};
  for (int p = threadIdx.x; p < total; p += kBlueThreads)
    if (mask[p] == want) b = better(b, Best{sign * density[p], p});
  for (int o = 16; o > 0; o >>= 1) {
    Best c;
    c.v = __shfl_xor_sync(0xffffffffu, b.v, o);
    c.i = __shfl_xor_sync(0xffffffffu, b.i, o);
    b = better(b, c);
  }
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = b;
  __syncthreads();
  if (threadIdx.x < 32) {
    Best c = red[threadIdx.x];
    for (int o = 16; o > 0; o >>= 1) {
      Best e;
      e.v = __shfl_xor_sync(0xffffffffu, c.v, o);
      e.i = __shfl_xor_sync(0xffffffffu, c.i, o);
      c = better(c, e);
    }
    if (threadIdx.x == 0) red[32] = c;
  }
  __syncthreads();
  const int r = red[32].i;
  __syncthreads();  // red is reused by the next search
  return r;
}

__device__ __forceinline__ double weight(const double* table, int h, int dx, int dy) {
  return table[abs(dy) * h + abs(dx)];
}

// density-change (bluenoise.clj:99-109) of every pixel by +/- the weight of
// its offset from `index`
__device__ void change(double* density, int m, const double* table, int index, bool add) {
  const int cy = index / m, cx = index % m, h = (m >> 1) + 1, total = m * m;
  for (int p = threadIdx.x; p < total; p += kBlueThreads) {
    const double f = weight(table, h, wrap_m(p % m - cx, m), wrap_m(p / m - cy, m));
    density[p] = add ? density[p] + f : density[p] - f;
  }
}

// density-array (bluenoise.clj:79-96): each pixel sums over the set pixels
// in row-major order, as density-sample does
__device__ void density_array(double* density, const unsigned char* mask, int m, const double* table) {
  const int h = (m >> 1) + 1, total = m * m;
  for (int p = threadIdx.x; p < total; p += kBlueThreads) {
    const int cy = p / m, cx = p % m;
    double s = 0.0;
    for (int y = 0; y < m; y++)
      for (int x = 0; x < m; x++)
        if (mask[y * m + x]) s += weight(table, h, wrap_m(x - cx, m), wrap_m(y - cy, m));
    density[p] = s;
  }
}

// One CTA runs the whole dithering: seed pattern, phases 1-3 (one arg search
// and one density change per step, two block barriers each).
__global__ void __launch_bounds__(kBlueThreads, 1) k_blue_noise(BlueArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ Best red[33];
  const int m = a.m, total = m * m, h = (m >> 1) + 1;
  double* table = reinterpret_cast<double*>(smem);
  unsigned char* base = smem + sizeof(double) * h * h;
  double* density = a.use_smem ? reinterpret_cast<double*>(base) : a.density;
  unsigned char* mask = a.use_smem ? base + sizeof(double) * total : a.mask;
  unsigned char* work = a.use_smem ? mask + total : a.work;
  for (int t = threadIdx.x; t < h * h; t += kBlueThreads) table[t] = a.table[t];
  for (int p = threadIdx.x; p < total; p += kBlueThreads) {
    mask[p] = 0;
    a.dither[p] = 0;
  }
  __syncthreads();
  for (int t = threadIdx.x; t < a.n; t += kBlueThreads) mask[a.seed[t]] = 1;
  __syncthreads();

  // seed-pattern (bluenoise.clj:112-124)
  density_array(density, mask, m, table);
  __syncthreads();
  for (int it = 0; it < total * 4; it++) {  // the pattern settles long before this bound
    const int cluster = block_arg(density, mask, total, 1, 1.0, red);
    if (cluster < 0) break;  // no set pixel: cannot happen for 1 <= n <= m*m/2
    if (threadIdx.x == 0) mask[cluster] = 0;
    change(density, m, table, cluster, false);
    __syncthreads();
    const int vd = block_arg(density, mask, total, 0, -1.0, red);
    if (vd < 0) break;
    if (threadIdx.x == 0) mask[vd] = 1;
    __syncthreads();
    if (cluster == vd) break;
    change(density, m, table, vd, true);
    __syncthreads();
  }
  density_array(a.density0, mask, m, table);
  __syncthreads();

  // phase 1 (bluenoise.clj:127-140) from the seed pattern
  for (int p = threadIdx.x; p < total; p += kBlueThreads) {
    work[p] = mask[p];
    density[p] = a.density0[p];
  }
  __syncthreads();
  for (int r = a.n; r > 0; r--) {
    const int cluster = block_arg(density, work, total, 1, 1.0, red);
    if (cluster < 0) break;
    change(density, m, table, cluster, false);
    if (threadIdx.x == 0) {
      work[cluster] = 0;
      a.dither[cluster] = r - 1;
    }
    __syncthreads();
  }
  // phase 2 (bluenoise.clj:143-154) from the seed pattern
  for (int p = threadIdx.x; p < total; p += kBlueThreads) {
    work[p] = mask[p];
    density[p] = a.density0[p];
  }
  __syncthreads();
  for (int r = a.n; r < total / 2; r++) {
    const int vd = block_arg(density, work, total, 0, -1.0, red);
    if (vd < 0) break;
    change(density, m, table, vd, true);
    if (threadIdx.x == 0) {
      work[vd] = 1;
      a.dither[vd] = r;
    }
    __syncthreads();
  }
  // phase 3 (bluenoise.clj:157-169) on the complement
  for (int p = threadIdx.x; p < total; p += kBlueThreads) work[p] = !work[p];
  __syncthreads();
  density_array(density, work, m, table);
  __syncthreads();
  for (int r = total / 2; r < total; r++) {
    const int cluster = block_arg(density, work, total, 1, 1.0, red);
    if (cluster < 0) break;
    change(density, m, table, cluster, false);
    if (threadIdx.x == 0) {
      work[cluster] = 0;
      a.dither[cluster] = r;
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------- launches

static inline unsigned blocks_for(long long n, int b) { return (unsigned)((n + b - 1) / b); }

void launch_worley(int divisions, int size, const double* grid, float4* local, float* out, unsigned int* max_bits,
                   cudaStream_t st) {
  const int nc = divisions * divisions * divisions;
  k_worley_local<<<blocks_for(nc, 256), 256, 0, st>>>(divisions, size, grid, local);
  const long long n = (long long)size * size * size;
  k_worley_distance<<<blocks_for(n, 256), 256, 0, st>>>(divisions, size, local, out, max_bits);
  k_worley_finish<<<blocks_for(n, 256), 256, 0, st>>>(n, max_bits, out);
}

void launch_perlin(int divisions, int size, const int* gradients, float* out, unsigned int* range,
                   cudaStream_t st) {
  const long long n = (long long)size * size * size;
  k_perlin_sample<<<blocks_for(n, 256), 256, 0, st>>>(divisions, size, gradients, out, range);
  k_perlin_finish<<<blocks_for(n, 256), 256, 0, st>>>(n, range, out);
}

size_t blue_noise_smem(int m, bool* use_smem) {
  const size_t h = (size_t)(m / 2 + 1);
  const size_t table = sizeof(double) * h * h;
  const size_t all = table + sizeof(double) * (size_t)m * m + 2 * (size_t)m * m;
  *use_smem = all <= 200 * 1024;
  return *use_smem ? all : table;
}

int launch_blue_noise(int m, int n, const int* seed, double sigma, const double* table, double* density,
                      double* density0, unsigned char* mask, unsigned char* work, int* dither, cudaStream_t st) {
  BlueArgs a;
  a.m = m;
  a.sigma = sigma;
  a.seed = seed;
  a.n = n;
  a.table = table;
  a.density = density;
  a.density0 = density0;
  a.mask = mask;
  a.work = work;
  a.dither = dither;
  bool use = false;
  const size_t smem = blue_noise_smem(m, &use);
  a.use_smem = use ? 1 : 0;
  if (cudaFuncSetAttribute(k_blue_noise, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return -1;
  k_blue_noise<<<1, kBlueThreads, smem, st>>>(a);
  return 0;
}

}  // namespace sfsim
