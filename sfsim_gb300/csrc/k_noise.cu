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
//
// The void-and-cluster steps are sequential: one CTA of 1024 threads runs
// them (k_blue_seed, k_blue_phases, k_blue_phase3) with the state in shared
// memory when it fits.  The full density sums (density-array), m^4 FP64
// additions each, run between them on every SM (k_blue_density).

constexpr int kBlueThreads = 1024;

struct BlueArgs {
  int m;
  const int* seed;       // n pixel indices
  int n;
  const double* table;   // Gauss weights [|dy|][|dx|], (m/2 + 1)^2
  double* density;       // m*m global scratch
  double* density0;      // m*m: the density of the seed pattern
  unsigned char* mask;   // m*m: the seed mask, then the seed pattern
  unsigned char* work;   // m*m: the complement of the half-filled pattern
  int* dither;           // m*m output ranks
  int use_smem;          // the single-CTA kernels keep density and mask in shared memory
  int* error;            // set to 1 when a cluster wait gave up
  int wait_limit;        // polls per cluster wait
};

// Order-preserving integer key of a double (no NaN; the densities are never
// -0.0): comparisons and reductions run on the integer pipes, not FP64.
__device__ __forceinline__ unsigned long long okey(double d) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(d);
  return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}

// Candidate (key, index) under "larger key wins, equal keys: larger index"
// (max-key / min-key keep the last of equal elements); arg-min searches
// complement the key.
struct Best {
  unsigned long long k;
  int i;
};
__device__ __forceinline__ Best better(Best a, Best b) {
  if (b.i < 0) return a;
  if (a.i < 0) return b;
  if (b.k > a.k || (b.k == a.k && b.i > a.i)) return b;
  return a;
}

// Block-wide reduction of each thread's candidate; all threads get the index.
__device__ int block_best(Best b, Best* red) {
  for (int o = 16; o > 0; o >>= 1) {
    Best c;
    c.k = __shfl_xor_sync(0xffffffffu, b.k, o);
    c.i = __shfl_xor_sync(0xffffffffu, b.i, o);
    b = better(b, c);
  }
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = b;
  __syncthreads();
  if (threadIdx.x < 32) {
    Best c = red[threadIdx.x];
    for (int o = 16; o > 0; o >>= 1) {
      Best e;
      e.k = __shfl_xor_sync(0xffffffffu, c.k, o);
      e.i = __shfl_xor_sync(0xffffffffu, c.i, o);
      c = better(c, e);
    }
    if (threadIdx.x == 0) red[32] = c;
  }
  __syncthreads();
  const int r = red[32].i;
  __syncthreads();  // red is reused by the next reduction
  return r;
}

__device__ __forceinline__ double weight(const double* table, int h, int dx, int dy) {
  return table[abs(dy) * h + abs(dx)];
}

// x - cx wrapped into [-m/2, m - m/2) (wrap, bluenoise.clj:72-76) for
// |x - cx| < m
__device__ __forceinline__ int wrap_near(int d, int m) {
  const int half = m >> 1;
  return d < -half ? d + m : d >= m - half ? d - m : d;
}

// The pixels of this thread, p = threadIdx.x + k * kBlueThreads, walked with
// their (x, y) so that the hot loop has no division.
struct Walk {
  int m, x0, y0, sx, sy;
  __device__ explicit Walk(int m_) : m(m_) {
    x0 = threadIdx.x % m_;
    y0 = threadIdx.x / m_;
    sx = kBlueThreads % m_;
    sy = kBlueThreads / m_;
  }
};

// Arg-extremum over pixels whose mask equals `want`, without changes: arg max
// of the density, or arg min when `least`.
__device__ int search(const double* density, const unsigned char* mask, int total, unsigned char want, bool least,
                      Best* red) {
  Best b{0ull, -1};
  for (int p = threadIdx.x; p < total; p += kBlueThreads)
    if (mask[p] == want) {
      const unsigned long long k = okey(density[p]);
      b = better(b, Best{least ? ~k : k, p});
    }
  return block_best(b, red);
}

// One step: mask[c] = mask_c and density-change (bluenoise.clj:99-109) by
// +/- the weight of every pixel's offset from c; in the same pass the
// arg-extremum of the next search over the updated pixels (mask == want).
__device__ int step(double* density, unsigned char* mask, const Walk& w, int total, const double* table, int c,
                    bool add, unsigned char mask_c, unsigned char want, bool least, Best* red) {
  const int m = w.m, h = (m >> 1) + 1, cy = c / m, cx = c - cy * m;
  Best b{0ull, -1};
  int x = w.x0, y = w.y0;
  for (int p = threadIdx.x; p < total; p += kBlueThreads) {
    if (p == c) mask[p] = mask_c;
    const double f = weight(table, h, wrap_near(x - cx, m), wrap_near(y - cy, m));
    const double d = add ? __dadd_rn(density[p], f) : __dsub_rn(density[p], f);
    density[p] = d;
    if (mask[p] == want) {
      const unsigned long long k = okey(d);
      b = better(b, Best{least ? ~k : k, p});
    }
    x += w.sx;
    y += w.sy;
    if (x >= m) {
      x -= m;
      y += 1;
    }
  }
  return block_best(b, red);
}

// density-array (bluenoise.clj:79-96) on every SM: pixel p sums the weights
// of the set pixels in row-major order, as density-sample does.  One warp
// per pixel row segment would reorder the sum; one thread per pixel keeps it.
__global__ void k_blue_density(int m, const double* __restrict__ table, const unsigned char* __restrict__ mask,
                               double* density) {
  extern __shared__ __align__(16) unsigned char dsm[];
  const int h = (m >> 1) + 1, total = m * m;
  double* tb = reinterpret_cast<double*>(dsm);
  unsigned char* mk = dsm + sizeof(double) * h * h;
  for (int t = threadIdx.x; t < h * h; t += blockDim.x) tb[t] = table[t];
  for (int t = threadIdx.x; t < total; t += blockDim.x) mk[t] = mask[t];
  __syncthreads();
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= total) return;
  const int cy = p / m, cx = p - cy * m;
  double s = 0.0;
  for (int y = 0; y < m; y++) {
    const int wy = wrap_near(y - cy, m);
    for (int x = 0; x < m; x++)
      if (mk[y * m + x]) s = __dadd_rn(s, weight(tb, h, wrap_near(x - cx, m), wy));
  }
  density[p] = s;
}

// State of the single-CTA kernels: the table always in shared memory, the
// density and a mask there too when they fit, else in global memory.
struct BlueState {
  double* table;
  double* density;
  unsigned char* mask;
};

__device__ BlueState blue_state(const BlueArgs& a, unsigned char* smem, double* g_density, unsigned char* g_mask) {
  const int m = a.m, total = m * m, h = (m >> 1) + 1;
  BlueState st;
  st.table = reinterpret_cast<double*>(smem);
  unsigned char* base = smem + sizeof(double) * h * h;
  st.density = a.use_smem ? reinterpret_cast<double*>(base) : g_density;
  st.mask = a.use_smem ? base + sizeof(double) * total : g_mask;
  for (int t = threadIdx.x; t < h * h; t += kBlueThreads) st.table[t] = a.table[t];
  return st;
}

// seed-pattern (bluenoise.clj:112-124) from a.mask with its density in
// a.density: remove the tightest cluster, add the largest void, until they
// coincide; the pattern is left in a.mask.
__global__ void __launch_bounds__(kBlueThreads, 1) k_blue_seed(BlueArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ Best red[33];
  const int m = a.m, total = m * m;
  const Walk w(m);
  BlueState st = blue_state(a, smem, a.density, a.mask);
  if (a.use_smem)
    for (int p = threadIdx.x; p < total; p += kBlueThreads) {
      st.density[p] = a.density[p];
      st.mask[p] = a.mask[p];
    }
  __syncthreads();
  int cluster = search(st.density, st.mask, total, 1, false, red);
  for (int it = 0; it < total * 4 && cluster >= 0; it++) {  // the pattern settles long before this bound
    const int vd = step(st.density, st.mask, w, total, st.table, cluster, false, 0, 0, true, red);
    if (vd < 0) break;  // cannot happen for 1 <= n <= m*m/2
    if (vd == cluster) {
      if (threadIdx.x == 0) st.mask[vd] = 1;
      break;
    }
    cluster = step(st.density, st.mask, w, total, st.table, vd, true, 1, 1, false, red);
  }
  __syncthreads();
  if (a.use_smem)
    for (int p = threadIdx.x; p < total; p += kBlueThreads) a.mask[p] = st.mask[p];
}

// dither-phase1 and dither-phase2 (bluenoise.clj:127-154), both from the
// seed pattern a.mask and its density a.density0: ranks n-1 .. 0 for the
// removed clusters, n .. m*m/2 - 1 for the filled voids.  The complement of
// the half-filled pattern is left in a.work for phase 3.
__global__ void __launch_bounds__(kBlueThreads, 1) k_blue_phases(BlueArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ Best red[33];
  const int m = a.m, total = m * m;
  const Walk w(m);
  BlueState st = blue_state(a, smem, a.density, a.work);
  for (int p = threadIdx.x; p < total; p += kBlueThreads) {
    st.mask[p] = a.mask[p];
    st.density[p] = a.density0[p];
  }
  __syncthreads();
  int c = search(st.density, st.mask, total, 1, false, red);
  for (int r = a.n; r > 0 && c >= 0; r--) {
    if (threadIdx.x == 0) a.dither[c] = r - 1;
    c = step(st.density, st.mask, w, total, st.table, c, false, 0, 1, false, red);
  }
  __syncthreads();
  for (int p = threadIdx.x; p < total; p += kBlueThreads) {
    st.mask[p] = a.mask[p];
    st.density[p] = a.density0[p];
  }
  __syncthreads();
  c = search(st.density, st.mask, total, 0, true, red);
  for (int r = a.n; r < total / 2 && c >= 0; r++) {
    if (threadIdx.x == 0) a.dither[c] = r;
    c = step(st.density, st.mask, w, total, st.table, c, true, 1, 0, true, red);
  }
  __syncthreads();
  for (int p = threadIdx.x; p < total; p += kBlueThreads) a.work[p] = !st.mask[p];
}

// dither-phase3 (bluenoise.clj:157-169) on the complement a.work with its
// density a.density: ranks m*m/2 .. m*m - 1 for the removed clusters.
__global__ void __launch_bounds__(kBlueThreads, 1) k_blue_phase3(BlueArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ Best red[33];
  const int m = a.m, total = m * m;
  const Walk w(m);
  BlueState st = blue_state(a, smem, a.density, a.work);
  if (a.use_smem)
    for (int p = threadIdx.x; p < total; p += kBlueThreads) {
      st.mask[p] = a.work[p];
      st.density[p] = a.density[p];
    }
  __syncthreads();
  int c = search(st.density, st.mask, total, 1, false, red);
  for (int r = total / 2; r < total && c >= 0; r++) {
    if (threadIdx.x == 0) a.dither[c] = r;
    c = step(st.density, st.mask, w, total, st.table, c, false, 0, 1, false, red);
  }
}

// ------------------------------------------- blue noise on a CTA cluster
//
// The same steps with the pixels split over a cluster of nc CTAs (8, or 16
// where the GPU can place such clusters and the table is large; one CTA per
// SM): each CTA keeps the density and mask of its m*m / nc pixels in shared
// memory and updates them; a step's arg-extremum is a block reduction per
// CTA, after which every CTA sends its candidate to every other (stores into
// their shared memory and a release-arrive on their mbarrier), and every
// warp of every CTA takes the best of the nc candidates.  All reduce the same
// candidates, and the order is total, so they pick the same pixel and take
// the same branches.  The candidates of step s sit in buffer s & 1:
// no CTA can be a whole step ahead of another, as a step ends only after
// every CTA's candidate for it has arrived.  Waits are bounded: a CTA that
// gives up records the error, and the others then give up too, as its
// candidates stop coming; all meet at the final cluster barrier.

constexpr int kBlueClusterMax = 16;
constexpr int kBlueCThreads = 512;

struct BlueCluster {
  int m, total, own, p0, rank, nc;  // pixels [p0, p0 + own) are this CTA's, of nc CTAs
  double* table;
  double* density;
  unsigned char* mask;
  Best (*slot)[kBlueClusterMax];  // [2][nc] candidates by step parity
  uint64_t* bar;                // [2]
  Best* red;                    // [2][33] reduction scratch by step parity
  int* fail;                    // shared flag: a wait gave up
  int step;
  int wait_limit;
};

__device__ __forceinline__ uint32_t cl_smem(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ uint32_t cl_map(uint32_t addr, int rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(addr), "r"(rank));
  return r;
}
__device__ __forceinline__ void cl_sync() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// The best candidate of the whole cluster; every thread gets its index, or
// -1 when a wait gave up (then every later step returns -1 at once).  Warp 0
// exchanges and reduces the candidates and the block barrier after it hands
// every thread the same answer, so the CTA takes one branch even when a wait
// gives up.  The reduction scratch alternates by step parity, so no second
// barrier is needed before the next step writes it.
__device__ int cluster_best(BlueCluster& c, Best b) {
  const int buf = c.step & 1, lane = threadIdx.x & 31;
  Best* red = c.red + 33 * buf;
  for (int o = 16; o > 0; o >>= 1) {
    Best e;
    e.k = __shfl_xor_sync(0xffffffffu, b.k, o);
    e.i = __shfl_xor_sync(0xffffffffu, b.i, o);
    b = better(b, e);
  }
  if (lane == 0) red[threadIdx.x >> 5] = b;
  __syncthreads();
  if (threadIdx.x < 32) {
    Best e = lane < (int)(blockDim.x >> 5) ? red[lane] : Best{0ull, -1};
    for (int o = 16; o > 0; o >>= 1) {
      Best f;
      f.k = __shfl_xor_sync(0xffffffffu, e.k, o);
      f.i = __shfl_xor_sync(0xffffffffu, e.i, o);
      e = better(e, f);
    }
    // every lane holds the CTA's candidate; lane r sends it to CTA r (slot
    // [buf][rank], then a release-arrive on its barrier [buf])
    const bool failed = *c.fail != 0;
    const uint32_t sb = cl_smem(&c.bar[buf]);
    if (!failed && lane < c.nc) {
      asm volatile("st.shared::cluster.u64 [%0], %1;" ::"r"(cl_map(cl_smem(&c.slot[buf][c.rank].k), lane)),
                   "l"(e.k)
                   : "memory");
      asm volatile("st.shared::cluster.u32 [%0], %1;" ::"r"(cl_map(cl_smem(&c.slot[buf][c.rank].i), lane)), "r"(e.i)
                   : "memory");
      asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(cl_map(sb, lane)) : "memory");
    }
    // all nc candidates of this step, then their best
    bool done = failed;
    if (!failed) {
      const uint32_t parity = (uint32_t)((c.step >> 1) & 1);
      for (int i = 0; i < c.wait_limit && !done; i++) {
        uint32_t ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.b32 %0, 1, 0, p;\n\t}"
            : "=r"(ok)
            : "r"(sb), "r"(parity)
            : "memory");
        done = ok != 0;
      }
    }
    const bool ok = __all_sync(0xffffffffu, done) && !failed;
    Best g = ok && lane < c.nc ? c.slot[buf][lane] : Best{0ull, -1};
    for (int o = kBlueClusterMax / 2; o > 0; o >>= 1) {
      Best f;
      f.k = __shfl_xor_sync(0xffffffffu, g.k, o);
      f.i = __shfl_xor_sync(0xffffffffu, g.i, o);
      g = better(g, f);
    }
    if (lane == 0) {
      if (!ok) *c.fail = 1;
      red[32] = ok ? g : Best{0ull, -1};
    }
  }
  __syncthreads();
  c.step++;
  return red[32].i;
}

// Arg-extremum over the cluster's pixels whose mask equals `want`.
__device__ int cluster_search(BlueCluster& c, unsigned char want, bool least) {
  Best b{0ull, -1};
  for (int q = threadIdx.x; q < c.own; q += blockDim.x)
    if (c.mask[q] == want) {
      const unsigned long long k = okey(c.density[q]);
      b = better(b, Best{least ? ~k : k, c.p0 + q});
    }
  return cluster_best(c, b);
}

// One step as `step` above on this CTA's pixels: mask[pc] = mask_c (by its
// owner) and the density change of every pixel by +/- the weight of its
// offset from pc, then the cluster's arg-extremum of the next search.
__device__ int cluster_step(BlueCluster& c, int pc, bool add, unsigned char mask_c, unsigned char want, bool least) {
  const int m = c.m, h = (m >> 1) + 1, cy = pc / m, cx = pc - cy * m;
  Best b{0ull, -1};
  const int first = c.p0 + threadIdx.x;
  int y = first / m, x = first - y * m;
  const int sy = blockDim.x / m, sx = blockDim.x - sy * m;
  for (int q = threadIdx.x; q < c.own; q += blockDim.x) {
    const int p = c.p0 + q;
    if (p == pc) c.mask[q] = mask_c;
    const double f = weight(c.table, h, wrap_near(x - cx, m), wrap_near(y - cy, m));
    const double d = add ? __dadd_rn(c.density[q], f) : __dsub_rn(c.density[q], f);
    c.density[q] = d;
    if (c.mask[q] == want) {
      const unsigned long long k = okey(d);
      b = better(b, Best{least ? ~k : k, p});
    }
    x += sx;
    y += sy;
    if (x >= m) {
      x -= m;
      y += 1;
    }
  }
  return cluster_best(c, b);
}

// Shared memory of a cluster CTA: the Gauss table, the CTA's densities and
// mask, the candidate slots, barriers and reduction scratch.
__host__ __device__ inline size_t blue_cluster_smem(int m, int nc) {
  const size_t h = (size_t)(m / 2 + 1), own = (size_t)m * m / nc;
  return ((sizeof(double) * (h * h + own) + own + 15) & ~size_t(15));
}

// Static part of a cluster CTA's shared memory.
struct BlueClusterShared {
  Best slot[2][kBlueClusterMax];
  uint64_t bar[2];
  Best red[2][33];
  int fail;
};

__device__ BlueCluster blue_cluster_setup(const BlueArgs& a, unsigned char* smem, BlueClusterShared& sh,
                                          const double* g_density, const unsigned char* g_mask) {
  BlueCluster c;
  c.m = a.m;
  c.total = a.m * a.m;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(c.rank));
  asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(c.nc));
  c.own = c.total / c.nc;
  c.p0 = c.rank * c.own;
  const int h = (a.m >> 1) + 1;
  c.table = reinterpret_cast<double*>(smem);
  c.density = c.table + h * h;
  c.mask = reinterpret_cast<unsigned char*>(c.density + c.own);
  c.slot = sh.slot;
  c.bar = sh.bar;
  c.red = &sh.red[0][0];
  c.fail = &sh.fail;
  c.step = 0;
  c.wait_limit = a.wait_limit;
  for (int t = threadIdx.x; t < h * h; t += blockDim.x) c.table[t] = a.table[t];
  for (int q = threadIdx.x; q < c.own; q += blockDim.x) {
    c.density[q] = g_density[c.p0 + q];
    c.mask[q] = g_mask[c.p0 + q];
  }
  if (threadIdx.x == 0) {
    sh.fail = 0;
    for (int b = 0; b < 2; b++)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(cl_smem(&sh.bar[b])), "r"(c.nc) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  // every CTA's barriers are initialised before any candidate is sent
  cl_sync();
  return c;
}

// The CTA's pixels of the mask back to `g_mask` (inverted when `invert`),
// then the final cluster barrier: no CTA leaves while another may still
// write into its shared memory; a wait that gave up is reported.
__device__ void blue_cluster_finish(const BlueArgs& a, BlueCluster& c, unsigned char* g_mask, bool invert) {
  __syncthreads();
  if (g_mask)
    for (int q = threadIdx.x; q < c.own; q += blockDim.x) g_mask[c.p0 + q] = invert ? !c.mask[q] : c.mask[q];
  if (threadIdx.x == 0 && *c.fail && a.error) atomicExch(a.error, 1);
  cl_sync();
}

__global__ void __launch_bounds__(kBlueCThreads, 1)
    k_blue_seed_cl(BlueArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ BlueClusterShared sh;
  BlueCluster c = blue_cluster_setup(a, smem, sh, a.density, a.mask);
  const int total = c.total;
  int cluster = cluster_search(c, 1, false);
  for (int it = 0; it < total * 4 && cluster >= 0; it++) {  // the pattern settles long before this bound
    const int vd = cluster_step(c, cluster, false, 0, 0, true);
    if (vd < 0) break;
    if (vd == cluster) {
      if (vd >= c.p0 && vd < c.p0 + c.own && threadIdx.x == 0) c.mask[vd - c.p0] = 1;
      break;
    }
    cluster = cluster_step(c, vd, true, 1, 1, false);
  }
  blue_cluster_finish(a, c, a.mask, false);
}

__global__ void __launch_bounds__(kBlueCThreads, 1)
    k_blue_phases_cl(BlueArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ BlueClusterShared sh;
  BlueCluster c = blue_cluster_setup(a, smem, sh, a.density0, a.mask);
  const int total = c.total;
  int pc = cluster_search(c, 1, false);
  for (int r = a.n; r > 0 && pc >= 0; r--) {
    if (c.rank == 0 && threadIdx.x == 0) a.dither[pc] = r - 1;
    pc = cluster_step(c, pc, false, 0, 1, false);
  }
  // back to the seed pattern and its density for phase 2
  __syncthreads();
  for (int q = threadIdx.x; q < c.own; q += blockDim.x) {
    c.density[q] = a.density0[c.p0 + q];
    c.mask[q] = a.mask[c.p0 + q];
  }
  __syncthreads();
  pc = cluster_search(c, 0, true);
  for (int r = a.n; r < total / 2 && pc >= 0; r++) {
    if (c.rank == 0 && threadIdx.x == 0) a.dither[pc] = r;
    pc = cluster_step(c, pc, true, 1, 0, true);
  }
  blue_cluster_finish(a, c, a.work, true);
}

__global__ void __launch_bounds__(kBlueCThreads, 1)
    k_blue_phase3_cl(BlueArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ BlueClusterShared sh;
  BlueCluster c = blue_cluster_setup(a, smem, sh, a.density, a.work);
  const int total = c.total;
  int pc = cluster_search(c, 1, false);
  for (int r = total / 2; r < total && pc >= 0; r++) {
    if (c.rank == 0 && threadIdx.x == 0) a.dither[pc] = r;
    pc = cluster_step(c, pc, false, 0, 1, false);
  }
  blue_cluster_finish(a, c, nullptr, false);
}

// scatter-mask (bluenoise.clj:39-43), first pass: clear the mask and the ranks
__global__ void k_blue_clear(int total, unsigned char* mask, int* dither) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= total) return;
  mask[t] = 0;
  dither[t] = 0;
}

// second pass: set the n seed pixels
__global__ void k_blue_seed_set(int n, const int* seed, unsigned char* mask) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) mask[seed[t]] = 1;
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
  const size_t all = table + (sizeof(double) + 1) * (size_t)m * m;
  *use_smem = all <= 200 * 1024;
  return *use_smem ? all : table;
}

// CTAs of the blue-noise cluster for an m x m table, 0 where the single-CTA
// kernels serve it.  The cluster kernels take tables whose pixels split
// evenly over the cluster, from 2048 pixels (below that one CTA's
// reductions are as fast), while a CTA's share, the Gauss table and the
// static part fit in 227 KB; 16 CTAs from 16384 pixels where the GPU can
// place such clusters (a non-portable size), else 8.
int blue_noise_cluster_size(int m) {
  const int total = m * m;
  auto fits = [&](int nc) {
    return total % nc == 0 && blue_cluster_smem(m, nc) + sizeof(BlueClusterShared) <= 227 * 1024;
  };
  if (total < 2048) return 0;
  if (total >= 16384 && fits(16)) {
    const size_t smem = blue_cluster_smem(m, 16);
    void (*kernels[3])(BlueArgs) = {k_blue_seed_cl, k_blue_phases_cl, k_blue_phase3_cl};
    bool ok = true;
    for (auto k : kernels) {
      ok = ok && cudaFuncSetAttribute(k, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess &&
           cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) == cudaSuccess;
      cudaLaunchConfig_t cfg = {};
      cudaLaunchAttribute attr;
      attr.id = cudaLaunchAttributeClusterDimension;
      attr.val.clusterDim.x = 16;
      attr.val.clusterDim.y = 1;
      attr.val.clusterDim.z = 1;
      cfg.gridDim = dim3(16);
      cfg.blockDim = dim3(kBlueCThreads);
      cfg.dynamicSmemBytes = smem;
      cfg.attrs = &attr;
      cfg.numAttrs = 1;
      int clusters = 0;
      ok = ok && cudaOccupancyMaxActiveClusters(&clusters, k, &cfg) == cudaSuccess && clusters >= 1;
    }
    cudaGetLastError();  // a refused query leaves no error behind
    if (ok) return 16;
  }
  return fits(8) ? 8 : 0;
}

int launch_blue_noise(int m, int n, const int* seed, double sigma, const double* table, double* density,
                      double* density0, unsigned char* mask, unsigned char* work, int* dither, int* error,
                      cudaStream_t st) {
  BlueArgs a;
  a.m = m;
  a.seed = seed;
  (void)sigma;  // the Gauss weights arrive in `table`
  a.n = n;
  a.table = table;
  a.density = density;
  a.density0 = density0;
  a.mask = mask;
  a.work = work;
  a.dither = dither;
  a.error = error;
  a.wait_limit = wait_limit();
  bool use = false;
  const size_t smem = blue_noise_smem(m, &use);
  a.use_smem = use ? 1 : 0;
  const int total = m * m, h = m / 2 + 1;
  const size_t dsmem = sizeof(double) * h * h + (size_t)total;
  if (dsmem > 220 * 1024) return -1;
  if (cudaFuncSetAttribute(k_blue_seed, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess ||
      cudaFuncSetAttribute(k_blue_phases, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess ||
      cudaFuncSetAttribute(k_blue_phase3, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess ||
      cudaFuncSetAttribute(k_blue_density, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dsmem) != cudaSuccess)
    return -1;
  const int nc = blue_noise_cluster_size(m);
  const size_t csmem = nc ? blue_cluster_smem(m, nc) : 0;
  if (nc && (cudaFuncSetAttribute(k_blue_seed_cl, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)csmem) !=
                 cudaSuccess ||
             cudaFuncSetAttribute(k_blue_phases_cl, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)csmem) !=
                 cudaSuccess ||
             cudaFuncSetAttribute(k_blue_phase3_cl, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)csmem) !=
                 cudaSuccess))
    return -1;
  // one cluster of nc CTAs
  auto on_cluster = [&](void (*k)(BlueArgs)) {
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr;
    attr.id = cudaLaunchAttributeClusterDimension;
    attr.val.clusterDim.x = nc;
    attr.val.clusterDim.y = 1;
    attr.val.clusterDim.z = 1;
    cfg.gridDim = dim3(nc);
    cfg.blockDim = dim3(kBlueCThreads);
    cfg.dynamicSmemBytes = csmem;
    cfg.stream = st;
    cfg.attrs = &attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k, a) == cudaSuccess;
  };
  const unsigned dblocks = (unsigned)((total + 255) / 256);
  // the seed mask, its density, the seed pattern, its density, phases 1-2,
  // the complement's density, phase 3
  k_blue_clear<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(total, mask, dither);
  k_blue_seed_set<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, seed, mask);
  k_blue_density<<<dblocks, 256, dsmem, st>>>(m, table, mask, density);
  if (nc) {
    if (!on_cluster(k_blue_seed_cl)) return -1;
  } else {
    k_blue_seed<<<1, kBlueThreads, smem, st>>>(a);
  }
  k_blue_density<<<dblocks, 256, dsmem, st>>>(m, table, mask, density0);
  if (nc) {
    if (!on_cluster(k_blue_phases_cl)) return -1;
  } else {
    k_blue_phases<<<1, kBlueThreads, smem, st>>>(a);
  }
  k_blue_density<<<dblocks, 256, dsmem, st>>>(m, table, work, density);
  if (nc) {
    if (!on_cluster(k_blue_phase3_cl)) return -1;
  } else {
    k_blue_phase3<<<1, kBlueThreads, smem, st>>>(a);
  }
  return 0;
}

}  // namespace sfsim
