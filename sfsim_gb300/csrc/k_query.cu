// k_query.cu -- queries of a built atmosphere at arbitrary points (the table
// lookups themselves live in k_lookup.cu):
//  * the rendered in-scatter S + M phase(mie, v.l) at (x, v, l) by direct
//    quadrature: the first order integrated at the point (atmosphere.clj:
//    154-200) plus ray scatter of the summed point-scatter tables;
//  * the surrogate's training pools and its fused tensor-core inference.
#include <cuda_bf16.h>

#include "atmo_device.cuh"
#include "kernels.h"
#include "tc.cuh"

namespace sfsim {

__device__ __forceinline__ unsigned long long hash64(unsigned long long z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

__device__ __forceinline__ double unit_uniform(unsigned long long h) { return (double)(h >> 11) * (1.0 / 9007199254740992.0); }

// Uniform direction on the sphere from two uniforms (z uniform in [-1, 1]).
__device__ __forceinline__ d3 sphere_direction(double u1, double u2) {
  const double z = 2.0 * u1 - 1.0, phi = 2.0 * 3.14159265358979323846 * u2;
  const double r = sqrt(dmax(0.0, 1.0 - z * z));
  return mk3(r * cos(phi), r * sin(phi), z);
}

// Random queries: height uniform in [0, H], position direction, view and sun
// uniform on the sphere.
__global__ void k_random_queries(long long n, unsigned long long seed, double R, double H, double* X, double* V,
                                 double* L) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= n) return;
  unsigned long long h = hash64(seed * 0x632BE59BD9B4E019ull + (unsigned long long)t);
  double u[7];
  for (int i = 0; i < 7; i++) {
    h = hash64(h);
    u[i] = unit_uniform(h);
  }
  const double r = R + H * u[0];
  const d3 p = sphere_direction(u[1], u[2]), v = sphere_direction(u[3], u[4]), l = sphere_direction(u[5], u[6]);
  X[3 * t] = r * p.x;
  X[3 * t + 1] = r * p.y;
  X[3 * t + 2] = r * p.z;
  V[3 * t] = v.x;
  V[3 * t + 1] = v.y;
  V[3 * t + 2] = v.z;
  L[3 * t] = l.x;
  L[3 * t + 1] = l.y;
  L[3 * t + 2] = l.z;
}

void launch_random_queries(long long n, unsigned long long seed, double R, double H, double* x, double* v, double* l,
                           cudaStream_t st) {
  k_random_queries<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, seed, R, H, x, v, l);
}

// Training pool of the table nodes: coordinates node / (size - 1) with a zero
// correction, since the lookup reproduces the stored value at a node.  The
// sun elevation inverts core/sun-elevation-to-index.glsl.
__global__ void k_node_pool(BuildDims d, float* pool) {
  const long long node = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (node >= d.n4()) return;
  float* o = pool + kPoolRow * node;
  o[0] = (float)(node / ((long long)d.n3 * d.n2 * d.n1)) / (d.n0 - 1);
  o[1] = (float)((node / ((long long)d.n3 * d.n2)) % d.n1) / (d.n1 - 1);
  o[2] = (float)((node / d.n3) % d.n2) / (d.n2 - 1);
  o[3] = (float)(node % d.n3) / (d.n3 - 1);
  const float sin_el = -(logf(1.0f - o[2] * (1.0f - expf(-3.6f))) + 0.6f) / 3.0f;
  o[4] = fminf(fmaxf(0.5f * (1.0f + sin_el), 0.0f), 1.0f);
  o[5] = o[1] > 0.5f ? 1.0f : 0.0f;
  for (int c = 0; c < kMlpPhases; c++) o[kMlpSmooth + c] = 0.0f;  // a node sits on a cell corner
  for (int c = 0; c < 3; c++) o[kMlpCoords + c] = 0.0f;
}

void launch_node_pool(const BuildDims& d, float* pool, cudaStream_t st) {
  k_node_pool<<<(unsigned)((d.n4() + 255) / 256), 256, 0, st>>>(d, pool);
}

// pool rows (coords, log(value + eps) - log(table + eps)) from coordinates,
// directly integrated values and the table lookups at the same queries
__global__ void k_make_pool(long long n, const float* coords, const float* values, const float* table, float eps,
                            float* pool) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= n) return;
  for (int c = 0; c < kMlpCoords; c++) pool[kPoolRow * t + c] = coords[kMlpCoords * t + c];
  for (int c = 0; c < 3; c++)
    pool[kPoolRow * t + kMlpCoords + c] =
        logf(fmaxf(values[3 * t + c], 0.0f) + eps) - logf(fmaxf(table[3 * t + c], 0.0f) + eps);
}

void launch_make_pool(long long n, const float* coords, const float* values, const float* table, float eps,
                      float* pool, cudaStream_t st) {
  k_make_pool<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, coords, values, table, eps, pool);
}

// ---------------------------------------------------------------------------
// Direct quadrature of the rendered in-scatter at (x, v, l)
// ---------------------------------------------------------------------------

// Elevation coordinate (atmosphere.clj:239-253) at a sample p of the ray
// x + t v in FP32.  (p.v)^2 - (|p|^2 - R^2) = R^2 - d^2 and
// (p.v)^2 - (|p|^2 - R^2) + H^2 = top^2 - d^2 with d the distance of the line
// from the centre, so both square roots are per-ray constants taken in FP64;
// the differences that cancel are rewritten with them.
__device__ __forceinline__ float elevation_coordinate_f(float q, float pv, float root_top, float root_gnd, float Hh,
                                                        bool above) {
  const float rho = sqrtf(fmaxf(q, 0.0f));
  if (above) {
    const float a = (pv > 0 && root_top > 0) ? (q - Hh * Hh) / (pv + root_top) : pv - root_top;
    return 0.5f - limit_quot_f(a, rho + rho + 2 * Hh, -0.5f, 0.0f);
  }
  const float a = (pv < 0 && root_gnd > 0) ? q / (pv - root_gnd) : pv + root_gnd;
  return 0.5f + limit_quot_f(a, rho + rho, -0.5f, 0.0f);
}

// The FP64 part of one query's view ray (atmosphere.clj:192-198), computed
// by one lane: GB300 runs FP64 at a small fraction of the FP32 rate, so a
// warp sets up 32 queries side by side before it integrates them one by one.
struct QueryRay {
  double x[3], D[3], l[3];  // for the FP64 horizon test near the horizon
  long long qi;
  float root_top, root_gnd, c0, two_xD, DD, b0, Dl, mu, L, xv, s3;
  int u3, above;
};

template <int WARPS, bool LIST>
__global__ void __launch_bounds__(WARPS * 32, 2) k_query_direct(const AtmoParams* params, BuildDims d,
                                                                const Vec4<float>* Jsum, long long n, const double* X,
                                                                const double* V, const double* Lt, float* out,
                                                                const long long* indices) {
  __shared__ QueryRay rays[WARPS][32];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long base = (blockIdx.x * (long long)WARPS + warp) * 32;
  if (base >= n) return;
  const AtmoParams& P = params[0];
  const int S = d.S;
  if (base + lane < n) {
    const long long qi = LIST ? indices[base + lane] : base + lane;
    const d3 x = mk3(X[3 * qi], X[3 * qi + 1], X[3 * qi + 2]);
    const d3 v = mk3(V[3 * qi], V[3 * qi + 1], V[3 * qi + 2]);
    const d3 l = mk3(Lt[3 * qi], Lt[3 * qi + 1], Lt[3 * qi + 2]);
    const int above = is_above_horizon(P, x, v);
    const d3 e = above ? atmosphere_intersection(P, x, v) : surface_intersection(P, x, v);
    const d3 D = sub3(e, x);
    const double xr = mag3(x);
    const double xv = dot3(x, v);
    const double dperp2 = dsub(dot3(x, x), sqr(xv));  // squared distance of the line from the centre
    QueryRay& R = rays[warp][lane];
    R.x[0] = x.x, R.x[1] = x.y, R.x[2] = x.z;
    R.D[0] = D.x, R.D[1] = D.y, R.D[2] = D.z;
    R.l[0] = l.x, R.l[1] = l.y, R.l[2] = l.z;
    R.qi = qi;
    R.root_top = (float)sqrt(dmax(0.0, dsub(P.top2, dperp2)));
    R.root_gnd = (float)sqrt(dmax(0.0, dsub(P.R2, dperp2)));
    R.c0 = (float)dmul(dsub(xr, P.R), dadd(xr, P.R));
    R.two_xD = (float)(2.0 * dot3(x, D));
    R.DD = (float)dot3(D, D);
    R.b0 = (float)dot3(x, l);
    R.Dl = (float)dot3(D, l);
    R.mu = (float)dot3(v, l);
    R.L = (float)mag3(D);
    R.xv = (float)xv;
    R.above = above;
    split_coord_r<float>(0.5f * (d.n3 - 1) * (1 + R.mu), d.n3, &R.u3, &R.s3);
  }
  __syncwarp();
  const float Hh = P.f_Hh, Hh2 = P.f_Hh2;
  const float* hp = P.f_hpoly;
  const float* hr = P.f_hpr4;
  const float scale2 = Bulk<float>::sun_scale(d);
  const PhaseCS<float> phase_ray(P.f_phR), phase_mie(P.f_phM);
  const int count = (int)(n - base < 32 ? n - base : 32);
  for (int k = 0; k < count; k++) {
    const QueryRay& R = rays[warp][k];
    const float fc0 = R.c0, two_xD = R.two_xD, DD = R.DD, b0 = R.b0, Dl = R.Dl, fL = R.L, fxv = R.xv;
    float accR[3] = {0, 0, 0}, accM[3] = {0, 0, 0}, accJ[3] = {0, 0, 0};
    for (int s = lane; s < S; s += 32) {
      const float su = (s + 0.5f) / S;
      // q and optical depth from x to p_s along the view ray
      const float q = fmaf(su, fmaf(su, DD, two_xD), fc0);
      float sr, sm;
      optical_sums_u<float, 5>(fc0, two_xD * su, DD * su * su, 1.0f / S, S, hp, P.f_alpha, P.f_beta, P.f_kr, P.f_km,
                               sr, sm);
      const float segL = fL * su / S;
      float taux[3];
#pragma unroll
      for (int c = 0; c < 3; c++) taux[c] = segL * (P.f_ray_ext[c] * sr + P.f_mie_ext[c] * sm);
      const float h = height_from_q<float, 5>(q, hp, P.f_alpha, P.f_beta);
      const float er = Bulk<float>::exp2(h * P.f_kr), em = Bulk<float>::exp2(h * P.f_km);
      // first order: the sun seen from p_s (atmosphere.clj:154-160)
      const float bp = fmaf(su, Dl, b0);
      bool lit = (bp >= 0.0f) || (bp * bp <= q);
      const float m = bp * bp - q;
      if ((bp < 4.0f) && (fabsf(m) < 1.0e8f || (bp > -4.0f && q < 1.0e8f))) {
        const double t = (0.5 + s) * (1.0 / S);
        const d3 p = add3(mk3(R.x[0], R.x[1], R.x[2]), mul3(mk3(R.D[0], R.D[1], R.D[2]), t));
        lit = is_above_horizon(P, p, mk3(R.l[0], R.l[1], R.l[2]));
      }
      if (lit) {
        const float ctop = q - Hh2;
        const float root = Bulk<float>::sqrt(fmaxf(bp * bp - ctop, 0.0f));
        float texit = bp >= 0.0f ? Bulk<float>::div(-ctop, bp + root) : root - bp;
        texit = fmaxf(texit, 0.0f);
        const float dt = texit / S;
        float tr, tm;
        sun_sums<float, 4>(q, bp, dt, S, hr, P.f_alpha, P.f_beta, P.f_hratio, tr, tm);
#pragma unroll
        for (int c = 0; c < 3; c++) {
          const float T = exp_neg(taux[c] + dt * (P.f_ray_ext[c] * tr + P.f_mie_ext[c] * tm));
          accR[c] = fmaf(T, er, accR[c]);
          accM[c] = fmaf(T, em, accM[c]);
        }
      }
      // higher orders: J summed over the orders at forward(p_s, v, l, above)
      if (Jsum) {
        const float pr = sqrtf(P.f_R * P.f_R + q);
        const float pv = fxv + su * fL;
        int u[4];
        float w[4];
        split_coord_r<float>((d.n0 - 1) * (sqrtf(fmaxf(q, 0.0f)) / Hh), d.n0, &u[0], &w[0]);
        split_coord_r<float>((d.n1 - 1) * elevation_coordinate_f(q, pv, R.root_top, R.root_gnd, Hh, R.above), d.n1,
                             &u[1], &w[1]);
        split_coord_r<float>(sun_elevation_index_r<float>(bp / pr, scale2), d.n2, &u[2], &w[2]);
        u[3] = R.u3;
        w[3] = R.s3;
        float jv[3];
        interp4<float>(Jsum, d, u, w, jv);
#pragma unroll
        for (int c = 0; c < 3; c++) accJ[c] = fmaf(exp_neg(taux[c]), jv[c], accJ[c]);
      }
    }
#pragma unroll
    for (int c = 0; c < 3; c++) {
      for (int o = 16; o > 0; o >>= 1) {
        accR[c] += __shfl_xor_sync(0xffffffffu, accR[c], o);
        accM[c] += __shfl_xor_sync(0xffffffffu, accM[c], o);
        accJ[c] += __shfl_xor_sync(0xffffffffu, accJ[c], o);
      }
    }
    if (lane == 0) {
      const float w = fL / S;
      const float phR = phase_ray(R.mu), phM = phase_mie(R.mu);
#pragma unroll
      for (int c = 0; c < 3; c++) {
        const float s1 = w * phR * P.f_srcR[c] * accR[c];
        const float m1 = w * P.f_srcM[c] * accM[c];
        out[3 * R.qi + c] = s1 + m1 * phM + w * accJ[c];
      }
    }
  }
}

void launch_query_direct(const AtmoParams* params, const BuildDims& d, const Vec4<float>* Jsum, long long n,
                         const double* x, const double* v, const double* l, float* out, cudaStream_t st,
                         const long long* indices) {
  if (n <= 0) return;
  constexpr int WARPS = 8;
  const unsigned blocks = (unsigned)((n + WARPS * 32 - 1) / (WARPS * 32));
  if (indices)
    k_query_direct<WARPS, true><<<blocks, WARPS * 32, 0, st>>>(params, d, Jsum, n, x, v, l, out, indices);
  else
    k_query_direct<WARPS, false><<<blocks, WARPS * 32, 0, st>>>(params, d, Jsum, n, x, v, l, out, nullptr);
}

// ---------------------------------------------------------------------------
// Fused surrogate inference on the tensor cores.
//
// The coordinates and the table value of each query come from the lookup
// kernel (k_query_coords) run just before.  A persistent CTA per SM then
// evaluates groups of 256 queries (two 128-row tiles A0, A1 of BF16
// activations, K-major core-matrix layout, 64 KB each).  Warps 0-7 own one
// query each per thread (warps 0-3 tile 0, 4-7 tile 1): they write the
// Fourier features, and after every layer read their row of the FP32
// accumulator from tensor memory (tcgen05.ld, the next 32 columns in flight
// while the current ones are processed), add the bias, apply SiLU and write
// the BF16 result back as the next layer's input; the last layer folds the
// 256 -> 4 head in.  The value is (table + eps) exp(r) - eps, and a query whose
// predicted squared error exp(s) exceeds threshold^2 is flagged for the direct
// quadrature.  The epilogue has 16 warps: two per group of 32 tensor-memory
// lanes of each tile, one for each half of the columns (the second adds its
// part of the head through shared memory).  Warp 16 is the producer: one thread
// streams the 32 weight chunks of a group (256 rows x 32 K, 16 KB each,
// pre-packed in the tensor cores' layout) through a five-stage shared-memory
// ring with bulk TMA copies, and issues the tcgen05.mma of both tiles on each
// chunk (one weight fetch serves 256 queries) into two 128 x 256 FP32
// accumulators in tensor memory (all 512 columns).  Stages are released by
// tcgen05.commit, layers handed over by two mbarriers (accumulator complete,
// activations written).  Every wait is bounded by the run-time poll limit
// (sfsim_atmo_set_wait_limit): on timeout the CTA records an error, lets its
// copies and MMAs drain and returns.
// ---------------------------------------------------------------------------

constexpr int kInferKC = 32;                                          // K per weight chunk
constexpr int kInferChunkBytes = kMlpHidden * kInferKC * 2;           // 16 KB
constexpr int kInferChunks0 = kMlpIn / kInferKC;                      // layer 0
constexpr int kInferChunksH = kMlpHidden / kInferKC;                  // hidden layers
constexpr int kInferChunks = kInferChunks0 + 3 * kInferChunksH;       // 32 per group
constexpr int kInferStages = 5;
constexpr int kInferTileBytes = 128 * kMlpHidden * 2;                 // 64 KB
constexpr int kInferEpilogueWarps = 16;  // 2 tiles x 4 lane quarters x 2 column halves
constexpr int kInferThreads = 32 * kInferEpilogueWarps + 32;
constexpr int kInferSmemRing = 2 * kInferTileBytes;
constexpr int kInferSmemBias = kInferSmemRing + kInferStages * kInferChunkBytes;
constexpr int kInferSmemHead = kInferSmemBias + 4 * kMlpHidden * 4;
constexpr int kInferSmemBar = kInferSmemHead + (kMlpOut * kMlpHidden + 4) * 4;  // W5 (4 x 256) and b5
constexpr int kInferSmemPart = kInferSmemBar + (2 * kInferStages + 3) * 8 + 16;  // head partial sums
constexpr int kInferSmem = kInferSmemPart + 256 * kMlpOut * 4;

size_t infer_packed_bytes() { return (size_t)kInferChunks * kInferChunkBytes; }

// Packs the BF16 hidden-layer weights W_l [256][in] into the chunk sequence
// the inference kernel streams: chunk c = (layer, 32-wide K slice), element
// (n, k) at byte (n / 8) * 512 + (k % 32 / 8) * 128 + (n % 8) * 16 + (k % 8) * 2.
// One thread moves 8 consecutive K of one row.
__global__ void k_pack_infer(const __nv_bfloat16* W0, const __nv_bfloat16* W1, const __nv_bfloat16* W2,
                             const __nv_bfloat16* W3, unsigned char* packed) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  constexpr int n0 = kMlpHidden * (kMlpIn / 8);
  constexpr int nh = kMlpHidden * (kMlpHidden / 8);
  if (t >= n0 + 3 * nh) return;
  int layer, r, K, chunk0;
  const __nv_bfloat16* W;
  if (t < n0) {
    layer = 0, r = t, K = kMlpIn, chunk0 = 0, W = W0;
  } else {
    layer = 1 + (t - n0) / nh, r = (t - n0) % nh, K = kMlpHidden;
    chunk0 = kInferChunks0 + (layer - 1) * kInferChunksH;
    W = layer == 1 ? W1 : layer == 2 ? W2 : W3;
  }
  const int n = r / (K / 8), k = (r % (K / 8)) * 8;
  const uint4 v = *reinterpret_cast<const uint4*>(W + (long long)n * K + k);
  unsigned char* dst = packed + (size_t)(chunk0 + k / kInferKC) * kInferChunkBytes + (n >> 3) * (kInferKC * 16) +
                       ((k % kInferKC) >> 3) * 128 + (n & 7) * 16;
  *reinterpret_cast<uint4*>(dst) = v;
}

struct InferArgs {
  long long n;
  const float* coords;          // [n][kMlpCoords]
  const float* table;           // [n][3], the lookup's value
  const unsigned char* packed;  // kInferChunks weight chunks
  const float* b[4];
  const float* W5;              // [kMlpOut][256]
  const float* b5;
  float* out;
  float log_var_limit;          // flag queries with s above this (2 log threshold), or +inf
  float eps;
  long long* list;              // indices (plus index_offset) of the flagged queries, or NULL
  long long index_offset;
  unsigned long long* count;    // flagged queries so far (also the next free slot of list)
  int* error;
  int wait_limit;               // polls per mbarrier wait
};

__device__ __forceinline__ float tanh_approx(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// Sines and cosines of pi 2 (k + 1) t for the 8 harmonics of a cell phase t,
// by the recurrences sin((k+1)a) = 2 cos(a) sin(ka) - sin((k-1)a) (and the
// same for cos), as 2 x 8 BF16 at K columns col0 .. col0 + 15.
__device__ __forceinline__ void write_phase_features(float t, unsigned char* A, int row, int col0) {
  float s[8], c[8];
  sincospif(2.0f * t, &s[0], &c[0]);
  const float c2 = c[0] + c[0];
  s[1] = c2 * s[0];
  c[1] = fmaf(c2, c[0], -1.0f);
#pragma unroll
  for (int k = 2; k < 8; k++) {
    s[k] = fmaf(c2, s[k - 1], -s[k - 2]);
    c[k] = fmaf(c2, c[k - 1], -c[k - 2]);
  }
#pragma unroll
  for (int q = 0; q < 2; q++) {
    uint32_t w[4];
#pragma unroll
    for (int j = 0; j < 4; j++) {
      const __nv_bfloat162 h = __floats2bfloat162_rn(s[4 * q + j], c[4 * q + j]);
      w[j] = *reinterpret_cast<const uint32_t*>(&h);
    }
    *reinterpret_cast<uint4*>(A + tc::tile_offset(row, col0 + 8 * q, kMlpHidden)) = make_uint4(w[0], w[1], w[2], w[3]);
  }
}

// Sines and cosines of pi f_k u for the 16 feature frequencies f_k = 2^(k/2):
// sincospi at f_0 and f_1, the rest by exact angle doubling
// (sin 2a = 2 sin a cos a, cos 2a = 1 - 2 sin^2 a), written as 4 x 8 BF16
// (sin, cos pairs in k order) at K columns col0 .. col0 + 31 of row `row`.
__device__ __forceinline__ void write_features(float u, unsigned char* A, int row, int col0) {
  float s[16], c[16];
  sincospif(u, &s[0], &c[0]);
  sincospif(kFeatureSqrt2 * u, &s[1], &c[1]);
#pragma unroll
  for (int k = 2; k < 16; k++) {
    const float ss = s[k - 2] + s[k - 2];
    s[k] = ss * c[k - 2];
    c[k] = fmaf(-ss, s[k - 2], 1.0f);
  }
#pragma unroll
  for (int q = 0; q < 4; q++) {
    uint32_t w[4];
#pragma unroll
    for (int j = 0; j < 4; j++) {
      const __nv_bfloat162 h = __floats2bfloat162_rn(s[4 * q + j], c[4 * q + j]);
      w[j] = *reinterpret_cast<const uint32_t*>(&h);
    }
    *reinterpret_cast<uint4*>(A + tc::tile_offset(row, col0 + 8 * q, kMlpHidden)) = make_uint4(w[0], w[1], w[2], w[3]);
  }
}

// Producer thread: weight chunks through the ring, MMAs of both tiles.
__device__ __forceinline__ void infer_producer(const InferArgs& g, long long my_groups, unsigned char* smem, uint32_t tmem,
                               uint64_t* full, uint64_t* empty, uint64_t* acc_bar, uint64_t* act_bar,
                               volatile int* abort_flag) {
  unsigned char* ring = smem + kInferSmemRing;
  const long long total = my_groups * kInferChunks;
  long long issued = 0, c = 0;
  auto issue = [&](long long k) {
    const int s = (int)(k % kInferStages);
    tc::mbar_expect_tx(&full[s], kInferChunkBytes);
    tc::bulk_g2s(ring + s * kInferChunkBytes, g.packed + (size_t)(k % kInferChunks) * kInferChunkBytes,
                 kInferChunkBytes, &full[s]);
  };
  for (; issued < total && issued < kInferStages; issued++) issue(issued);
  const uint32_t idesc = tc::idesc_bf16(128, kMlpHidden);
  const uint32_t a_base = tc::smem_u32(smem), w_base = tc::smem_u32(ring);
  uint32_t act_phase = 0;
  bool ok = true;
  for (long long gi = 0; gi < my_groups && ok; gi++) {
    for (int layer = 0; layer < 4 && ok; layer++) {
      ok = tc::mbar_wait(act_bar, act_phase & 1, g.wait_limit) && !*abort_flag;
      act_phase++;
      if (!ok) break;
      tc::fence_after();
      const int nk = layer == 0 ? kInferChunks0 : kInferChunksH;
      for (int j = 0; j < nk; j++, c++) {
        const int s = (int)(c % kInferStages);
        if (!(ok = tc::mbar_wait(&full[s], (uint32_t)((c / kInferStages) & 1), g.wait_limit))) break;
        tc::fence_after();
        const uint32_t w0 = w_base + s * kInferChunkBytes;
#pragma unroll
        for (int tile = 0; tile < 2; tile++) {
          const uint32_t a0 = a_base + tile * kInferTileBytes + j * (kInferKC / 8) * 128;
#pragma unroll
          for (int ks = 0; ks < kInferKC / 16; ks++)
            tc::mma(tmem + tile * kMlpHidden, tc::smem_desc(a0 + ks * 256, 128, kMlpHidden * 16),
                    tc::smem_desc(w0 + ks * 256, 128, kInferKC * 16), idesc, (j > 0 || ks > 0) ? 1u : 0u);
        }
        tc::commit(&empty[s]);
        if (c >= 1 && issued < total) {  // refill the stage of the previous chunk
          const long long p = c - 1;
          if (!(ok = tc::mbar_wait(&empty[p % kInferStages], (uint32_t)((p / kInferStages) & 1), g.wait_limit)))
            break;
          issue(issued++);
        }
      }
      if (ok) tc::commit(acc_bar);
    }
  }
  if (!ok) {
    *abort_flag = 1;
    if (g.error) atomicExch(g.error, 1);
    // let the copies in flight land and the issued MMAs finish before the CTA leaves
    for (long long k = c; k < issued; k++)
      tc::mbar_wait(&full[k % kInferStages], (uint32_t)((k / kInferStages) & 1), g.wait_limit);
    if (c >= 1) tc::mbar_wait(&empty[(c - 1) % kInferStages], (uint32_t)(((c - 1) / kInferStages) & 1), g.wait_limit);
  }
}

__global__ void __launch_bounds__(kInferThreads, 1) k_surrogate_infer(InferArgs g) {
  extern __shared__ __align__(1024) unsigned char smem[];
  float* s_bias = reinterpret_cast<float*>(smem + kInferSmemBias);  // 0.5 b_l, 4 x 256
  float* s_w5 = reinterpret_cast<float*>(smem + kInferSmemHead);    // W5 [4][256], then b5
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + kInferSmemBar);
  uint64_t* empty = full + kInferStages;
  uint64_t* acc_bar = empty + kInferStages;
  uint64_t* act_bar = acc_bar + 1;
  uint64_t* head_bar = act_bar + 1;  // the second column half's head parts are in s_part
  float* s_part = reinterpret_cast<float*>(smem + kInferSmemPart);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(head_bar + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  const long long ngroups = (g.n + 255) / 256;
  const long long my_groups = blockIdx.x < ngroups ? (ngroups - 1 - blockIdx.x) / gridDim.x + 1 : 0;

#pragma unroll
  for (int layer = 0; layer < 4; layer++)  // constant indices keep the kernel parameters out of local memory
    for (int i = t; i < kMlpHidden; i += kInferThreads) s_bias[layer * kMlpHidden + i] = 0.5f * g.b[layer][i];
  for (int i = t; i < kMlpOut * kMlpHidden; i += kInferThreads) s_w5[i] = g.W5[i];
  if (t < kMlpOut) s_w5[kMlpOut * kMlpHidden + t] = g.b5[t];
  if (warp == 0) tc::tmem_alloc(tmem_slot, 2 * kMlpHidden);
  if (t == 0) {
    for (int s = 0; s < kInferStages; s++) {
      tc::mbar_init(&full[s], 1);
      tc::mbar_init(&empty[s], 1);
    }
    tc::mbar_init(acc_bar, 1);
    tc::mbar_init(act_bar, 32 * kInferEpilogueWarps);
    tc::mbar_init(head_bar, 16 * kInferEpilogueWarps);
    *abort_flag = 0;
    tc::fence_mbar_init();
  }
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == kInferEpilogueWarps) {
    if (lane == 0) infer_producer(g, my_groups, smem, tmem, full, empty, acc_bar, act_bar, abort_flag);
    __syncwarp();
  } else {
    // warp w: tensor-memory lanes 32 (w % 4) .., tile (w / 4) % 2, column half w / 8
    const int tile = (warp >> 2) & 1, half = warp >> 3, row = (warp & 3) * 32 + lane;
    const int col0 = half * (kMlpHidden / 2);
    unsigned char* A = smem + tile * kInferTileBytes;
    const uint32_t trow = tmem + ((uint32_t)((warp & 3) * 32) << 16) + (uint32_t)(tile * kMlpHidden + col0);
    float* part = s_part + (tile * 128 + row) * kMlpOut;
    uint32_t acc_phase = 0, head_phase = 0;
    bool ok = true;
    for (long long gi = 0; gi < my_groups && ok; gi++) {
      const long long q = (blockIdx.x + gi * gridDim.x) * 256 + tile * 128 + row;
      const bool valid = q < g.n;
      const long long qq = valid ? q : g.n - 1;
      // the features of a row split between its two threads: smooth
      // coordinates 0-3, and smooth 4-5 with the four phases
      if (half == 0) {
#pragma unroll
        for (int dd = 0; dd < 4; dd++) write_features(g.coords[kMlpCoords * qq + dd], A, row, 32 * dd);
      } else {
#pragma unroll
        for (int dd = 4; dd < kMlpSmooth; dd++) write_features(g.coords[kMlpCoords * qq + dd], A, row, 32 * dd);
#pragma unroll
        for (int dd = 0; dd < kMlpPhases; dd++)
          write_phase_features(g.coords[kMlpCoords * qq + kMlpSmooth + dd], A, row, 32 * kMlpSmooth + 16 * dd);
      }
      tc::fence_async_smem();
      tc::fence_before();
      tc::mbar_arrive(act_bar);
      float head[kMlpOut] = {};
      for (int layer = 0; layer < 4; layer++) {
        bool done = tc::mbar_wait(acc_bar, acc_phase & 1, g.wait_limit);
        acc_phase++;
        if (!__all_sync(0xffffffffu, done) || *abort_flag) {
          ok = false;
          break;
        }
        tc::fence_after();
        const float* hb = s_bias + layer * kMlpHidden;
        uint32_t rb[2][32];
        tc::tmem_ld32_async(trow, rb[0]);
        tc::tmem_wait_ld(rb[0]);
        constexpr int kBlocks = kMlpHidden / 2 / 32;
#pragma unroll
        for (int blk = 0; blk < kBlocks; blk++) {
          if (blk + 1 < kBlocks) tc::tmem_ld32_async(trow + (uint32_t)(32 * (blk + 1)), rb[(blk + 1) & 1]);
          const uint32_t* r = rb[blk & 1];
#pragma unroll
          for (int i8 = 0; i8 < 4; i8++) {
            const int n0 = col0 + 32 * blk + 8 * i8;
            const float4 b0 = *reinterpret_cast<const float4*>(hb + n0);
            const float4 b1 = *reinterpret_cast<const float4*>(hb + n0 + 4);
            const float bb[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
            uint32_t w[4];
            float hv[8];
#pragma unroll
            for (int j = 0; j < 8; j += 2) {
              // SiLU(z) = z sigmoid(z) = hz (1 + tanh hz) with hz = z / 2
              const float h0 = fmaf(0.5f, __uint_as_float(r[8 * i8 + j]), bb[j]);
              const float h1 = fmaf(0.5f, __uint_as_float(r[8 * i8 + j + 1]), bb[j + 1]);
              const __nv_bfloat162 hh =
                  __floats2bfloat162_rn(fmaf(h0, tanh_approx(h0), h0), fmaf(h1, tanh_approx(h1), h1));
              w[j / 2] = *reinterpret_cast<const uint32_t*>(&hh);
              hv[j] = __low2float(hh);
              hv[j + 1] = __high2float(hh);
            }
            if (layer < 3) {
              *reinterpret_cast<uint4*>(A + tc::tile_offset(row, n0, kMlpHidden)) = make_uint4(w[0], w[1], w[2], w[3]);
            } else {
#pragma unroll
              for (int cc = 0; cc < kMlpOut; cc++) {
                const float4 w0 = *reinterpret_cast<const float4*>(s_w5 + cc * kMlpHidden + n0);
                const float4 w1 = *reinterpret_cast<const float4*>(s_w5 + cc * kMlpHidden + n0 + 4);
                head[cc] = fmaf(hv[0], w0.x, fmaf(hv[1], w0.y, fmaf(hv[2], w0.z, fmaf(hv[3], w0.w, head[cc]))));
                head[cc] = fmaf(hv[4], w1.x, fmaf(hv[5], w1.y, fmaf(hv[6], w1.z, fmaf(hv[7], w1.w, head[cc]))));
              }
            }
          }
          if (blk + 1 < kBlocks) tc::tmem_wait_ld(rb[(blk + 1) & 1]);
        }
        if (layer < 3) {
          tc::fence_async_smem();
          tc::fence_before();
          tc::mbar_arrive(act_bar);
        }
      }
      if (!ok) break;
      // the head: the second half hands its partial sums to the first
      if (half == 1) {
#pragma unroll
        for (int cc = 0; cc < kMlpOut; cc++) part[cc] = head[cc];
        tc::mbar_arrive(head_bar);
        continue;
      }
      {
        const bool done = tc::mbar_wait(head_bar, head_phase & 1, g.wait_limit);
        head_phase++;
        if (!__all_sync(0xffffffffu, done) || *abort_flag) {
          ok = false;
          break;
        }
#pragma unroll
        for (int cc = 0; cc < kMlpOut; cc++) head[cc] += part[cc];
      }
      bool flag = false;
      if (valid) {
        const float tv[3] = {g.table[3 * q], g.table[3 * q + 1], g.table[3 * q + 2]};
#pragma unroll
        for (int cc = 0; cc < 3; cc++) {
          const float r = head[cc] + s_w5[kMlpOut * kMlpHidden + cc];
          g.out[3 * q + cc] = fmaxf((fmaxf(tv[cc], 0.0f) + g.eps) * expf(r) - g.eps, 0.0f);
        }
        flag = head[3] + s_w5[kMlpOut * kMlpHidden + 3] > g.log_var_limit;
      }
      if (g.count) {
        // one atomic per warp reserves the slots of its flagged queries
        const unsigned bal = __ballot_sync(0xffffffffu, flag);
        unsigned long long base = 0;
        if (lane == 0 && bal) base = atomicAdd(g.count, (unsigned long long)__popc(bal));
        base = __shfl_sync(0xffffffffu, base, 0);
        if (flag && g.list) g.list[base + __popc(bal & ((1u << lane) - 1u))] = g.index_offset + q;
      }
    }
    if (!ok) {
      *abort_flag = 1;
      if (lane == 0 && g.error) atomicExch(g.error, 1);
    }
  }
  tc::fence_before();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, 2 * kMlpHidden);
}

void launch_pack_infer(const __nv_bfloat16* const* W, unsigned char* packed, cudaStream_t st) {
  constexpr int nthreads = kMlpHidden * (kMlpIn / 8) + 3 * kMlpHidden * (kMlpHidden / 8);
  k_pack_infer<<<(nthreads + 255) / 256, 256, 0, st>>>(W[0], W[1], W[2], W[3], packed);
}

int launch_surrogate_infer(long long n, const float* coords, const float* table, const unsigned char* packed,
                           const float* const* b, const float* W5, const float* b5, float eps, float threshold,
                           float* out, long long* list, long long index_offset, unsigned long long* count, int* error,
                           int num_sms, cudaStream_t st) {
  InferArgs g;
  g.n = n;
  g.coords = coords;
  g.table = table;
  g.packed = packed;
  for (int i = 0; i < 4; i++) g.b[i] = b[i];
  g.W5 = W5;
  g.b5 = b5;
  g.out = out;
  g.log_var_limit = threshold > 0 ? 2.0f * logf(threshold) : INFINITY;
  g.eps = eps;
  g.list = list;
  g.index_offset = index_offset;
  g.count = count;
  g.error = error;
  g.wait_limit = wait_limit();
  if (cudaFuncSetAttribute(k_surrogate_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, kInferSmem) !=
      cudaSuccess)
    return -1;
  const long long groups = (n + 255) / 256;
  const unsigned grid = (unsigned)(groups < num_sms ? groups : num_sms);
  k_surrogate_infer<<<grid, kInferThreads, kInferSmem, st>>>(g);
  return 0;
}

}  // namespace sfsim
