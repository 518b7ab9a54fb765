// kernels.h -- host-side launchers of the atmosphere LUT build kernels.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "atmo_params.h"

namespace sfsim {

template <class Real>
struct SetupBuffers {
  Remap4<Real>* remapS;
  CellGeom<Real>* geom;
  Remap2<Real>* remapT;
  Remap2<Real>* remapE;
  RowInfo* rowinfo;
  Remap2<Real>* rowmap;  // [B][rows]: height and elevation coordinates of each view row
  RowSample<Real>* rows;
  SphereDir<Real>* sdirs;
  // sdirs partitioned per height row: the directions that end in the sky,
  // then those that end on the ground, each part filled to a multiple of
  // kDirBlock with zero-weight entries (pad = 1); kDirRow entries per row,
  // pcount = {first ground entry, entries used}
  SphereDir<Real>* pdirs;
  int2* pcount;
  // point scatter's shared-memory image of each height's partitioned
  // directions (dir_image_bytes per height): the fields as arrays, then uE0
  unsigned char* dimage;
  PointRow<Real>* prow;  // [B][n0][n2]
  double* hdvs;          // [n3]: 2 a / (n3 - 1) - 1, index-to-sun-direction's v.l of heading a
  SurfRow<Real>* erow;   // [B][nE0][nE1]
  HalfDir<Real>* hdir;   // [B][nE0][Ph]
};

constexpr int kDirBlock = 8;
__host__ __device__ constexpr int dir_row(int P) { return P + 2 * kDirBlock; }

// Fields per direction in point scatter's shared direction arrays: x0, x1,
// x2, weight, tR, ground0..2, sE0 (then uE0 as ints).
constexpr int kDirFields = 9;
// Bytes of the direction image of `used` directions, a multiple of 16.
__host__ __device__ inline size_t dir_image_bytes(int used, size_t real_size) {
  return ((size_t)used * (kDirFields * real_size + sizeof(int)) + 15) & ~size_t(15);
}
// Room per height in the global images: the most partitioned directions.
__host__ __device__ inline size_t dir_image_stride(const BuildDims& d, size_t real_size) {
  return dir_image_bytes((dir_row(d.P) + 7) / 8 * 8, real_size);
}

// Reals of one (height, sun elevation) pair's heading rows in point
// scatter's global row table: the dS and Mie rows of every partitioned
// direction, n3 + 2 RGB texels each; a multiple of 48.
__host__ __device__ inline long long heading_rows_stride(const BuildDims& d) {
  return 2LL * ((dir_row(d.P) + 7) / 8 * 8) * (d.n3 + 2) * 3;
}

// The set-up tables in parts: the rows (row info and point rows), then the
// 4-D node maps with each node's light direction (remap4) and the view-row
// samples, which both read the rows but not each other, and the rest
// (remapT, remapE, sphere directions and their partition, surface rows, half
// directions).  launch_setup runs them all on one stream.
template <class Real>
void launch_setup_rows(const AtmoParams* params, const BuildDims& d, const SetupBuffers<Real>& o, cudaStream_t st);
template <class Real>
void launch_node_maps(const AtmoParams* params, const BuildDims& d, const SetupBuffers<Real>& o, cudaStream_t st);
template <class Real>
void launch_view_rows(const AtmoParams* params, const BuildDims& d, const SetupBuffers<Real>& o, cudaStream_t st);
// Returns the number of kernels it launched.
template <class Real>
int launch_setup_aux(const AtmoParams* params, const BuildDims& d, const DirLocal* dirs,
                     const DirLocal* half_dirs, const SetupBuffers<Real>& o, cudaStream_t st);
template <class Real>
void launch_setup(const AtmoParams* params, const BuildDims& d, const DirLocal* dirs,
                  const DirLocal* half_dirs, const SetupBuffers<Real>& o, cudaStream_t st);

template <class Real>
void launch_transmittance(const AtmoParams* params, const BuildDims& d, Vec4<Real>* T, cudaStream_t st);

template <class Real>
void launch_surface_base(const AtmoParams* params, const BuildDims& d, Vec4<Real>* E0, cudaStream_t st);

// First-order Rayleigh ray scatter and Mie strength (fused).  With `geom`
// NULL each block forms its cells' light directions from the point rows and
// the per-heading table (as k_remap4 does), so the launch needs the rows and
// the view-row samples but not the node maps.  -1 when its shared memory
// (first_order_smem: the row's samples, and the cells' geometry when
// `cells`) cannot be configured.
template <class Real>
size_t first_order_smem(const BuildDims& d, bool cells);
template <class Real>
int launch_first_order(const AtmoParams* params, const BuildDims& d, const RowInfo* rowinfo,
                       const RowSample<Real>* rows, const CellGeom<Real>* geom, const PointRow<Real>* prow,
                       const double* hdvs, const unsigned char* sun_table, Vec4<Real>* rayleigh, Vec4<Real>* mie,
                       cudaStream_t st);

// Sun-ray optical-depth tables of the FP32 first order, per atmosphere: the
// climbing rays' kSunNR x kSunNM float2, then the descending rays' kDescNX x
// kDescNY float2 (see k_first_order.cu).
constexpr int kSunNR = 2048;
constexpr int kSunNM = 2048;
constexpr int kDescNX = 1024;
constexpr int kDescNY = 2048;
constexpr long long kSunTableLen = (long long)kSunNR * kSunNM + (long long)kDescNX * kDescNY;
// Bytes of the tables per atmosphere: the climbing table's rows, then the
// descending table's.  A table of paired texels holds (v(j), v(j + 1)) per
// entry, 16 bytes; otherwise v(j), 8 bytes.  Pairing the climbing table
// (most lookups) halves its L1 sectors; pairing the descending one too made
// the tables (96 MB) spill from L2 and gained nothing.
constexpr bool kSunPairClimb = true, kSunPairDesc = false;
constexpr size_t kSunClimbBytes = (size_t)kSunNR * kSunNM * (kSunPairClimb ? 16 : 8);
constexpr size_t kSunDescBytes = (size_t)kDescNX * kDescNY * (kSunPairDesc ? 16 : 8);
constexpr size_t kSunTableBytes = kSunClimbBytes + kSunDescBytes;
void launch_sun_table(const AtmoParams* params, const BuildDims& d, unsigned char* table, cudaStream_t st);

template <class Real>
void launch_first_order_census(const AtmoParams* params, const BuildDims& d, const RowInfo* rowinfo,
                               const RowSample<Real>* rows, const CellGeom<Real>* geom, unsigned long long* count,
                               cudaStream_t st);

// Throughput probe of the SFU: `iters` ex2.approx per chain, 8 chains per thread.
void launch_sfu_probe(int blocks, int threads, int iters, float* sink, cudaStream_t st);
// Throughput probe of shared-memory reads: blocks of 1024 threads, each
// reading `iters` x 8 16-byte words.
int launch_smem_probe(int blocks, int iters, float* sink, cudaStream_t st);

// J = point scatter of (dS, dE), planar [atmosphere][channel][node]; when
// `mie` is non-NULL dS is the first iteration's rayleigh + mie * phase(mie, v.l).
// hrows: scratch for the heading rows, B * n0 * n2 * heading_rows_stride(d) Reals.
template <class Real>
int launch_point_scatter(const AtmoParams* params, const BuildDims& d, const RowInfo* rowinfo,
                         const SphereDir<Real>* pdirs, const unsigned char* dimage, const int2* pcount,
                         const PointRow<Real>* prow, const CellGeom<Real>* geom, const Vec4<Real>* dS,
                         const Vec4<Real>* mie, const Vec4<Real>* dE, Real* hrows, Real* J, cudaStream_t st);

// dE = surface radiance of dS (same first-iteration convention).
template <class Real>
void launch_surface_radiance(const AtmoParams* params, const BuildDims& d, const SurfRow<Real>* erow,
                             const HalfDir<Real>* hdir, const Vec4<Real>* dS, const Vec4<Real>* mie,
                             Vec4<Real>* dE, cudaStream_t st);

// dS = ray scatter of J (planar [atmosphere][channel][node]).
template <class Real>
int launch_ray_scatter(const AtmoParams* params, const BuildDims& d, const RowInfo* rowinfo,
                       const RowSample<Real>* rows, const CellGeom<Real>* geom, const Remap4<Real>* remap,
                       const Real* J, Vec4<Real>* dS, cudaStream_t st);

// out = re-interpolation of (a + b) at the node maps; b may be NULL and, for
// the 2-D variant, a may be NULL.
template <class Real>
void launch_accumulate4(const BuildDims& d, const Remap4<Real>* remap, const Vec4<Real>* a, const Vec4<Real>* b,
                        Vec4<Real>* out, cudaStream_t st);

template <class Real>
void launch_accumulate2(int B, int n0, int n1, const Remap2<Real>* remap, const Vec4<Real>* a, const Vec4<Real>* b,
                        Vec4<Real>* out, cudaStream_t st);

// Final tables in the .scatter layout (float RGB, 4-D tables tiled 2-D).
template <class Real>
void launch_output4(const BuildDims& d, const Remap4<Real>* remap, const Vec4<Real>* tab, float* out,
                    cudaStream_t st);

template <class Real>
void launch_output2(int B, int n0, int n1, const Remap2<Real>* remap, const Vec4<Real>* tab, float* out,
                    cudaStream_t st);

// Tables of a built atmosphere as sfsim's shaders read them (.scatter layout).
struct QueryTables {
  float radius, max_height, mie_g;
  int t_height, t_elevation;
  int height, elevation, light, heading;
  const float* T;
  const float* S;
  const float* M;
};

// kind 0 transmittance_track(a, b), 1 transmittance_outer(a, b), 2
// ray_scatter_track(l, a, b), 3 ray_scatter_outer(l, a, b), 4 in-scatter at
// (a, b, l) with the horizon test choosing the table half.  Points [n][3].
void launch_query_table(const QueryTables& q, int kind, long long n, const float* a, const float* b, const float* l,
                        float* out, int weight_bits, cudaStream_t st);
void launch_query_attenuation(const QueryTables& q, int kind, long long n, const float* light, const float* p,
                              const float* d, const float* s, const float* incoming, float amplification, float* out,
                              int weight_bits, cudaStream_t st);

// Rendered in-scatter S + M phase(mie, v.l) at (x, v, l) by quadrature with
// the order-summed point-scatter table Jsum (NULL: first order only).
// With `indices`, warp w evaluates query indices[w] (n of them).
void launch_query_direct(const AtmoParams* params, const BuildDims& d, const Vec4<float>* Jsum, long long n,
                         const double* x, const double* v, const double* l, float* out, cudaStream_t st,
                         const long long* indices = nullptr);

// The surrogate's kMlpCoords coordinates of (x, v, l), the first four the
// table coordinates as the in-scatter lookup forms them; the lookup's value
// too when `table` is non-NULL.
void launch_query_coords(const QueryTables& q, long long n, const double* x, const double* v, const double* l,
                         float* coords, float* table, cudaStream_t st);
void launch_random_queries(long long n, unsigned long long seed, double R, double H, double* x, double* v, double* l,
                           cudaStream_t st);
void launch_node_pool(const BuildDims& d, float* pool, cudaStream_t st);
void launch_make_pool(long long n, const float* coords, const float* values, const float* table, float eps,
                      float* pool, cudaStream_t st);
// Fused tensor-core inference of the surrogate for n queries from their
// coordinates and table values (launch_query_coords); see k_query.cu.
int launch_surrogate_infer(long long n, const float* coords, const float* table, const unsigned char* packed,
                           const float* const* b, const float* W5, const float* b5, float eps, float threshold,
                           float* out, long long* list, long long index_offset, unsigned long long* count, int* error,
                           int num_sms, cudaStream_t st);
// Packs the BF16 hidden-layer weights into the inference kernel's chunks.
void launch_pack_infer(const __nv_bfloat16* const* W, unsigned char* packed, cudaStream_t st);
// Bytes of the packed weight chunks the inference kernel streams.
size_t infer_packed_bytes();

// jsum = (first ? 0 : jsum) + J, converted to float; J planar
// [atmosphere][channel][node] with n4 nodes per atmosphere.
template <class Real>
void launch_add_to_sum(long long n4, int B, const Real* J, Vec4<float>* jsum, bool first, cudaStream_t st);

// Float [atmosphere][node][channel] copy of a planar table.
template <class Real>
void launch_export_planar(long long n4, int B, const Real* tab, float* out, cudaStream_t st);

// Plain-order float copy of an internal table (debug intermediates).
template <class Real>
void launch_export(long long n, const Vec4<Real>* tab, float* out, cudaStream_t st);

// Tensor-core GEMM C[m][n] = alpha * sum_k A[m][k] B[n][k] (BF16 in, FP32
// accumulate) with the epilogue the surrogate MLP needs.  M any, N <= 256,
// K a multiple of 64 * splits; split > 1 only with the Cacc output.
// Poll limit of the tensor-core kernels' mbarrier waits: kDefaultWaitLimit
// unless sfsim_atmo_set_wait_limit changed it.
constexpr int kDefaultWaitLimit = 1 << 22;
int wait_limit();

struct GemmArgs {
  const __nv_bfloat16* A;
  long long lda;
  const __nv_bfloat16* B;
  long long ldb;
  int M, N;
  long long K;
  float alpha;
  const float* bias;  // [N] added after alpha, or NULL
  const float* row_bias;  // [groups][N] added by row: row_bias[row_group[m]][n], or NULL
  const int* row_group;   // [M] group of each row (with row_bias)
  const float* dact;  // [M][N] multiplier applied after the bias, or NULL
  float* Cf32;        // [M][ldc] or NULL
  long long ldc;
  float* Cacc;        // [M][ldc] accumulated with atomicAdd, or NULL
  float* Dsilu;       // SiLU'(z) [M][N], or NULL
  int silu;           // apply SiLU before the BF16 outputs
  __nv_bfloat16* Hbf16;   // [M][ldh] or NULL
  long long ldh;
  __nv_bfloat16* HTbf16;  // transposed [N][ldht] or NULL
  long long ldht;
  int* error;         // set to 1 when a wait times out
  int wait_limit;     // polls per mbarrier wait; 0: wait_limit()
  int stall_polls;    // > 0: self-test, the epilogue first waits this many polls on a barrier nothing arrives on
};

int launch_gemm_tn(const GemmArgs& g, int splits, cudaStream_t st);

// ---- surrogate MLP: 10 coordinates -> 256 Fourier features -> 4 x 256 SiLU -> 4 ----
// Coordinates in [0, 1]: the four table coordinates (height, elevation, sun
// elevation, sun heading), the sun elevation (1 + sin) / 2 without the
// table's clamp at sin = -0.2, 0 / 1 for the upper / lower table half, and
// the four cell phases: the position inside the table cell along each axis
// (frac(coordinate * (size - 1))), where the lookup's interpolation error
// repeats.  The six smooth coordinates get 16 frequencies 2^(k/2) each, the
// phases 8 harmonics 2 (k + 1) each (sin and cos of pi f u).
// Outputs: r_c (c < 3), the correction log(value_c + eps) - log(table_c + eps)
// to the table lookup, and s, the log of the expected squared error of r.
constexpr int kMlpSmooth = 6;
constexpr int kMlpPhases = 4;
constexpr int kMlpCoords = kMlpSmooth + kMlpPhases;
constexpr int kMlpIn = 32 * kMlpSmooth + 16 * kMlpPhases;
constexpr int kPoolRow = kMlpCoords + 3;  // floats per training sample: coordinates, corrections
constexpr int kMlpHidden = 256;
constexpr int kMlpLayers = 4;
constexpr int kMlpOut = 4;
// Feature frequencies f_k = 2^(k/2), k = 0..15: powers of two times 1 or the
// float nearest sqrt(2), so that doubling the angle steps k by two exactly.
constexpr float kFeatureSqrt2 = 1.41421356237309505f;
__host__ __device__ __forceinline__ float feature_frequency(int k) {
  return (k & 1 ? kFeatureSqrt2 : 1.0f) * (float)(1 << (k >> 1));
}
// Feature pair f (0 .. kMlpIn/2 - 1): its coordinate and its frequency.
__host__ __device__ __forceinline__ void feature_pair(int f, int* coord, float* freq) {
  if (f < 16 * kMlpSmooth) {
    *coord = f >> 4;
    *freq = feature_frequency(f & 15);
  } else {
    const int g = f - 16 * kMlpSmooth;
    *coord = kMlpSmooth + (g >> 3);
    *freq = (float)(2 * ((g & 7) + 1));
  }
}

void launch_features(long long n, const float* coords, __nv_bfloat16* F, __nv_bfloat16* FT, cudaStream_t st);
void launch_head_forward(long long n, const __nv_bfloat16* H, const float* W5, const float* b5, float* out,
                         cudaStream_t st);
// Loss: mean squared error of r (Huber with threshold `huber` when > 0) plus,
// weighted by `var_weight` in the gradients, the Gaussian negative
// log-likelihood of s given the squared error (which does not reach r).  The
// loss value is the mean squared error alone.
void launch_loss_grad(long long n, const float* out, const float* target, float huber, float var_weight, float* dout,
                      float* loss, cudaStream_t st);
void launch_head_backward(long long n, const float* dout, const __nv_bfloat16* H, const float* W5,
                          const float* dsilu, __nv_bfloat16* dZ, __nv_bfloat16* dZT, float* dW5, float* db5,
                          cudaStream_t st);
void launch_bias_grad(long long n, int width, const __nv_bfloat16* dZT, float* db, cudaStream_t st);
// The weight matrices whose BF16 copies (and transposes) an Adam step over
// the whole parameter vector refreshes: matrix k occupies [start, start +
// rows * cols) of the vector.
struct AdamMatrices {
  static constexpr int kMax = 4;
  int n;
  long long start[kMax];
  int rows[kMax], cols[kMax];
  __nv_bfloat16* wb[kMax];
  __nv_bfloat16* wbt[kMax];
};
void launch_adam_all(long long count, float* w, const float* g, float* m, float* v, float lr, float beta1, float beta2,
                     float eps, int step, const AdamMatrices& mats, cudaStream_t st);
void launch_adam(long long count, float* w, const float* g, float* m, float* v, float lr, float beta1, float beta2,
                 float eps, int step, int rows, int cols, __nv_bfloat16* wb, __nv_bfloat16* wbt, cudaStream_t st);
void launch_to_bf16(long long count, const float* w, int rows, int cols, __nv_bfloat16* wb, __nv_bfloat16* wbt,
                    cudaStream_t st);
void launch_gather_batch(long long n, unsigned long long seed, float node_frac, const float* poolA, long long na,
                         const float* poolB, long long nb, float* coords, float* target, cudaStream_t st);

// ---- conditioned surrogate: kCondInputs atmosphere inputs per group ----
// The inputs enter the first layer linearly: z1 = W1 F + b1 + U g, U
// [kMlpHidden][kCondInputs], so per group of rows (one atmosphere) U g is a
// constant row bias.
constexpr int kCondInputs = 8;
constexpr int kMaxCondGroups = 256;
// C[a][j] = (b1 ? b1[j] : 0) + sum_p U[j][p] G[a][p], a < groups.
void launch_cond_bias(int groups, const float* U, const float* G, const float* b1, float* C, cudaStream_t st);
// dU[j][p] += sum_a (sum_{i: group[i] = a} dZT[j][i]) G[a][p].
void launch_cond_grad(long long n, const __nv_bfloat16* dZT, const int* group, int groups, const float* G, float* dU,
                      cudaStream_t st);
// Batch of n rows from `groups` pairs of pools (poolsA[a]: na rows,
// poolsB[a]: nb rows; device arrays of device pointers): each row picks its
// group uniformly, then pool A with probability node_frac; group[i] records it.
void launch_gather_batch_groups(long long n, unsigned long long seed, float node_frac, int groups,
                                const float* const* poolsA, long long na, const float* const* poolsB, long long nb,
                                float* coords, float* target, int* group, cudaStream_t st);

// ---- cloud-noise builders (k_noise.cu) ----
// max_bits (one uint, zeroed) and range (two uints: 0xFFFFFFFF, 0) are scratch.
void launch_worley(int divisions, int size, const double* grid, float4* local, float* out, unsigned int* max_bits,
                   cudaStream_t st);
void launch_perlin(int divisions, int size, const int* gradients, float* out, unsigned int* range, cudaStream_t st);
// density, mask and work are used only when the state does not fit in
// shared memory (blue_noise_smem sets use_smem false).  Tables of at least
// 2048 pixels that split evenly over 8 (or 16) CTAs run on a CTA cluster
// (blue_noise_cluster_size); `error` (device int, zeroed by the caller) is
// set when one of its bounded waits gave up.
size_t blue_noise_smem(int m, bool* use_smem);
int blue_noise_cluster_size(int m);
int launch_blue_noise(int m, int n, const int* seed, double sigma, const double* table, double* density,
                      double* density0, unsigned char* mask, unsigned char* work, int* dither, int* error,
                      cudaStream_t st);

}  // namespace sfsim
