// k_scatter.cu -- multiple-scattering passes of the atmosphere LUT build
// (atmosphere_lut.clj:86-97): point scatter J, surface radiance dE, ray
// scatter dS, and the re-interpolating accumulation of E and S.
#include <cstddef>
#include <type_traits>

#include "atmo_device.cuh"
#include "kernels.h"

namespace sfsim {

// ---------------------------------------------------------------------------
// Point scatter J (atmosphere.clj:203-222) for all nodes of one (height i,
// sun elevation k) pair.  For such a pair every dS lookup shares the height
// coordinate (x is fixed) and the sun-elevation coordinate (x.l/|x| is the
// sin of the sun elevation), and a direction's elevation coordinate depends
// on the direction alone.  So the block first gathers, per direction, dS
// along the heading axis (8 corners per heading) into a row in shared
// memory; a node then reads two texels of its direction's row at its own
// sun-angle coordinate (omega.l).  The ground term reads the dE table, also
// staged in shared memory.  One thread per node (elevation j, heading a);
// directions, ground ends and T(x, ground) come from k_sphere_setup.
// ---------------------------------------------------------------------------

template <class Real>
__device__ __forceinline__ void gather_heading_row(const Vec4<Real>* t, const BuildDims& d, int u0, int v0, Real s0,
                                                   int u1, int v1, Real s1, int u2, int v2, Real s2, int a,
                                                   Real* dst) {
  // height and sun elevation first, then elevation; a corner whose weight
  // is exactly 0 is not loaded (mix3(x, y, 0) = x exactly)
  auto pair = [&](int h, int e, Real* out) {  // mixed over the sun elevation
    Real A[3], B[3];
    ld3(t, idx4(d, h, e, u2, a), A);
    if (s2 != Real(0)) {
      ld3(t, idx4(d, h, e, v2, a), B);
      mix3(A, B, s2, out);
    } else {
#pragma unroll
      for (int c = 0; c < 3; c++) out[c] = A[c];
    }
  };
  auto row = [&](int e, Real* out) {  // mixed over the height
    Real lo[3], hi[3];
    pair(u0, e, lo);
    if (s0 != Real(0)) {
      pair(v0, e, hi);
      mix3(lo, hi, s0, out);
    } else {
#pragma unroll
      for (int c = 0; c < 3; c++) out[c] = lo[c];
    }
  };
  Real e0[3], e1[3];
  row(u1, e0);
  row(v1, e1);
  mix3(e0, e1, s1, dst);
}

// Shared-memory rows of RGB texels, three values per texel.  (16-byte texels
// were measured slower: a warp's lanes read few distinct texels of a row,
// which scalar loads serve as broadcasts in one wavefront each, while 16-byte
// loads take four.)
template <class Real>
struct TexelRow {
  static constexpr int kStride = 3;
  static __device__ __forceinline__ void load(const Real* base, int idx, Real* out) {
    out[0] = base[3 * idx];
    out[1] = base[3 * idx + 1];
    out[2] = base[3 * idx + 2];
  }
  static __device__ __forceinline__ void store(Real* base, int idx, const Real* v) {
    base[3 * idx] = v[0];
    base[3 * idx + 1] = v[1];
    base[3 * idx + 2] = v[2];
  }
};

// The heading rows of one (height i, sun elevation k) pair: for each of the
// `used` partitioned directions, dS (and in the first iteration the Mie
// strength) gathered along the heading axis at the pair's height and
// sun-elevation coordinates and the direction's elevation coordinate, n3
// texels between copies of the first and last (rows, then rowsM).
template <class Real, bool FIRST>
__device__ __forceinline__ void heading_rows(const BuildDims& d, const SphereDir<Real>* src, int used,
                                             const Vec4<Real>* dS, const Vec4<Real>* Mt, const PointRow<Real>& pk,
                                             Real* rows, int t0, int nt) {
  using TR = TexelRow<Real>;
  const int rlen = d.n3 + 2;
  Real* rowsM = rows + TR::kStride * used * rlen;
  const int u0 = pk.u0, u2 = pk.u2;
  const Real s0 = pk.s0, s2 = pk.s2;
  const int v0 = upper_index(u0, d.n0), v2 = upper_index(u2, d.n2);
  for (int t = t0; t < used * d.n3; t += nt) {
    const int w = t / d.n3, a = t - w * d.n3;
    Real v[3] = {0, 0, 0}, vm[3] = {0, 0, 0};
    if (!src[w].pad) {
      const int u1 = src[w].u1, v1 = upper_index(u1, d.n1);
      const Real s1 = src[w].s1;
      gather_heading_row(dS, d, u0, v0, s0, u1, v1, s1, u2, v2, s2, a, v);
      if (FIRST) gather_heading_row(Mt, d, u0, v0, s0, u1, v1, s1, u2, v2, s2, a, vm);
    }
    const int o = w * rlen + 1 + a;
    TR::store(rows, o, v);
    if (FIRST) TR::store(rowsM, o, vm);
    if (a == 0) {
      TR::store(rows, o - 1, v);
      if (FIRST) TR::store(rowsM, o - 1, vm);
    }
    if (a == d.n3 - 1) {
      TR::store(rows, o + 1, v);
      if (FIRST) TR::store(rowsM, o + 1, vm);
    }
  }
}

// The rows of every (i, k) pair into the global row table, once per
// iteration, so that the point-scatter blocks of a pair copy them instead
// of each gathering them.
template <class Real, bool FIRST>
__global__ void __launch_bounds__(256) k_heading_rows(BuildDims d, const SphereDir<Real>* pdirs, const int2* pcount,
                                                      const PointRow<Real>* prow, const Vec4<Real>* dS,
                                                      const Vec4<Real>* Mt, Real* hrows) {
  const int b = blockIdx.y;
  const int i = blockIdx.x / d.n2, k = blockIdx.x % d.n2;
  const long long pair = ((long long)b * d.n0 + i) * d.n2 + k;
  const SphereDir<Real>* src = pdirs + ((long long)b * d.n0 + i) * dir_row(d.P);
  const long long base4 = (long long)b * d.n4();
  heading_rows<Real, FIRST>(d, src, pcount[(long long)b * d.n0 + i].y, dS + base4, FIRST ? Mt + base4 : nullptr,
                            prow[pair], hrows + pair * heading_rows_stride(d), threadIdx.x, blockDim.x);
}

// Shared-memory layout of point scatter for one (height i, sun elevation k)
// pair, `used` directions (a multiple of kDirBlock):
//   dirs  [kDirFields][used] Real: x0, x1, x2, weight, tR, ground0..2, sE0
//         of each direction (structure of arrays, so that two consecutive
//         directions' components load as one pair);
//   uE0   [used] int;
//   rows  [used][n3 + 2][3] dS gathered along the heading axis between
//         copies of its first and last texel (and the Mie rows in the first
//         iteration);
//   etab  [nE0][nE1][3] the dE table.

template <class Real>
__device__ __forceinline__ V2<Real> ld2(const Real* p) {
  return *reinterpret_cast<const V2<Real>*>(p);
}

static_assert(kDirBlock % 2 == 0, "direction pairs start at even indices (8-byte loads of pair fields)");

// Blocks per (height, sun elevation) pair when each evaluates `cpb` of the
// pair's `nchunks` chunks of 256 nodes; the launch and the kernel share it.
__host__ __device__ __forceinline__ int point_scatter_blocks_per_pair(int nchunks, int cpb) {
  return (nchunks + cpb - 1) / cpb;
}

// Three FP32 blocks of 256 share an SM (80 registers a thread); FP64 blocks
// are register-bound anyway.
constexpr int point_scatter_min_blocks(size_t real_size) { return real_size == 4 ? 3 : 1; }

template <class Real, bool FIRST>
__global__ void __launch_bounds__(256, point_scatter_min_blocks(sizeof(Real))) k_point_scatter(const AtmoParams* params, BuildDims d,
                                                          const RowInfo* rowinfo, const SphereDir<Real>* pdirs,
                                                          const unsigned char* dimage, const int2* pcount,
                                                          const PointRow<Real>* prow,
                                                          const CellGeom<Real>* geom,
                                                          const Real* hrows, const Vec4<Real>* dE, Real* J,
                                                          int nchunks, int chunks_per_block) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  using TR = TexelRow<Real>;
  using R2 = V2<Real>;
  constexpr int RS = TR::kStride;
  constexpr int DB = kDirBlock;
  const int b = blockIdx.y;
  // one (height i, sun elevation k) pair, chunks_per_block chunks of 256 of
  // its (elevation, heading) nodes: the rows are gathered once for them all
  const int nblk = point_scatter_blocks_per_pair(nchunks, chunks_per_block);
  const int chunk0 = (blockIdx.x % nblk) * chunks_per_block;
  const int ik = blockIdx.x / nblk;
  if (ik >= d.n0 * d.n2) return;  // the grid is n0 * n2 * nblk blocks; nothing beyond
  const int i = ik / d.n2, k = ik % d.n2;
  const AtmoParams& P = params[b];
  const PointRow<Real>* prk = prow + ((long long)b * d.n0 + i) * d.n2 + k;
  const int2 pc = pcount[(long long)b * d.n0 + i];
  const int sky_end = pc.x, used = pc.y;
  // texels of a heading row: a copy of texel 0, the n3 texels, a copy of
  // texel n3 - 1, so that a sun-angle coordinate that rounding pushed just
  // outside [0, n3 - 1] reads the edge texel without a clamp
  const int rlen = d.n3 + 2;
  Real* dirs = reinterpret_cast<Real*>(smem_raw);
  int* uE0s = reinterpret_cast<int*>(dirs + kDirFields * used);
  const size_t dir_bytes = dir_image_bytes(used, sizeof(Real));
  Real* rows = reinterpret_cast<Real*>(smem_raw + dir_bytes);
  Real* rowsM = rows + RS * used * rlen;
  Real* etab = rowsM + (FIRST ? RS * used * rlen : 0);

  const long long base4 = (long long)b * d.n4();
  {
    // the height's direction arrays, prepared by k_sphere_partition
    const int4* ds = reinterpret_cast<const int4*>(dimage + ((long long)b * d.n0 + i) *
                                                                dir_image_stride(d, sizeof(Real)));
    int4* dd = reinterpret_cast<int4*>(smem_raw);
    for (int t = threadIdx.x; t < (int)(dir_bytes / 16); t += blockDim.x) dd[t] = ds[t];
  }
  {
    // the pair's heading rows from the row table (k_heading_rows), 16 bytes
    // a thread at a time: a multiple of 24 values, both ends 16-byte aligned
    const int4* hs = reinterpret_cast<const int4*>(hrows + (((long long)b * d.n0 + i) * d.n2 + k) *
                                                                heading_rows_stride(d));
    int4* hd = reinterpret_cast<int4*>(rows);
    const int n16 = (int)((FIRST ? 2 : 1) * (size_t)RS * used * rlen * sizeof(Real) / 16);
    for (int t = threadIdx.x; t < n16; t += blockDim.x) hd[t] = hs[t];
  }
  const long long nE = d.nE();
  for (int t = threadIdx.x; t < nE; t += blockDim.x) {
    Real A[3];
    ld3(dE, b * nE + t, A);
    TR::store(etab, t, A);
  }
  __syncthreads();

  for (int chunk = chunk0; chunk < min(chunk0 + chunks_per_block, nchunks); chunk++) {
    // a lane past the last node keeps running (it feeds the warp's shuffles) but stores nothing
    const int nslab = d.n1 * d.n3;
    const int cell_raw = chunk * blockDim.x + threadIdx.x;
    const bool valid = cell_raw < nslab;
    const int cell = valid ? cell_raw : nslab - 1;
    const int j = cell / d.n3, a = cell % d.n3;
    const RowR<Real> rw = row_r<Real>(rowinfo[(long long)b * d.rows() + (long long)i * d.n1 + j]);
    const Real sv = rw.sv, cv = rw.cv;
    const long long node = base4 + idx4(d, i, j, k, a);
    const CellGeom<Real> g = geom[node];
    const PhaseCS<Real> phR(Bulk<Real>::phase_ray(P)), phM(Bulk<Real>::phase_mie(P));
    const Real scale3 = Real(0.5) * Real(d.n3 - 1);
    const Real scaleE = Bulk<Real>::sun_scale_E(d);
    // The weighted phases depend on (j, direction) only.  When the n3 headings
    // of one j fill aligned lane groups of at least DB lanes, lane p of a group
    // evaluates them for direction p of a block of DB and the group exchanges
    // them by shuffles.
    const int G = d.n3;
    const bool share = G >= DB && (32 % G == 0) && (blockDim.x % G == 0);
    const int lane = threadIdx.x & 31;
    const int gbase = share ? (lane & ~(G - 1)) : lane;
    const int gpos = lane - gbase;
    const int row_len = RS * rlen;
    const R2 lx2 = mk2(g.lx, g.lx), ly2 = mk2(g.ly, g.ly), lz2 = mk2(g.lz, g.lz);
    const R2 sv2 = mk2(sv, sv), cv2 = mk2(cv, cv), sc3 = mk2(scale3, scale3);
    const Real gA = prk->gA;
    const R2 gA2 = mk2(gA, gA);

    // compensated totals (x: Rayleigh, y: Mie) per channel, and the plain
    // partial sums of the current directions (x: even, y: odd direction)
    R2 acc[3], cmp[3], ringR[3], ringM[3];
  #pragma unroll
    for (int c = 0; c < 3; c++) acc[c] = cmp[c] = ringR[c] = ringM[c] = mk2(Real(0), Real(0));
    // One block of DB directions starting at w0 (all sky or all ground), two
    // directions per step.
    auto dir_block = [&](int w0, auto ground) {
      Real wRb = 0, wMb = 0;
      if (share && gpos < DB) {
        const int wb = w0 + gpos;
        const Real mu_v = fma(sv, dirs[wb], cv * dirs[used + wb]);
        wRb = dirs[3 * used + wb] * phR(mu_v);
        wMb = dirs[3 * used + wb] * phM(mu_v);
      }
  #pragma unroll
      for (int q = 0; q < DB; q += 2) {
        const int wa = w0 + q;
        const R2 X0 = ld2(dirs + wa), X1 = ld2(dirs + used + wa), X2 = ld2(dirs + 2 * used + wa);
        R2 wR, wM;
        if (share) {
          wR = mk2(__shfl_sync(0xffffffffu, wRb, gbase + q), __shfl_sync(0xffffffffu, wRb, gbase + q + 1));
          wM = mk2(__shfl_sync(0xffffffffu, wMb, gbase + q), __shfl_sync(0xffffffffu, wMb, gbase + q + 1));
        } else {
          const R2 wt = ld2(dirs + 3 * used + wa);
          const R2 mu_v = fma2(sv2, X0, mul2(cv2, X1));
          wR = mul2(wt, phR.pair(mu_v));
          wM = mul2(wt, phM.pair(mu_v));
        }
        const R2 mu_l = fma2(X0, lx2, fma2(X1, ly2, mul2(X2, lz2)));
        // sun-angle coordinates of (omega, l) along the two directions' heading rows
        const R2 c3 = fma2(sc3, mu_l, sc3);
        // |mu| <= 1 up to rounding, so floor(c) lies in [-1, n3 - 1]: texels u
        // and u + 1 of the padded row give the clamped interpolation exactly
        // (at u = -1 both are texel 0, at u = n3 - 1 the weight s of the copy
        // is rounding-small and both are texel n3 - 1)
        const Real fa = floor(c3.x), fb = floor(c3.y);
        const int ua = (int)fa, ub = (int)fb;
        const R2 s3 = sub2(c3, mk2(fa, fb));
        const Real* ra = rows + wa * row_len + 3 * (ua + 1);
        const Real* rb = rows + (wa + 1) * row_len + 3 * (ub + 1);
        R2 X[3];
  #pragma unroll
        for (int c = 0; c < 3; c++) {
          const R2 lo = mk2(ra[c], rb[c]), hi = mk2(ra[3 + c], rb[3 + c]);
          X[c] = fma2(sub2(hi, lo), s3, lo);
        }
        if (FIRST) {
          const R2 ph = phM.pair(mu_l);
          const Real* ma = rowsM + wa * row_len + 3 * (ua + 1);
          const Real* mb = rowsM + (wa + 1) * row_len + 3 * (ub + 1);
  #pragma unroll
          for (int c = 0; c < 3; c++) {
            const R2 lo = mk2(ma[c], mb[c]), hi = mk2(ma[3 + c], mb[3 + c]);
            X[c] = fma2(fma2(sub2(hi, lo), s3, lo), ph, X[c]);
          }
        }
        if (decltype(ground)::value) {
          // the ground point's sin of the sun elevation, g.l / |g| = gA + tR (omega . l)
          const R2 sg = fma2(ld2(dirs + 4 * used + wa), mu_l, gA2);
          int ea, eb;
          Real ta, tb;
          split_coord_r<Real>(sun_elevation_index_r<Real>(sg.x, scaleE), d.nE1, &ea, &ta);
          split_coord_r<Real>(sun_elevation_index_r<Real>(sg.y, scaleE), d.nE1, &eb, &tb);
          const int fa = upper_index(ea, d.nE1), fb = upper_index(eb, d.nE1);
          // both directions' height rows in one 8-byte load (wa is even and
          // the int array starts 8-byte aligned: kDirFields * used floats, used
          // a multiple of kDirBlock)
          const int2 hab = *reinterpret_cast<const int2*>(uE0s + wa);
          const int ha = hab.x, hb = hab.y;
          const int ka = upper_index(ha, d.nE0), kb = upper_index(hb, d.nE0);
          const R2 sE1 = mk2(ta, tb), sE0 = ld2(dirs + 8 * used + wa);
          const R2 one = mk2(Real(1), Real(1));
          const R2 oi = sub2(one, sE1);
          const Real* e0a = etab + 3 * ha * d.nE1;
          const Real* e0b = etab + 3 * hb * d.nE1;
          if (sE0.x == Real(0) && sE0.y == Real(0)) {
            // the vE0 row has weight 0: the bilinear mix is its uE0 row exactly
            // (the same for every lane: both directions are the warp's)
  #pragma unroll
            for (int c = 0; c < 3; c++) {
              const R2 Y = fma2(mk2(e0a[3 * fa + c], e0b[3 * fb + c]), sE1, mul2(mk2(e0a[3 * ea + c], e0b[3 * eb + c]), oi));
              X[c] = fma2(ld2(dirs + (5 + c) * used + wa), Y, X[c]);
            }
          } else {
            const R2 oo = sub2(one, sE0);
            const Real* e1a = etab + 3 * ka * d.nE1;
            const Real* e1b = etab + 3 * kb * d.nE1;
  #pragma unroll
            for (int c = 0; c < 3; c++) {
              // bilinear in height rows (uE0, vE0) and sun-elevation columns (uE1, vE1)
              const R2 lo =
                  fma2(mk2(e0a[3 * fa + c], e0b[3 * fb + c]), sE1, mul2(mk2(e0a[3 * ea + c], e0b[3 * eb + c]), oi));
              const R2 hi =
                  fma2(mk2(e1a[3 * fa + c], e1b[3 * fb + c]), sE1, mul2(mk2(e1a[3 * ea + c], e1b[3 * eb + c]), oi));
              const R2 Y = fma2(hi, sE0, mul2(lo, oo));
              X[c] = fma2(ld2(dirs + (5 + c) * used + wa), Y, X[c]);
            }
          }
        }
  #pragma unroll
        for (int c = 0; c < 3; c++) {
          ringR[c] = fma2(wR, X[c], ringR[c]);
          ringM[c] = fma2(wM, X[c], ringM[c]);
        }
      }
    };
    // the partial sums of up to two blocks go to the compensated totals
    auto flush = [&]() {
  #pragma unroll
      for (int c = 0; c < 3; c++) {
        const R2 x = mk2(ringR[c].x + ringR[c].y, ringM[c].x + ringM[c].y);
        const R2 y = sub2(x, cmp[c]);
        const R2 t = add2(acc[c], y);
        cmp[c] = sub2(sub2(t, acc[c]), y);
        acc[c] = t;
        ringR[c] = ringM[c] = mk2(Real(0), Real(0));
      }
    };
    for (int w0 = 0; w0 < sky_end; w0 += DB) {
      dir_block(w0, std::false_type{});
      if (w0 & DB) flush();
    }
    flush();
    for (int w0 = sky_end; w0 < used; w0 += DB) {
      dir_block(w0, std::true_type{});
      if ((w0 - sky_end) & DB) flush();
    }
    flush();
    if (valid) {
      // beta_c(x) (atmosphere.clj:42-47, 140-151)
      const PointRow<Real> pr = *prk;
      Vec4<Real> o;
      o.x = pr.bR[0] * acc[0].x + pr.bM[0] * acc[0].y;
      o.y = pr.bR[1] * acc[1].x + pr.bM[1] * acc[1].y;
      o.z = pr.bR[2] * acc[2].x + pr.bM[2] * acc[2].y;
      // J planar, [atmosphere][channel][node], for the ray-scatter gathers
      Real* Jb = J + (long long)b * 3 * d.n4() + (node - base4);
      Jb[0] = o.x;
      Jb[d.n4()] = o.y;
      Jb[2 * d.n4()] = o.z;
    }
  }
}

template <class Real>
size_t point_scatter_smem(const BuildDims& d, bool first) {
  const size_t n = dir_row(d.P);
  return ((n * (kDirFields * sizeof(Real) + sizeof(int)) + 15) & ~size_t(15)) +
         sizeof(Real) * 3 * (n * (d.n3 + 2) * (first ? 2 : 1) + d.nE());
}

template <class Real>
int launch_point_scatter(const AtmoParams* params, const BuildDims& d, const RowInfo* rowinfo,
                         const SphereDir<Real>* pdirs, const unsigned char* dimage, const int2* pcount,
                         const PointRow<Real>* prow, const CellGeom<Real>* geom, const Vec4<Real>* dS,
                         const Vec4<Real>* mie, const Vec4<Real>* dE, Real* hrows, Real* J, cudaStream_t st) {
  const int block = 256;
  const int nchunks = (d.n1 * d.n3 + block - 1) / block;
  const int cpb = 2;
  const bool first = mie != nullptr;
  size_t smem = point_scatter_smem<Real>(d, first);
  const dim3 rgrid((unsigned)(d.n0 * d.n2), d.B);
  dim3 grid((unsigned)(d.n0 * d.n2 * point_scatter_blocks_per_pair(nchunks, cpb)), d.B);
  if (first) {
    if (cudaFuncSetAttribute(k_point_scatter<Real, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess)
      return -1;
    k_heading_rows<Real, true><<<rgrid, block, 0, st>>>(d, pdirs, pcount, prow, dS, mie, hrows);
    k_point_scatter<Real, true><<<grid, block, smem, st>>>(params, d, rowinfo, pdirs, dimage, pcount, prow, geom,
                                                           hrows, dE, J, nchunks, cpb);
  } else {
    if (cudaFuncSetAttribute(k_point_scatter<Real, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem) != cudaSuccess)
      return -1;
    k_heading_rows<Real, false><<<rgrid, block, 0, st>>>(d, pdirs, pcount, prow, dS, nullptr, hrows);
    k_point_scatter<Real, false><<<grid, block, smem, st>>>(params, d, rowinfo, pdirs, dimage, pcount, prow, geom,
                                                            hrows, dE, J, nchunks, cpb);
  }
  return 0;
}

// Threads per surface-radiance node: 128 lets about seven blocks share an
// SM, so the 1024 nodes of the production tables run in about one wave.
constexpr int kSurfaceThreads = 128;

// ---------------------------------------------------------------------------
// Surface radiance dE (atmosphere.clj:225-230): integral over the upper half
// sphere of dS(x, w, l, above) (w.n); the reference passes the ray steps as
// the sphere steps (atmosphere_lut.clj:89).  One block per node, threads over
// directions, block reduction.  The per-node coordinates and the world-space
// directions come from FP64 setup tables, so no thread uses the FP64 pipe.
// ---------------------------------------------------------------------------

template <class Real, bool FIRST>
__global__ void __launch_bounds__(kSurfaceThreads) k_surface_radiance(const AtmoParams* params, BuildDims d,
                                                          const SurfRow<Real>* erow, const HalfDir<Real>* hdir,
                                                          const Vec4<Real>* dS, const Vec4<Real>* Mt,
                                                          Vec4<Real>* dE) {
  __shared__ Real red[3][kSurfaceThreads];
  const int b = blockIdx.y;
  const long long node = blockIdx.x;
  const AtmoParams& P = params[b];
  const int iE = (int)(node / d.nE1);
  // per node, from FP64 (k_surface_rows): x = (r, 0, 0), l = (lx, ly, 0) and
  // the height and sun-elevation coordinates shared by every direction
  const SurfRow<Real> er = erow[(long long)b * d.nE() + node];
  int u[4] = {er.u0, 0, er.u2, 0};
  Real s[4] = {er.s0, 0, er.s2, 0};
  // elevation coordinate of (x, w, above) (atmosphere.clj:239-253) in Real:
  // r sin_el = x.w, rho^2 = q, Delta + H^2 = (x.w)^2 + (H^2 - q) with both
  // terms non-negative, and r sin_el - sqrt(Delta + H^2) rewritten without
  // cancellation when x.w > 0
  const Real Hh2mq = er.Hh2mq, den = er.den, rr = er.rr, lx = er.lx, ly = er.ly;
  const Real scale1 = Real(d.n1 - 1), scale3 = Real(0.5) * Real(d.n3 - 1);
  const Vec4<Real>* tS = dS + (long long)b * d.n4();
  const Vec4<Real>* tM = FIRST ? Mt + (long long)b * d.n4() : nullptr;
  const HalfDir<Real>* hd = hdir + ((long long)b * d.nE0 + iE) * d.Ph;
  const PhaseCS<Real> phase_mie(Bulk<Real>::phase_mie(P));
  Real acc[3] = {0, 0, 0}, cmp[3] = {0, 0, 0};
  for (int w = threadIdx.x; w < d.Ph; w += blockDim.x) {
    const HalfDir<Real> qd = hd[w];
    const Real wx = qd.wx, wy = qd.wy;
    const Real pv = rr * wx;
    const Real root = Bulk<Real>::sqrt(fma(pv, pv, Hh2mq));
    const Real a = pv > Real(0) ? -Hh2mq / (pv + root) : pv - root;
    int uu[4] = {u[0], 0, u[2], 0};
    Real sx[4] = {s[0], 0, s[2], 0};
    Real lq;
    {
      // limit-quot (util.clj:403-420) with limits -0.5, 0
      Real aa = a, bb = den;
      if (aa == Real(0)) lq = Real(0);
      else {
        if (bb < Real(0)) { aa = -aa; bb = -bb; }
        lq = aa < Real(0) ? (aa > bb * Real(-0.5) ? aa / bb : Real(-0.5)) : Real(0);
      }
    }
    {
      // (n1 - 1)(1/2 - lq) with the exact base (n1 - 1)/2 split off: the
      // fraction keeps the precision of the part above it, -(n1 - 1) lq,
      // which is small for the rays near the horizon that carry the most
      // light (in FP32 the whole coordinate near n1/2 resolves only ~1e-5 of
      // a texel there, and the table is steep)
      const Real t = ((d.n1 - 1) & 1 ? Real(0.5) : Real(0)) - scale1 * lq;
      const Real ft = floor(t);
      uu[1] = ((d.n1 - 1) >> 1) + (int)ft;
      sx[1] = t - ft;
      if (uu[1] >= d.n1 - 1) {
        uu[1] = d.n1 - 1;
        sx[1] = Real(0);
      }
    }
    const Real mu = fma(wx, lx, wy * ly);  // w.l, l.z = 0
    split_coord_r<Real>(scale3 * (Real(1) + mu), d.n3, &uu[3], &sx[3]);
    Real val[3];
    interp4(tS, d, uu, sx, val);
    if (FIRST) {
      Real vm[3];
      interp4(tM, d, uu, sx, vm);
      const Real ph = phase_mie(mu);
#pragma unroll
      for (int c = 0; c < 3; c++) val[c] = fma(vm[c], ph, val[c]);
    }
    const Real wgt = qd.wgt;
#pragma unroll
    for (int c = 0; c < 3; c++) kahan_add(acc[c], cmp[c], val[c] * wgt);
  }
#pragma unroll
  for (int c = 0; c < 3; c++) red[c][threadIdx.x] = acc[c];
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
#pragma unroll
      for (int c = 0; c < 3; c++) red[c][threadIdx.x] += red[c][threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    Vec4<Real> o;
    o.x = red[0][0];
    o.y = red[1][0];
    o.z = red[2][0];
    o.w = 0;
    dE[(long long)b * d.nE() + node] = o;
  }
}

template <class Real>
void launch_surface_radiance(const AtmoParams* params, const BuildDims& d, const SurfRow<Real>* erow,
                             const HalfDir<Real>* hdir, const Vec4<Real>* dS, const Vec4<Real>* mie,
                             Vec4<Real>* dE, cudaStream_t st) {
  dim3 grid((unsigned)d.nE(), d.B);
  if (mie)
    k_surface_radiance<Real, true><<<grid, kSurfaceThreads, 0, st>>>(params, d, erow, hdir, dS, mie, dE);
  else
    k_surface_radiance<Real, false><<<grid, kSurfaceThreads, 0, st>>>(params, d, erow, hdir, dS, mie, dE);
}

// ---------------------------------------------------------------------------
// Ray scatter dS (atmosphere.clj:192-200) with J from the point-scatter table.
// One block per view row (i, j); one thread per node (sun elevation k, sun
// heading a).  For a ray sample p_s the J lookup's height and elevation
// coordinates depend on the row only, so the block collapses them into a
// plane [sun elevation][heading] per sample in shared memory; each node then
// gathers bilinearly from the plane at its own sun-elevation coordinate
// (from p_s.l) and sun-angle coordinate (v.l, constant along the ray).
// T(x, p_s) comes from k_view_rows.
//
// Plane layout (three values a texel).  With 32 sun elevations (the
// production shapes) the planes are stored column by column, texel
// (sun elevation r, heading a) at a * 36 + r: a warp of the plane build then
// stores 4 sun elevations x 8 headings to 32 distinct banks, and the
// gather's loads (a warp's 32 nodes read rows spread by their own sun
// elevations in up to 8 heading columns) meet a third fewer bank conflicts
// than with rows of 24 values.  Other shapes keep rows (texel at r * n3 + a):
// at 16 sun elevations a CPU model of the gathers finds rows best.
// ---------------------------------------------------------------------------

// Per-sample constants of one chunk of CH ray samples, as arrays so that two
// consecutive samples' values load as one pair: T(x, p_s), (s + 1/2)/S and
// 1/|p_s| for the nodes, the (height, elevation) fractions and the J offsets
// of the four corner planes for the plane build.
template <class Real, int CH>
struct RayChunk {
  Real T[3][CH];
  Real us[CH], inv_r[CH], s0[CH], s1[CH];
  int p[4][CH];
};

// Column-major planes (see above) for multiples of 32 sun elevations, with
// columns of n2 + 4 texels; rows of n3 texels otherwise.
__host__ __device__ constexpr bool ray_plane_by_column(int n2) { return n2 % 32 == 0; }
__host__ __device__ constexpr int ray_plane_texels(const BuildDims& d) {
  return ray_plane_by_column(d.n2) ? (d.n2 + 4) * d.n3 : d.n2 * d.n3;
}

// Bytes of the CH planes of one chunk (a multiple of 16 for even CH).
template <class Real, int CH>
__host__ __device__ constexpr size_t ray_plane_bytes(const BuildDims& d) {
  return sizeof(Real) * 3 * (size_t)CH * ray_plane_texels(d);
}

// The view row's samples (k_view_rows) are copied into shared memory once
// per block when they take at most this many bytes, so that each chunk's
// constants come from there instead of a global-memory round trip.
constexpr size_t kRayStageBytes = 16384;
template <class Real>
__host__ __device__ constexpr bool ray_stage_rows(int S) {
  return (size_t)S * sizeof(RowSample<Real>) <= kRayStageBytes;
}

// Three FP32 blocks per SM: 80 registers a thread hold the plane build's
// cached J corners without spills (four blocks at 64 registers spilled).
constexpr int ray_scatter_min_blocks(size_t real_size) { return real_size == 4 ? 3 : 1; }

// WIDE: a row has more cells than the block has threads, and the plane build
// walks them blockDim.x apart; a separate instantiation, so that the
// one-cell-per-thread build keeps its registers.  COLS: column-major planes.
template <class Real, int CH, bool WIDE, bool COLS>
__global__ void __launch_bounds__(256, ray_scatter_min_blocks(sizeof(Real)))
    k_ray_scatter(const AtmoParams* params, BuildDims d, const RowInfo* rowinfo, const RowSample<Real>* rows,
                  const CellGeom<Real>* geom, const Remap4<Real>* remap, const Real* J, Vec4<Real>* dS) {
  static_assert(CH % 2 == 0, "samples go in pairs");
  using R2 = V2<Real>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int b = blockIdx.y;
  const long long row = blockIdx.x;
  const long long nrows = d.rows();
  const int ncell = d.n2 * d.n3;
  RayChunk<Real, CH>& sc = *reinterpret_cast<RayChunk<Real, CH>*>(smem_raw);
  Real* plane = reinterpret_cast<Real*>(smem_raw + ((sizeof(RayChunk<Real, CH>) + 15) & ~size_t(15)));
  const RowSample<Real>* rs = rows + (b * nrows + row) * d.S;
  if (ray_stage_rows<Real>(d.S)) {
    // 16-byte words where the row's samples start on a 16-byte boundary and
    // fill whole words (S = 128: 6656 bytes a row), else 4-byte words
    // (sizeof(RowSample<float>) is 52); the stage itself is 16-byte aligned.
    // The first chunk's barrier publishes the copy.
    static_assert(sizeof(RowSample<Real>) % 4 == 0, "rows are copied in 4-byte words");
    RowSample<Real>* stage = reinterpret_cast<RowSample<Real>*>(
        reinterpret_cast<unsigned char*>(plane) + ray_plane_bytes<Real, CH>(d));
    const size_t bytes = d.S * sizeof(RowSample<Real>);
    if ((reinterpret_cast<size_t>(rs) & 15) == 0 && bytes % 16 == 0) {
      const int4* g = reinterpret_cast<const int4*>(rs);
      int4* sd = reinterpret_cast<int4*>(stage);
      for (int w = threadIdx.x; w < (int)(bytes / 16); w += blockDim.x) sd[w] = g[w];
    } else {
      const int* g = reinterpret_cast<const int*>(rs);
      int* sd = reinterpret_cast<int*>(stage);
      for (int w = threadIdx.x; w < (int)(bytes / 4); w += blockDim.x) sd[w] = g[w];
    }
    rs = stage;
  }
  const RowInfo ri = rowinfo[b * nrows + row];
  const long long n4 = d.n4();
  const Real* tJ = J + (long long)b * 3 * n4;  // planar [channel][node]
  const long long node0 = (b * nrows + row) * ncell;
  const Real scale2 = Bulk<Real>::sun_scale(d);
  const RowR<Real> rw = row_r<Real>(ri);
  const Real rr = rw.r, D0 = rw.D[0], D1 = rw.D[1], D2 = rw.D[2];
  // values between texels one sun elevation (row3) and one heading (col3)
  // apart, and of a plane; one of the steps is a constant
  const int row3 = COLS ? 3 : 3 * d.n3;
  const int col3 = COLS ? 3 * (d.n2 + 4) : 3;
  const int pl3 = 3 * ray_plane_texels(d);

  for (int c0 = 0; c0 < ncell; c0 += blockDim.x) {
    const int cell = c0 + threadIdx.x;
    const bool active = cell < ncell;
    Real b0 = 0, Dl = 0, s3 = 0;
    int o3u = 0, o3v = 0;
    if (active) {
      const CellGeom<Real> g = geom[node0 + cell];
      b0 = rr * g.lx;
      Dl = fma(D0, g.lx, fma(D1, g.ly, D2 * g.lz));
      const Remap4<Real> m = remap[node0 + cell];  // its sun-angle coordinate is that of (v, l)
      o3u = col3 * m.u[3];
      o3v = col3 * upper_index(m.u[3], d.n3);
      s3 = m.s[3];
    }
    const R2 b02 = mk2(b0, b0), Dl2 = mk2(Dl, Dl), s32 = mk2(s3, s3);
    // x: even samples, y: odd samples (independent FMA chains)
    R2 acc[3] = {mk2(Real(0), Real(0)), mk2(Real(0), Real(0)), mk2(Real(0), Real(0))};
    // the plane build's cached J corners of the last even and odd samples
    Real ca[12], cb[12];
    int key_a = -1, key_b = -1, a1 = -1, a2 = -1, b1 = -1, b2 = -1;  // keys and corners 1, 2 of the caches
    for (int sb = 0; sb < d.S; sb += CH) {
      const int nch = min(CH, d.S - sb);
      __syncthreads();
      if (threadIdx.x < nch) {
        const int u = threadIdx.x;
        const RowSample<Real> q = rs[sb + u];
        sc.T[0][u] = exp_neg(q.tau[0]);
        sc.T[1][u] = exp_neg(q.tau[1]);
        sc.T[2][u] = exp_neg(q.tau[2]);
        sc.us[u] = q.us;
        sc.inv_r[u] = q.inv_r;
        sc.s0[u] = q.s0;
        sc.s1[u] = q.s1;
        const int v0 = upper_index(q.u0, d.n0), v1 = upper_index(q.u1, d.n1);
        sc.p[0][u] = (q.u0 * d.n1 + q.u1) * ncell;
        sc.p[1][u] = (q.u0 * d.n1 + v1) * ncell;
        sc.p[2][u] = (v0 * d.n1 + q.u1) * ncell;
        sc.p[3][u] = (v0 * d.n1 + v1) * ncell;
      }
      __syncthreads();
      // the plane of samples (ch, ch + 1): bilinear in (height, elevation)
      if constexpr (!WIDE) {
        // one cell per thread: its J corner values stay in registers while
        // consecutive samples share their (height, elevation) corners (the
        // first corner's offset identifies all four); about half the pairs do
        if (threadIdx.x < ncell) {
          const int t = threadIdx.x;
          const int st3 = COLS ? (t % d.n3) * col3 + 3 * (t / d.n3) : 3 * t;  // texel (k = t / n3, a = t mod n3)
          for (int ch = 0; ch < nch; ch += 2) {
            const bool two = ch + 1 < nch;
            const int ch1 = two ? ch + 1 : ch;
            const int pa = sc.p[0][ch], pb = sc.p[0][ch1];
            // sample s's corners into v from the previous sample's cache src
            // (offsets k0 = its key, k1, k2): a step of one cell along one
            // axis carries two corners over, the other two are loaded
            auto refill = [&](int s, Real (&v)[12], const Real (&src)[12], int k0, int k1, int k2, int& o1,
                              int& o2) {
              const int q0 = sc.p[0][s], q1 = sc.p[1][s], q2 = sc.p[2][s], q3 = sc.p[3][s];
              const Real* tt = tJ + t;
              if (q0 == k1) {  // elevation + 1: corners 1, 3 become 0, 2
#pragma unroll
                for (int c = 0; c < 3; c++) {
                  v[4 * c] = src[4 * c + 1], v[4 * c + 2] = src[4 * c + 3];
                  v[4 * c + 1] = tt[c * n4 + q1], v[4 * c + 3] = tt[c * n4 + q3];
                }
              } else if (q1 == k0) {  // elevation - 1: corners 0, 2 become 1, 3
#pragma unroll
                for (int c = 0; c < 3; c++) {
                  v[4 * c + 1] = src[4 * c], v[4 * c + 3] = src[4 * c + 2];
                  v[4 * c] = tt[c * n4 + q0], v[4 * c + 2] = tt[c * n4 + q2];
                }
              } else if (q0 == k2) {  // height + 1: corners 2, 3 become 0, 1
#pragma unroll
                for (int c = 0; c < 3; c++) {
                  v[4 * c] = src[4 * c + 2], v[4 * c + 1] = src[4 * c + 3];
                  v[4 * c + 2] = tt[c * n4 + q2], v[4 * c + 3] = tt[c * n4 + q3];
                }
              } else if (q2 == k0) {  // height - 1: corners 0, 1 become 2, 3
#pragma unroll
                for (int c = 0; c < 3; c++) {
                  v[4 * c + 2] = src[4 * c], v[4 * c + 3] = src[4 * c + 1];
                  v[4 * c] = tt[c * n4 + q0], v[4 * c + 1] = tt[c * n4 + q1];
                }
              } else {
#pragma unroll
                for (int c = 0; c < 3; c++) {
                  v[4 * c] = tt[c * n4 + q0], v[4 * c + 1] = tt[c * n4 + q1];
                  v[4 * c + 2] = tt[c * n4 + q2], v[4 * c + 3] = tt[c * n4 + q3];
                }
              }
              o1 = q1;
              o2 = q2;
            };
            if (pa != key_a) {
              if (pa == key_b) {
#pragma unroll
                for (int m = 0; m < 12; m++) ca[m] = cb[m];
                a1 = b1, a2 = b2;
              } else {
                refill(ch, ca, cb, key_b, b1, b2, a1, a2);
              }
              key_a = pa;
            }
            if (pb != key_b) {
              if (pb == key_a) {
#pragma unroll
                for (int m = 0; m < 12; m++) cb[m] = ca[m];
                b1 = a1, b2 = a2;
              } else {
                refill(ch1, cb, ca, key_a, a1, a2, b1, b2);
              }
              key_b = pb;
            }
            const R2 s0 = mk2(sc.s0[ch], sc.s0[ch1]), s1 = mk2(sc.s1[ch], sc.s1[ch1]);
            Real* dst0 = plane + ch * pl3 + st3;
            Real* dst1 = dst0 + pl3;
#pragma unroll
            for (int c = 0; c < 3; c++) {
              const R2 A = mk2(ca[4 * c], cb[4 * c]), B = mk2(ca[4 * c + 1], cb[4 * c + 1]);
              const R2 C = mk2(ca[4 * c + 2], cb[4 * c + 2]), E = mk2(ca[4 * c + 3], cb[4 * c + 3]);
              const R2 lo = fma2(sub2(B, A), s1, A), hi = fma2(sub2(E, C), s1, C);
              const R2 v = fma2(sub2(hi, lo), s0, lo);
              dst0[c] = v.x;
              if (two) dst1[c] = v.y;
            }
          }
        }
      } else {
        for (int t = threadIdx.x; t < ncell; t += blockDim.x) {
          const int st3 = COLS ? (t % d.n3) * col3 + 3 * (t / d.n3) : 3 * t;
          for (int ch = 0; ch < nch; ch += 2) {
            const bool two = ch + 1 < nch;
            const int ch1 = two ? ch + 1 : ch;
            const int pa[4] = {sc.p[0][ch], sc.p[1][ch], sc.p[2][ch], sc.p[3][ch]};
            const int pb[4] = {sc.p[0][ch1], sc.p[1][ch1], sc.p[2][ch1], sc.p[3][ch1]};
            const R2 s0 = mk2(sc.s0[ch], sc.s0[ch1]), s1 = mk2(sc.s1[ch], sc.s1[ch1]);
            Real* dst0 = plane + ch * pl3 + st3;
            Real* dst1 = dst0 + pl3;
#pragma unroll
            for (int c = 0; c < 3; c++) {
              const Real* tc = tJ + c * n4 + t;
              const R2 A = mk2(tc[pa[0]], tc[pb[0]]), B = mk2(tc[pa[1]], tc[pb[1]]);
              const R2 C = mk2(tc[pa[2]], tc[pb[2]]), E = mk2(tc[pa[3]], tc[pb[3]]);
              const R2 lo = fma2(sub2(B, A), s1, A), hi = fma2(sub2(E, C), s1, C);
              const R2 v = fma2(sub2(hi, lo), s0, lo);
              dst0[c] = v.x;
              if (two) dst1[c] = v.y;
            }
          }
        }
      }
      __syncthreads();
      if (active) {
        int ch = 0;
        for (; ch + 1 < nch; ch += 2) {
          const R2 sin_el = mul2(fma2(ld2(sc.us + ch), Dl2, b02), ld2(sc.inv_r + ch));  // p_s.l / |p_s|
          const R2 ie = sun_elevation_index_r2<Real>(sin_el, scale2);
          int ua, ub;
          Real sa, sb;
          split_coord_r<Real>(ie.x, d.n2, &ua, &sa);
          split_coord_r<Real>(ie.y, d.n2, &ub, &sb);
          const R2 s2 = mk2(sa, sb);
          const Real* loa = plane + ch * pl3 + row3 * ua;
          const Real* hia = ua + 1 < d.n2 ? loa + row3 : loa;
          const Real* lob = plane + (ch + 1) * pl3 + row3 * ub;
          const Real* hib = ub + 1 < d.n2 ? lob + row3 : lob;
#pragma unroll
          for (int c = 0; c < 3; c++) {
            const R2 lu = mk2(loa[o3u + c], lob[o3u + c]), lv = mk2(loa[o3v + c], lob[o3v + c]);
            const R2 hu = mk2(hia[o3u + c], hib[o3u + c]), hv = mk2(hia[o3v + c], hib[o3v + c]);
            const R2 x0 = fma2(sub2(lv, lu), s32, lu);
            const R2 x1 = fma2(sub2(hv, hu), s32, hu);
            acc[c] = fma2(ld2(sc.T[c] + ch), fma2(sub2(x1, x0), s2, x0), acc[c]);
          }
        }
        if (ch < nch) {
          const Real sin_el = fma(sc.us[ch], Dl, b0) * sc.inv_r[ch];
          int u2;
          Real s2;
          split_coord_r<Real>(sun_elevation_index_r<Real>(sin_el, scale2), d.n2, &u2, &s2);
          const Real* lo = plane + ch * pl3 + row3 * u2;
          const Real* hi = u2 + 1 < d.n2 ? lo + row3 : lo;
#pragma unroll
          for (int c = 0; c < 3; c++) {
            const Real x0 = fma(lo[o3v + c] - lo[o3u + c], s3, lo[o3u + c]);
            const Real x1 = fma(hi[o3v + c] - hi[o3u + c], s3, hi[o3u + c]);
            acc[c].x = fma(sc.T[c][ch], fma(x1 - x0, s2, x0), acc[c].x);
          }
        }
      }
    }
    if (active) {
      const Real w = rw.Ls;
      Vec4<Real> o;
      o.x = w * (acc[0].x + acc[0].y);
      o.y = w * (acc[1].x + acc[1].y);
      o.z = w * (acc[2].x + acc[2].y);
      o.w = 0;
      dS[node0 + cell] = o;
    }
  }
}

constexpr int kRayChunk = 16;  // ray samples per chunk of k_ray_scatter

// Dynamic shared memory of k_ray_scatter: the chunk's constants, one plane
// of n3 heading columns of RGB texels per sample, and the staged row
// samples.
template <class Real>
size_t ray_scatter_smem(const BuildDims& d) {
  return ((sizeof(RayChunk<Real, kRayChunk>) + 15) & ~size_t(15)) + ray_plane_bytes<Real, kRayChunk>(d) +
         (ray_stage_rows<Real>(d.S) ? (size_t)d.S * sizeof(RowSample<Real>) : 0);
}

template <class Real>
int launch_ray_scatter(const AtmoParams* params, const BuildDims& d, const RowInfo* rowinfo,
                       const RowSample<Real>* rows, const CellGeom<Real>* geom, const Remap4<Real>* remap,
                       const Real* J, Vec4<Real>* dS, cudaStream_t st) {
  constexpr int CH = kRayChunk;
  const int ncell = d.n2 * d.n3;
  const int block = ncell >= 256 ? 256 : ((ncell + 31) / 32) * 32;
  const size_t smem = ray_scatter_smem<Real>(d);
  auto pick = [&](auto cols) {
    constexpr bool C = decltype(cols)::value;
    return ncell > block ? k_ray_scatter<Real, CH, true, C> : k_ray_scatter<Real, CH, false, C>;
  };
  auto kernel = ray_plane_by_column(d.n2) ? pick(std::true_type{}) : pick(std::false_type{});
  if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return -1;
  dim3 grid((unsigned)d.rows(), d.B);
  kernel<<<grid, block, smem, st>>>(params, d, rowinfo, rows, geom, remap, J, dS);
  return 0;
}

// ---------------------------------------------------------------------------
// Re-interpolating accumulation and outputs
// ---------------------------------------------------------------------------

template <class Real>
__global__ void k_accumulate4(BuildDims d, const Remap4<Real>* remap, const Vec4<Real>* A, const Vec4<Real>* Bt,
                              Vec4<Real>* out) {
  const long long n4 = d.n4();
  const long long node = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const int b = blockIdx.y;
  if (node >= n4) return;
  const Remap4<Real> m = remap[b * n4 + node];
  Real va[3], vb[3] = {0, 0, 0};
  interp4<Real, true>(A + b * n4, d, m.u, m.s, va);
  if (Bt) interp4<Real, true>(Bt + b * n4, d, m.u, m.s, vb);
  Vec4<Real> o;
  o.x = va[0] + vb[0];
  o.y = va[1] + vb[1];
  o.z = va[2] + vb[2];
  o.w = 0;
  out[b * n4 + node] = o;
}

template <class Real>
__global__ void k_accumulate2(int n0, int n1, const Remap2<Real>* remap, const Vec4<Real>* A, const Vec4<Real>* Bt,
                              Vec4<Real>* out) {
  const long long n = (long long)n0 * n1;
  const long long node = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const int b = blockIdx.y;
  if (node >= n) return;
  const Remap2<Real> m = remap[b * n + node];
  Real va[3] = {0, 0, 0}, vb[3] = {0, 0, 0};
  if (A) interp2(A + b * n, n0, n1, m.u, m.s, va);
  if (Bt) interp2(Bt + b * n, n0, n1, m.u, m.s, vb);
  Vec4<Real> o;
  o.x = va[0] + vb[0];
  o.y = va[1] + vb[1];
  o.z = va[2] + vb[2];
  o.w = 0;
  out[b * n + node] = o;
}

// convert-4d-to-2d (image.clj:299-312) + pack-matrices (matrix.clj:130-134)
template <class Real>
__global__ void k_output4(BuildDims d, const Remap4<Real>* remap, const Vec4<Real>* tab, float* out) {
  const long long n4 = d.n4();
  const long long node = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const int b = blockIdx.y;
  if (node >= n4) return;
  const Remap4<Real> m = remap[b * n4 + node];
  Real v[3];
  interp4<Real, true>(tab + b * n4, d, m.u, m.s, v);
  const int a = (int)(node % d.n3);
  const int k = (int)((node / d.n3) % d.n2);
  const int j = (int)((node / ((long long)d.n3 * d.n2)) % d.n1);
  const int i = (int)(node / ((long long)d.n3 * d.n2 * d.n1));
  const long long dst = ((long long)i * d.n2 + k) * ((long long)d.n1 * d.n3) + (long long)j * d.n3 + a;
  float* o = out + 3 * (b * n4 + dst);
  o[0] = (float)v[0];
  o[1] = (float)v[1];
  o[2] = (float)v[2];
}

template <class Real>
__global__ void k_output2(int n0, int n1, const Remap2<Real>* remap, const Vec4<Real>* tab, float* out) {
  const long long n = (long long)n0 * n1;
  const long long node = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const int b = blockIdx.y;
  if (node >= n) return;
  const Remap2<Real> m = remap[b * n + node];
  Real v[3] = {0, 0, 0};
  if (tab) interp2(tab + b * n, n0, n1, m.u, m.s, v);
  float* o = out + 3 * (b * n + node);
  o[0] = (float)v[0];
  o[1] = (float)v[1];
  o[2] = (float)v[2];
}

template <class Real>
__global__ void k_add_to_sum(long long n4, int B, const Real* J, Vec4<float>* jsum, bool first) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= n4 * B) return;
  const Real* src = J + (t / n4) * 3 * n4 + t % n4;
  Vec4<float> o;
  if (first) {
    o.x = 0;
    o.y = 0;
    o.z = 0;
    o.w = 0;
  } else {
    o = jsum[t];
  }
  o.x += (float)src[0];
  o.y += (float)src[n4];
  o.z += (float)src[2 * n4];
  jsum[t] = o;
}

template <class Real>
__global__ void k_export(long long n, const Vec4<Real>* tab, float* out) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= n) return;
  const Vec4<Real> v = tab[t];
  out[3 * t] = (float)v.x;
  out[3 * t + 1] = (float)v.y;
  out[3 * t + 2] = (float)v.z;
}

static inline dim3 grid1(long long n, int block, int B) { return dim3((unsigned)((n + block - 1) / block), B); }

template <class Real>
void launch_accumulate4(const BuildDims& d, const Remap4<Real>* remap, const Vec4<Real>* a, const Vec4<Real>* b,
                        Vec4<Real>* out, cudaStream_t st) {
  k_accumulate4<Real><<<grid1(d.n4(), 256, d.B), 256, 0, st>>>(d, remap, a, b, out);
}

template <class Real>
void launch_accumulate2(int B, int n0, int n1, const Remap2<Real>* remap, const Vec4<Real>* a, const Vec4<Real>* b,
                        Vec4<Real>* out, cudaStream_t st) {
  k_accumulate2<Real><<<grid1((long long)n0 * n1, 256, B), 256, 0, st>>>(n0, n1, remap, a, b, out);
}

template <class Real>
void launch_output4(const BuildDims& d, const Remap4<Real>* remap, const Vec4<Real>* tab, float* out,
                    cudaStream_t st) {
  k_output4<Real><<<grid1(d.n4(), 256, d.B), 256, 0, st>>>(d, remap, tab, out);
}

template <class Real>
void launch_output2(int B, int n0, int n1, const Remap2<Real>* remap, const Vec4<Real>* tab, float* out,
                    cudaStream_t st) {
  k_output2<Real><<<grid1((long long)n0 * n1, 256, B), 256, 0, st>>>(n0, n1, remap, tab, out);
}

template <class Real>
void launch_add_to_sum(long long n4, int B, const Real* J, Vec4<float>* jsum, bool first, cudaStream_t st) {
  k_add_to_sum<Real><<<grid1(n4 * B, 256, 1), 256, 0, st>>>(n4, B, J, jsum, first);
}

template <class Real>
__global__ void k_export_planar(long long n4, int B, const Real* tab, float* out) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= n4 * B) return;
  const Real* src = tab + (t / n4) * 3 * n4 + t % n4;
  out[3 * t] = (float)src[0];
  out[3 * t + 1] = (float)src[n4];
  out[3 * t + 2] = (float)src[2 * n4];
}

template <class Real>
void launch_export_planar(long long n4, int B, const Real* tab, float* out, cudaStream_t st) {
  k_export_planar<Real><<<grid1(n4 * B, 256, 1), 256, 0, st>>>(n4, B, tab, out);
}

template <class Real>
void launch_export(long long n, const Vec4<Real>* tab, float* out, cudaStream_t st) {
  k_export<Real><<<grid1(n, 256, 1), 256, 0, st>>>(n, tab, out);
}

#define SFSIM_INSTANTIATE(Real)                                                                                     \
  template int launch_point_scatter<Real>(const AtmoParams*, const BuildDims&, const RowInfo*,                     \
                                          const SphereDir<Real>*, const unsigned char*, const int2*,               \
                                          const PointRow<Real>*, const CellGeom<Real>*, const Vec4<Real>*,         \
                                          const Vec4<Real>*, const Vec4<Real>*, Real*, Real*, cudaStream_t);       \
  template void launch_surface_radiance<Real>(const AtmoParams*, const BuildDims&, const SurfRow<Real>*,          \
                                              const HalfDir<Real>*, const Vec4<Real>*, const Vec4<Real>*,          \
                                              Vec4<Real>*, cudaStream_t);                                          \
  template int launch_ray_scatter<Real>(const AtmoParams*, const BuildDims&, const RowInfo*, const RowSample<Real>*, \
                                        const CellGeom<Real>*, const Remap4<Real>*, const Real*, Vec4<Real>*,      \
                                        cudaStream_t);                                                             \
  template void launch_accumulate4<Real>(const BuildDims&, const Remap4<Real>*, const Vec4<Real>*,                 \
                                         const Vec4<Real>*, Vec4<Real>*, cudaStream_t);                            \
  template void launch_accumulate2<Real>(int, int, int, const Remap2<Real>*, const Vec4<Real>*, const Vec4<Real>*, \
                                         Vec4<Real>*, cudaStream_t);                                               \
  template void launch_output4<Real>(const BuildDims&, const Remap4<Real>*, const Vec4<Real>*, float*,             \
                                     cudaStream_t);                                                                \
  template void launch_output2<Real>(int, int, int, const Remap2<Real>*, const Vec4<Real>*, float*, cudaStream_t);  \
  template void launch_export<Real>(long long, const Vec4<Real>*, float*, cudaStream_t);                           \
  template void launch_add_to_sum<Real>(long long, int, const Real*, Vec4<float>*, bool, cudaStream_t);           \
  template void launch_export_planar<Real>(long long, int, const Real*, float*, cudaStream_t);                      \
  template size_t point_scatter_smem<Real>(const BuildDims&, bool);                                                 \
  template size_t ray_scatter_smem<Real>(const BuildDims&);

SFSIM_INSTANTIATE(float)
SFSIM_INSTANTIATE(double)

}  // namespace sfsim
