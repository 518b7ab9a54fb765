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
  Real A[3], B[3], lo[3], hi[3], e0[3], e1[3];
  // height and sun elevation first, then elevation
  ld3(t, idx4(d, u0, u1, u2, a), A);
  ld3(t, idx4(d, u0, u1, v2, a), B);
  mix3(A, B, s2, lo);
  ld3(t, idx4(d, v0, u1, u2, a), A);
  ld3(t, idx4(d, v0, u1, v2, a), B);
  mix3(A, B, s2, hi);
  mix3(lo, hi, s0, e0);
  ld3(t, idx4(d, u0, v1, u2, a), A);
  ld3(t, idx4(d, u0, v1, v2, a), B);
  mix3(A, B, s2, lo);
  ld3(t, idx4(d, v0, v1, u2, a), A);
  ld3(t, idx4(d, v0, v1, v2, a), B);
  mix3(A, B, s2, hi);
  mix3(lo, hi, s0, e1);
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

// Direction vector and quadrature weight of a SphereDir in shared memory:
// one 16-byte broadcast load for FP32 entries.
template <class Real>
__device__ __forceinline__ void load_dir(const SphereDir<Real>& D, Real& x0, Real& x1, Real& x2, Real& weight) {
  x0 = D.w[0], x1 = D.w[1], x2 = D.w[2], weight = D.weight;
}
template <>
__device__ __forceinline__ void load_dir<float>(const SphereDir<float>& D, float& x0, float& x1, float& x2,
                                                float& weight) {
  static_assert(offsetof(SphereDir<float>, weight) == 12 && sizeof(SphereDir<float>) % 16 == 0, "layout");
  const float4 v = *reinterpret_cast<const float4*>(&D);
  x0 = v.x, x1 = v.y, x2 = v.z, weight = v.w;
}

template <class Real, bool FIRST>
__global__ void __launch_bounds__(256, 3) k_point_scatter(const AtmoParams* params, BuildDims d,
                                                          const RowInfo* rowinfo, const SphereDir<Real>* pdirs,
                                                          const int2* pcount, const PointRow<Real>* prow,
                                                          const CellGeom<Real>* geom,
                                                          const Vec4<Real>* dS, const Vec4<Real>* Mt,
                                                          const Vec4<Real>* dE, Vec4<Real>* J, int nchunks) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  using TR = TexelRow<Real>;
  constexpr int RS = TR::kStride;
  constexpr int DB = kDirBlock;
  const int b = blockIdx.y;
  const int chunk = blockIdx.x % nchunks;
  const int ik = blockIdx.x / nchunks;
  const int i = ik / d.n2, k = ik % d.n2;
  const AtmoParams& P = params[b];
  const PointRow<Real>* prk = prow + ((long long)b * d.n0 + i) * d.n2 + k;
  const int2 pc = pcount[(long long)b * d.n0 + i];
  const int sky_end = pc.x, used = pc.y;
  const int nrow = used * d.n3;
  SphereDir<Real>* dirs = reinterpret_cast<SphereDir<Real>*>(smem_raw);
  Real* rows = reinterpret_cast<Real*>(dirs + dir_row(d.P));
  Real* rowsM = rows + RS * nrow;
  Real* etab = rowsM + (FIRST ? RS * nrow : 0);

  // the (i, k) coordinates of the dS lookups
  const int u0 = prk->u0, u2 = prk->u2;
  const Real s0 = prk->s0, s2 = prk->s2;
  const int v0 = upper_index(u0, d.n0), v2 = upper_index(u2, d.n2);

  const long long base4 = (long long)b * d.n4();
  const SphereDir<Real>* src = pdirs + ((long long)b * d.n0 + i) * dir_row(d.P);
  for (int t = threadIdx.x; t < used; t += blockDim.x) dirs[t] = src[t];
  for (int t = threadIdx.x; t < nrow; t += blockDim.x) {
    const int w = t / d.n3, a = t - w * d.n3;
    Real v[3] = {0, 0, 0}, vm[3] = {0, 0, 0};
    if (!src[w].pad) {
      const int u1 = src[w].u1, v1 = upper_index(u1, d.n1);
      const Real s1 = src[w].s1;
      gather_heading_row(dS + base4, d, u0, v0, s0, u1, v1, s1, u2, v2, s2, a, v);
      if (FIRST) gather_heading_row(Mt + base4, d, u0, v0, s0, u1, v1, s1, u2, v2, s2, a, vm);
    }
    TR::store(rows, t, v);
    if (FIRST) TR::store(rowsM, t, vm);
  }
  const long long nE = d.nE();
  for (int t = threadIdx.x; t < nE; t += blockDim.x) {
    Real A[3];
    ld3(dE, b * nE + t, A);
    TR::store(etab, t, A);
  }
  __syncthreads();

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
  const int row_len = RS * d.n3;

  Real accR[3] = {0, 0, 0}, accM[3] = {0, 0, 0}, cR[3] = {0, 0, 0}, cM[3] = {0, 0, 0};
  Real ringR[3] = {0, 0, 0}, ringM[3] = {0, 0, 0};
  // One block of DB directions starting at w0 (all sky or all ground),
  // summed plainly into ringR/ringM.
  auto dir_block = [&](int w0, auto ground) {
    Real wRb = 0, wMb = 0;
    if (share && gpos < DB) {
      Real x0, x1, x2, wt;
      load_dir(dirs[w0 + gpos], x0, x1, x2, wt);
      const Real mu_v = fma(sv, x0, cv * x1);
      wRb = wt * phR(mu_v);
      wMb = wt * phM(mu_v);
    }
#pragma unroll
    for (int q = 0; q < DB; q++) {
      const SphereDir<Real>& D = dirs[w0 + q];
      Real x0, x1, x2, wt;
      load_dir(D, x0, x1, x2, wt);
      Real wR, wM;
      if (share) {
        wR = __shfl_sync(0xffffffffu, wRb, gbase + q);
        wM = __shfl_sync(0xffffffffu, wMb, gbase + q);
      } else {
        const Real mu_v = fma(sv, x0, cv * x1);
        wR = wt * phR(mu_v);
        wM = wt * phM(mu_v);
      }
      const Real mu_l = fma(x0, g.lx, fma(x1, g.ly, x2 * g.lz));
      // sun-angle coordinate of (omega, l) along the direction's heading row
      int u3;
      Real s3;
      split_coord_r<Real>(fma(scale3, mu_l, scale3), d.n3, &u3, &s3);
      const int v3 = upper_index(u3, d.n3);
      Real X[3], lo[3], hi[3];
      const Real* row_w = rows + (w0 + q) * row_len;
      TR::load(row_w, u3, lo);
      TR::load(row_w, v3, hi);
#pragma unroll
      for (int c = 0; c < 3; c++) X[c] = fma(hi[c] - lo[c], s3, lo[c]);
      if (FIRST) {
        const Real ph = phM(mu_l);
        const Real* rowM_w = rowsM + (w0 + q) * row_len;
        TR::load(rowM_w, u3, lo);
        TR::load(rowM_w, v3, hi);
#pragma unroll
        for (int c = 0; c < 3; c++) X[c] = fma(fma(hi[c] - lo[c], s3, lo[c]), ph, X[c]);
      }
      if (decltype(ground)::value) {
        const Real sg = fma(D.gdir[0], g.lx, fma(D.gdir[1], g.ly, D.gdir[2] * g.lz));
        int uE1;
        Real sE1;
        split_coord_r<Real>(sun_elevation_index_r<Real>(sg, scaleE), d.nE1, &uE1, &sE1);
        const int vE1 = upper_index(uE1, d.nE1), vE0 = upper_index(D.uE0, d.nE0);
        Real e00[3], e01[3], e10[3], e11[3], Y[3];
        TR::load(etab, D.uE0 * d.nE1 + uE1, e00);
        TR::load(etab, D.uE0 * d.nE1 + vE1, e01);
        TR::load(etab, vE0 * d.nE1 + uE1, e10);
        TR::load(etab, vE0 * d.nE1 + vE1, e11);
        mix4(e00, e01, e10, e11, D.sE0, sE1, Y);
#pragma unroll
        for (int c = 0; c < 3; c++) X[c] = fma(D.ground[c], Y[c], X[c]);
      }
#pragma unroll
      for (int c = 0; c < 3; c++) {
        ringR[c] = fma(wR, X[c], ringR[c]);
        ringM[c] = fma(wM, X[c], ringM[c]);
      }
    }
  };
  // the partial sums of up to two blocks go to the compensated totals
  auto flush = [&]() {
#pragma unroll
    for (int c = 0; c < 3; c++) {
      kahan_add(accR[c], cR[c], ringR[c]);
      kahan_add(accM[c], cM[c], ringM[c]);
      ringR[c] = ringM[c] = 0;
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
  if (!valid) return;
  // beta_c(x) (atmosphere.clj:42-47, 140-151)
  const PointRow<Real> pr = *prk;
  Vec4<Real> o;
  o.x = pr.bR[0] * accR[0] + pr.bM[0] * accM[0];
  o.y = pr.bR[1] * accR[1] + pr.bM[1] * accM[1];
  o.z = pr.bR[2] * accR[2] + pr.bM[2] * accM[2];
  o.w = 0;
  J[node] = o;
}

template <class Real>
size_t point_scatter_smem(const BuildDims& d, bool first) {
  return sizeof(SphereDir<Real>) * dir_row(d.P) +
         sizeof(Real) * 3 * ((size_t)dir_row(d.P) * d.n3 * (first ? 2 : 1) + d.nE());
}

template <class Real>
int launch_point_scatter(const AtmoParams* params, const BuildDims& d, const RowInfo* rowinfo,
                         const SphereDir<Real>* pdirs, const int2* pcount, const PointRow<Real>* prow,
                         const CellGeom<Real>* geom, const Vec4<Real>* dS, const Vec4<Real>* mie,
                         const Vec4<Real>* dE, Vec4<Real>* J, cudaStream_t st) {
  const int block = 256;
  const int nchunks = (d.n1 * d.n3 + block - 1) / block;
  const bool first = mie != nullptr;
  size_t smem = point_scatter_smem<Real>(d, first);
  dim3 grid((unsigned)(d.n0 * d.n2 * nchunks), d.B);
  if (first) {
    if (cudaFuncSetAttribute(k_point_scatter<Real, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess)
      return -1;
    k_point_scatter<Real, true><<<grid, block, smem, st>>>(params, d, rowinfo, pdirs, pcount, prow, geom, dS, mie,
                                                           dE, J, nchunks);
  } else {
    if (cudaFuncSetAttribute(k_point_scatter<Real, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem) != cudaSuccess)
      return -1;
    k_point_scatter<Real, false><<<grid, block, smem, st>>>(params, d, rowinfo, pdirs, pcount, prow, geom, dS,
                                                            mie, dE, J, nchunks);
  }
  return 0;
}

// ---------------------------------------------------------------------------
// Surface radiance dE (atmosphere.clj:225-230): integral over the upper half
// sphere of dS(x, w, l, above) (w.n); the reference passes the ray steps as
// the sphere steps (atmosphere_lut.clj:89).  One block per node, threads over
// directions, block reduction.  The per-node coordinates and the world-space
// directions come from FP64 setup tables, so no thread uses the FP64 pipe.
// ---------------------------------------------------------------------------

template <class Real, bool FIRST>
__global__ void __launch_bounds__(256) k_surface_radiance(const AtmoParams* params, BuildDims d,
                                                          const SurfRow<Real>* erow, const HalfDir<Real>* hdir,
                                                          const Vec4<Real>* dS, const Vec4<Real>* Mt,
                                                          Vec4<Real>* dE) {
  __shared__ Real red[3][256];
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
    split_coord_r<Real>(scale1 * (Real(0.5) - lq), d.n1, &uu[1], &sx[1]);
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
    k_surface_radiance<Real, true><<<grid, 256, 0, st>>>(params, d, erow, hdir, dS, mie, dE);
  else
    k_surface_radiance<Real, false><<<grid, 256, 0, st>>>(params, d, erow, hdir, dS, mie, dE);
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
// ---------------------------------------------------------------------------

// Per-sample constants, laid out so that FP32 blocks read each group with
// one 16-byte broadcast load: {T, us} and {inv_r, -, s0, s1} for the
// nodes, {s0, s1} and the J offsets for the plane build.
template <class Real>
struct RaySample {
  Real T[3], us;
  Real inv_r, unused, s0, s1;
  int p00, p01, p10, p11;  // J offsets of the four (height, elevation) planes
};

template <class Real>
struct SampleView {
  Real T[3], us, inv_r;
  __device__ __forceinline__ SampleView(const RaySample<Real>& v) {
    T[0] = v.T[0], T[1] = v.T[1], T[2] = v.T[2], us = v.us, inv_r = v.inv_r;
  }
};
template <>
struct SampleView<float> {
  float T[3], us, inv_r;
  __device__ __forceinline__ SampleView(const RaySample<float>& v) {
    const float4 a = *reinterpret_cast<const float4*>(&v);
    T[0] = a.x, T[1] = a.y, T[2] = a.z, us = a.w;
    inv_r = v.inv_r;
  }
};

template <class Real>
struct SampleCorners {
  int p[4];
  Real s0, s1;
  __device__ __forceinline__ SampleCorners(const RaySample<Real>& v) {
    p[0] = v.p00, p[1] = v.p01, p[2] = v.p10, p[3] = v.p11, s0 = v.s0, s1 = v.s1;
  }
};
template <>
struct SampleCorners<float> {
  int p[4];
  float s0, s1;
  __device__ __forceinline__ SampleCorners(const RaySample<float>& v) {
    static_assert(sizeof(RaySample<float>) == 48 && offsetof(RaySample<float>, p00) == 32, "layout");
    const int4 o = *reinterpret_cast<const int4*>(&v.p00);
    const float2 f = *reinterpret_cast<const float2*>(&v.s0);
    p[0] = o.x, p[1] = o.y, p[2] = o.z, p[3] = o.w, s0 = f.x, s1 = f.y;
  }
};

// Four FP32 blocks fit in shared memory; the hint keeps ptxas from trading
// registers for spills below that.
constexpr int ray_scatter_min_blocks(size_t real_size) { return real_size == 4 ? 4 : 1; }

template <class Real, int CH>
__global__ void __launch_bounds__(256, ray_scatter_min_blocks(sizeof(Real)))
    k_ray_scatter(const AtmoParams* params, BuildDims d, const RowInfo* rowinfo, const RowSample<Real>* rows,
                  const CellGeom<Real>* geom, const Remap4<Real>* remap, const Vec4<Real>* J, Vec4<Real>* dS) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int b = blockIdx.y;
  const long long row = blockIdx.x;
  const long long nrows = d.rows();
  const int ncell = d.n2 * d.n3;
  RaySample<Real>* smp = reinterpret_cast<RaySample<Real>*>(smem_raw);
  Real* plane = reinterpret_cast<Real*>(smp + CH);
  const RowSample<Real>* rs = rows + (b * nrows + row) * d.S;
  const RowInfo ri = rowinfo[b * nrows + row];
  const Vec4<Real>* tJ = J + (long long)b * d.n4();
  const long long node0 = (b * nrows + row) * ncell;
  const Real scale2 = Bulk<Real>::sun_scale(d);
  const RowR<Real> rw = row_r<Real>(ri);
  const Real rr = rw.r, D0 = rw.D[0], D1 = rw.D[1], D2 = rw.D[2];
  const int n3x3 = 3 * d.n3;

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
      o3u = 3 * m.u[3];
      o3v = 3 * upper_index(m.u[3], d.n3);
      s3 = m.s[3];
    }
    Real acc[2][3] = {{0, 0, 0}, {0, 0, 0}};
    for (int sb = 0; sb < d.S; sb += CH) {
      const int nch = min(CH, d.S - sb);
      __syncthreads();
      if (threadIdx.x < nch) {
        const RowSample<Real> q = rs[sb + threadIdx.x];
        RaySample<Real> v;
        v.T[0] = exp_neg(q.tau[0]);
        v.T[1] = exp_neg(q.tau[1]);
        v.T[2] = exp_neg(q.tau[2]);
        v.us = q.us;
        v.inv_r = q.inv_r;
        v.unused = 0;
        v.s0 = q.s0;
        v.s1 = q.s1;
        const int v0 = upper_index(q.u0, d.n0), v1 = upper_index(q.u1, d.n1);
        v.p00 = (q.u0 * d.n1 + q.u1) * ncell;
        v.p01 = (q.u0 * d.n1 + v1) * ncell;
        v.p10 = (v0 * d.n1 + q.u1) * ncell;
        v.p11 = (v0 * d.n1 + v1) * ncell;
        smp[threadIdx.x] = v;
      }
      __syncthreads();
      for (int ch = 0; ch < nch; ch++) {
        const SampleCorners<Real> v(smp[ch]);
        for (int t = threadIdx.x; t < ncell; t += blockDim.x) {
          Real A[3], B[3], lo[3], hi[3];
          ld3(tJ, (long long)v.p[0] + t, A);
          ld3(tJ, (long long)v.p[1] + t, B);
#pragma unroll
          for (int c = 0; c < 3; c++) lo[c] = fma(B[c] - A[c], v.s1, A[c]);
          ld3(tJ, (long long)v.p[2] + t, A);
          ld3(tJ, (long long)v.p[3] + t, B);
#pragma unroll
          for (int c = 0; c < 3; c++) hi[c] = fma(B[c] - A[c], v.s1, A[c]);
          Real* dst = plane + 3 * (ch * ncell + t);
#pragma unroll
          for (int c = 0; c < 3; c++) dst[c] = fma(hi[c] - lo[c], v.s0, lo[c]);
        }
      }
      __syncthreads();
      if (active) {
        // samples alternate between two sums for independent FMA chains
        auto sample = [&](int ch, Real(&a)[3]) {
          const SampleView<Real> v(smp[ch]);
          const Real sin_el = fma(v.us, Dl, b0) * v.inv_r;  // p_s.l / |p_s|
          int u2;
          Real s2;
          split_coord_r<Real>(sun_elevation_index_r<Real>(sin_el, scale2), d.n2, &u2, &s2);
          const Real* lo = plane + 3 * ch * ncell + u2 * n3x3;
          const Real* hi = u2 + 1 < d.n2 ? lo + n3x3 : lo;
#pragma unroll
          for (int c = 0; c < 3; c++) {
            const Real x0 = fma(lo[o3v + c] - lo[o3u + c], s3, lo[o3u + c]);
            const Real x1 = fma(hi[o3v + c] - hi[o3u + c], s3, hi[o3u + c]);
            a[c] = fma(v.T[c], fma(x1 - x0, s2, x0), a[c]);
          }
        };
        int ch = 0;
        for (; ch + 1 < nch; ch += 2) {
          sample(ch, acc[0]);
          sample(ch + 1, acc[1]);
        }
        if (ch < nch) sample(ch, acc[0]);
      }
    }
    if (active) {
      const Real w = rw.Ls;
      Vec4<Real> o;
      o.x = w * (acc[0][0] + acc[1][0]);
      o.y = w * (acc[0][1] + acc[1][1]);
      o.z = w * (acc[0][2] + acc[1][2]);
      o.w = 0;
      dS[node0 + cell] = o;
    }
  }
}

template <class Real>
int launch_ray_scatter(const AtmoParams* params, const BuildDims& d, const RowInfo* rowinfo,
                       const RowSample<Real>* rows, const CellGeom<Real>* geom, const Remap4<Real>* remap,
                       const Vec4<Real>* J, Vec4<Real>* dS, cudaStream_t st) {
  constexpr int CH = 16;
  const int ncell = d.n2 * d.n3;
  const int block = ncell >= 256 ? 256 : ((ncell + 31) / 32) * 32;
  size_t smem = sizeof(RaySample<Real>) * CH + sizeof(Real) * 3 * (size_t)CH * ncell;
  if (cudaFuncSetAttribute(k_ray_scatter<Real, CH>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
      cudaSuccess)
    return -1;
  dim3 grid((unsigned)d.rows(), d.B);
  k_ray_scatter<Real, CH><<<grid, block, smem, st>>>(params, d, rowinfo, rows, geom, remap, J, dS);
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
  interp4(A + b * n4, d, m.u, m.s, va);
  if (Bt) interp4(Bt + b * n4, d, m.u, m.s, vb);
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
  interp4(tab + b * n4, d, m.u, m.s, v);
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
__global__ void k_add_to_sum(long long n, const Vec4<Real>* J, Vec4<float>* jsum, bool first) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= n) return;
  const Vec4<Real> v = J[t];
  Vec4<float> o;
  if (first) {
    o.x = (float)v.x;
    o.y = (float)v.y;
    o.z = (float)v.z;
  } else {
    o = jsum[t];
    o.x += (float)v.x;
    o.y += (float)v.y;
    o.z += (float)v.z;
  }
  o.w = 0;
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
void launch_add_to_sum(long long n, const Vec4<Real>* J, Vec4<float>* jsum, bool first, cudaStream_t st) {
  k_add_to_sum<Real><<<grid1(n, 256, 1), 256, 0, st>>>(n, J, jsum, first);
}

template <class Real>
void launch_export(long long n, const Vec4<Real>* tab, float* out, cudaStream_t st) {
  k_export<Real><<<grid1(n, 256, 1), 256, 0, st>>>(n, tab, out);
}

#define SFSIM_INSTANTIATE(Real)                                                                                     \
  template int launch_point_scatter<Real>(const AtmoParams*, const BuildDims&, const RowInfo*,                     \
                                          const SphereDir<Real>*, const int2*, const PointRow<Real>*,              \
                                          const CellGeom<Real>*, const Vec4<Real>*, const Vec4<Real>*,             \
                                          const Vec4<Real>*, Vec4<Real>*, cudaStream_t);                           \
  template void launch_surface_radiance<Real>(const AtmoParams*, const BuildDims&, const SurfRow<Real>*,          \
                                              const HalfDir<Real>*, const Vec4<Real>*, const Vec4<Real>*,          \
                                              Vec4<Real>*, cudaStream_t);                                          \
  template int launch_ray_scatter<Real>(const AtmoParams*, const BuildDims&, const RowInfo*, const RowSample<Real>*, \
                                        const CellGeom<Real>*, const Remap4<Real>*, const Vec4<Real>*,             \
                                        Vec4<Real>*, cudaStream_t);                                                \
  template void launch_accumulate4<Real>(const BuildDims&, const Remap4<Real>*, const Vec4<Real>*,                 \
                                         const Vec4<Real>*, Vec4<Real>*, cudaStream_t);                            \
  template void launch_accumulate2<Real>(int, int, int, const Remap2<Real>*, const Vec4<Real>*, const Vec4<Real>*, \
                                         Vec4<Real>*, cudaStream_t);                                               \
  template void launch_output4<Real>(const BuildDims&, const Remap4<Real>*, const Vec4<Real>*, float*,             \
                                     cudaStream_t);                                                                \
  template void launch_output2<Real>(int, int, int, const Remap2<Real>*, const Vec4<Real>*, float*, cudaStream_t);  \
  template void launch_export<Real>(long long, const Vec4<Real>*, float*, cudaStream_t);                           \
  template void launch_add_to_sum<Real>(long long, const Vec4<Real>*, Vec4<float>*, bool, cudaStream_t);            \
  template size_t point_scatter_smem<Real>(const BuildDims&, bool);

SFSIM_INSTANTIATE(float)
SFSIM_INSTANTIATE(double)

}  // namespace sfsim
