// k_first_order.cu -- first-order Rayleigh ray scatter and Mie strength,
// atmosphere_lut.clj:68-78 with atmosphere.clj:154-200.
//
// For a 4-D node (x, v, l, above) the reference integrates, over the S
// midpoint samples p_s of the view ray from x to its extremity,
//   T(x, p_s) * beta_c(p_s) * [phase_c(v.l)] * I * T(p_s, l)   (sun above p_s's horizon)
// once for Rayleigh (with phase) and once for the Mie strength (no phase).
// Both share T(x, p_s) and T(p_s, l); this kernel evaluates them once.
//
// Mapping: one block per view row (height i, elevation j).  The row's S
// samples (positions, T(x, p_s), the heights' exponentials) come from
// k_view_rows and sit in shared memory, and so do the row's cells' light
// directions when the block forms them itself (CELLS).  Each warp takes one cell (sun
// elevation k, sun heading a) at a time and its lanes take the samples: a
// lane integrates the optical depth of the sun ray from its p_s (S midpoint
// samples, FP32, compensated sums), and the warp reduces the samples with
// shuffles.  Shadowed samples form contiguous runs along a ray, so lanes of a
// warp mostly agree on whether to integrate.
//
// FP32 builds read every sun ray's optical depths from two tables of the
// same S-sample midpoint sums, both evaluated by k_sun_table:
//  * a climbing ray (p_s.l >= 0) from a 2048 x 2048 grid of (sqrt(q / q_top),
//    the exit distance between its zenith and horizontal values), sums
//    interpolated bilinearly: its integrand falls monotonically, so the sums
//    are smooth in those coordinates (transmittance error below 1e-5), except
//    in the top eight rows of an atmosphere dense at the top (the reference's
//    35 km one), whose rays are integrated directly;
//  * a descending ray (p_s.l < 0) from a 1024 x 2048 grid of (perigee height
//    / H, asinh(d / s) / asinh(dmax / s)), d the distance from p_s to the
//    perigee, dmax that from the perigee to the exit, s = 1.2 sqrt(2 R H_mie).
//    What is stored is log2 of the mean density along the ray, sum / S, whose
//    bilinear interpolation is smooth even at the perigee's density peak and
//    stays finite for the short rays near the top; the optical depth is the
//    exit distance times 2^interpolated.  A numpy model of the same sums put
//    the optical-depth error at <= 3e-6 (FP32 storage included) over Earth,
//    the reference's 35 km atmosphere and the sweep's extremes (radius 3000
//    and 7000 km, Mie scale heights 0.8 and 2 km).
// A table of paired texels (kSunPairClimb, kSunPairDesc) is read with one
// aligned 16-byte load per row of a bilinear lookup.
#include "atmo_device.cuh"
#include "kernels.h"

namespace sfsim {

template <class Real>
struct FirstOrderSmem {
  Real tau[3];
  Real er, em, q, us;
};

// Shared memory of a first-order block: the row's samples, then (when the
// block forms its cells' light directions itself) one CellGeom per cell.
template <class Real>
size_t first_order_smem(const BuildDims& d, bool cells) {
  const size_t samples = (sizeof(FirstOrderSmem<Real>) * d.S + 15) & ~size_t(15);
  return samples + (cells ? sizeof(CellGeom<Real>) * d.n2 * d.n3 : 0);
}
template size_t first_order_smem<float>(const BuildDims&, bool);
template size_t first_order_smem<double>(const BuildDims&, bool);

// Horizon test of the sun at p_s (atmosphere.clj:95-102, filtered-sun-light
// :154-160) from b = p_s.l and q = |p_s|^2 - R^2.  Near the boundary FP32
// inputs cannot decide (b carries ~1 m of rounding), so the test is repeated
// in FP64 on p_s as integral-ray forms it (ray.clj:22-24).
template <class Real>
__device__ __forceinline__ bool sun_visible(const AtmoParams& P, const BuildDims& d, const RowInfo& ri, Real bp,
                                            Real q, int cell, int s) {
  bool lit = (bp >= Real(0)) || (bp * bp <= q);
  if (std::is_same<Real, float>::value) {
    const Real m = bp * bp - q;
    if ((bp < Real(4)) && (fabs(m) < Real(1.0e8) || (bp > Real(-4) && q < Real(1.0e8)))) {
      const d3 l = light_direction(d, ri.sv, ri.cv, cell / d.n3, cell % d.n3);
      const d3 p = add3(mk3(ri.r, 0, 0), mul3(mk3(ri.D[0], ri.D[1], ri.D[2]), (0.5 + s) * (1.0 / d.S)));
      lit = is_above_horizon(P, p, l);
    }
  }
  return lit;
}

template <class Real>
__device__ __forceinline__ Real warp_sum(Real v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// ---- sun-ray optical-depth table (FP32 builds) ----

// Node (i, j) of the table: q = (i / (NR - 1))^2 q_top and the exit distance
// d = dmin + (j / (NM - 1)) (dh - dmin) between the zenith (dmin = top - r)
// and horizontal (dh = sqrt(top^2 - r^2)) exits; p.l follows from
// top^2 = r^2 + 2 d (p.l) + d^2.  Stored: dt * sum exp2 of the Rayleigh and
// Mie exponents (dt = d / S), the quantities k_first_order integrates.
//
// Descending rays, node (i, j) at kSunNR * kSunNM + i * kDescNY + j: perigee
// height h* = (i / (NX - 1)) H (q* = h* (2 R + h*)), dmax = sqrt(q_top - q*),
// the distance d = s sinh((j / (NY - 1)) asinh(dmax / s)) before the perigee;
// the ray starts at q = q* + d^2 with p.l = -d and leaves after d + dmax.
// Stored: log2 of sum / S for Rayleigh and Mie (the row h* = H holds the
// density at the top: all S samples of a zero-length ray sit at its start).
__device__ __forceinline__ void desc_table_node(const AtmoParams& P, int S, int i, int j, float2* out) {
  const float Hh2 = P.f_Hh2;
  const float hs = (float)i / (float)(kDescNX - 1) * P.f_H;
  const float qs = hs * (2.0f * P.f_R + hs);
  const float dmax = sqrtf(fmaxf(Hh2 - qs, 0.0f));
  const float y = (float)j / (float)(kDescNY - 1);
  const float d = fminf(P.f_desc_s * sinhf(y * asinhf(dmax * P.f_desc_inv_s)), dmax);
  const float q0 = fmaf(d, d, qs);
  const float dt = (d + dmax) / (float)S;
  constexpr int NP = Bulk<float>::kSunNP;
  float hc[NP];
#pragma unroll
  for (int c = 0; c < NP; c++) hc[c] = Bulk<float>::hpr(P)[c];
  float sr, smie;
  sun_sums<float, NP>(q0, -d, dt, S, hc, Bulk<float>::alpha(P), Bulk<float>::beta(P), Bulk<float>::hratio(P), sr,
                      smie);
  // 2^-126 keeps the logarithm finite where the density underflows
  const float inv_s = 1.0f / (float)S;
  *out = make_float2(log2f(fmaxf(sr * inv_s, 1.17549435e-38f)), log2f(fmaxf(smie * inv_s, 1.17549435e-38f)));
}

// Node value v at column j (of `width`) of entry `idx` of a table.  Paired:
// entry idx holds (v(j), v(j + 1)) as one 16-byte float4, so a bilinear
// lookup reads each of its two rows with one aligned load from one 32-byte
// sector; v goes to entry idx's first half and entry idx - 1's second (the
// last entry of a row repeats v there, never read).  Otherwise entry idx is v.
template <bool PAIRED>
__device__ __forceinline__ void store_node(unsigned char* tab, long long idx, int j, int width, float2 v) {
  if (PAIRED) {
    float2* e = reinterpret_cast<float2*>(reinterpret_cast<float4*>(tab) + idx);
    e[0] = v;
    if (j > 0) e[-1] = v;
    if (j == width - 1) e[1] = v;
  } else {
    reinterpret_cast<float2*>(tab)[idx] = v;
  }
}

// The four texels of the bilinear footprint at entry idx of a table of rows
// of `width`.
template <bool PAIRED>
__device__ __forceinline__ void load_footprint(const unsigned char* tab, long long idx, int width, float2& v00,
                                               float2& v01, float2& v10, float2& v11) {
  if (PAIRED) {
    const float4* p = reinterpret_cast<const float4*>(tab) + idx;
    const float4 e0 = __ldg(p), e1 = __ldg(p + width);
    v00 = make_float2(e0.x, e0.y);
    v01 = make_float2(e0.z, e0.w);
    v10 = make_float2(e1.x, e1.y);
    v11 = make_float2(e1.z, e1.w);
  } else {
    const float2* p = reinterpret_cast<const float2*>(tab) + idx;
    v00 = __ldg(p);
    v01 = __ldg(p + 1);
    v10 = __ldg(p + width);
    v11 = __ldg(p + width + 1);
  }
}

__global__ void k_sun_table(const AtmoParams* params, int S, unsigned char* table) {
  const int b = blockIdx.y;
  const AtmoParams& P = params[b];
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= kSunTableLen) return;
  unsigned char* tab = table + (size_t)b * kSunTableBytes;
  if (t >= (long long)kSunNR * kSunNM) {
    const int u = (int)(t - (long long)kSunNR * kSunNM);
    const int i = u / kDescNY, j = u - i * kDescNY;
    float2 v;
    desc_table_node(P, S, i, j, &v);
    store_node<kSunPairDesc>(tab + kSunClimbBytes, u, j, kDescNY, v);
    return;
  }
  const int i = (int)t / kSunNM, j = (int)t - ((int)t / kSunNM) * kSunNM;
  const float Hh2 = P.f_Hh2, R2 = P.f_R * P.f_R, top = P.f_top;
  const float xr = (float)i / (float)(kSunNR - 1), xm = (float)j / (float)(kSunNM - 1);
  const float q = xr * xr * Hh2;
  const float cq = fmaxf(Hh2 - q, 0.0f);  // top^2 - r^2
  const float r = sqrtf(R2 + q);
  const float dmin = cq / (top + r), dh = sqrtf(cq);
  const float dist = fmaf(xm, dh - dmin, dmin);
  float2 out = make_float2(0.0f, 0.0f);
  if (dist > 0.0f) {
    const float bp = (cq - dist * dist) / (2.0f * dist);
    constexpr int NP = Bulk<float>::kSunNP;
    float hc[NP];
#pragma unroll
    for (int c = 0; c < NP; c++) hc[c] = Bulk<float>::hpr(P)[c];
    const float dt = dist / (float)S;
    float sr, smie;
    sun_sums<float, NP>(q, bp, dt, S, hc, Bulk<float>::alpha(P), Bulk<float>::beta(P), Bulk<float>::hratio(P), sr,
                        smie);
    out = make_float2(dt * sr, dt * smie);
  }
  store_node<kSunPairClimb>(tab, t, j, kSunNM, out);
}

void launch_sun_table(const AtmoParams* params, const BuildDims& d, unsigned char* table, cudaStream_t st) {
  dim3 grid((unsigned)((kSunTableLen + 255) / 256), d.B);
  k_sun_table<<<grid, 256, 0, st>>>(params, d.S, table);
}

// Bilinear lookup of the table at (q, exit distance) for a climbing ray.
__device__ __forceinline__ float2 sun_lookup(const unsigned char* __restrict__ tab, const AtmoParams& P, float q,
                                             float texit) {
  const float Hh2 = P.f_Hh2, R2 = P.f_R * P.f_R, top = P.f_top;
  const float qc = fminf(fmaxf(q, 0.0f), Hh2);
  const float cq = Hh2 - qc;
  const float r = sqrtf(R2 + qc);
  const float dmin = cq / (top + r), dh = sqrtf(cq);
  const float span = dh - dmin;
  const float xm = span > 0.0f ? fminf(fmaxf((texit - dmin) / span, 0.0f), 1.0f) : 0.0f;
  const float xr = sqrtf(qc / Hh2);
  const float fi = xr * (float)(kSunNR - 1), fj = xm * (float)(kSunNM - 1);
  const int i0 = min((int)fi, kSunNR - 2), j0 = min((int)fj, kSunNM - 2);
  const float a = fi - (float)i0, c = fj - (float)j0;
  float2 v00, v01, v10, v11;
  load_footprint<kSunPairClimb>(tab, (long long)i0 * kSunNM + j0, kSunNM, v00, v01, v10, v11);
  const float w00 = (1.0f - a) * (1.0f - c), w01 = (1.0f - a) * c, w10 = a * (1.0f - c), w11 = a * c;
  return make_float2(w00 * v00.x + w01 * v01.x + w10 * v10.x + w11 * v11.x,
                     w00 * v00.y + w01 * v01.y + w10 * v10.y + w11 * v11.y);
}

// Optical depths of a descending ray (bp = p.l < 0) from q = |p|^2 - R^2 and
// its exit distance texit = d + dmax, from the descending table.
__device__ __forceinline__ float2 sun_lookup_desc(const unsigned char* __restrict__ tab, const AtmoParams& P,
                                                  float q, float bp, float texit) {
  const float R = P.f_R;
  const float qs = fmaxf(fmaf(-bp, bp, q), 0.0f);
  const float hs = qs / (R + sqrtf(fmaf(R, R, qs)));
  const float dmax = sqrtf(fmaxf(P.f_Hh2 - qs, 0.0f));
  const float den = asinhf(dmax * P.f_desc_inv_s);
  const float x = fminf(hs / P.f_H, 1.0f);
  const float y = den > 0.0f ? fminf(asinhf(-bp * P.f_desc_inv_s) / den, 1.0f) : 0.0f;
  const float fi = x * (float)(kDescNX - 1), fj = y * (float)(kDescNY - 1);
  const int i0 = min((int)fi, kDescNX - 2), j0 = min((int)fj, kDescNY - 2);
  const float a = fi - (float)i0, c = fj - (float)j0;
  float2 v00, v01, v10, v11;
  load_footprint<kSunPairDesc>(tab, (long long)i0 * kDescNY + j0, kDescNY, v00, v01, v10, v11);
  const float w00 = (1.0f - a) * (1.0f - c), w01 = (1.0f - a) * c, w10 = a * (1.0f - c), w11 = a * c;
  const float lr = w00 * v00.x + w01 * v01.x + w10 * v10.x + w11 * v11.x;
  const float lm = w00 * v00.y + w01 * v01.y + w10 * v10.y + w11 * v11.y;
  return make_float2(texit * Bulk<float>::exp2(lr), texit * Bulk<float>::exp2(lm));
}

// CELLS: the block forms its cells' light directions (node_light, as
// k_remap4 does) in shared memory instead of reading them from `geom`, so
// that the first order need not wait for k_remap4.
template <class Real, int WARPS, bool CELLS>
__global__ void __launch_bounds__(WARPS * 32, 4) k_first_order(const AtmoParams* params, BuildDims d,
                                                            const RowInfo* rowinfo, const RowSample<Real>* rows,
                                                            const CellGeom<Real>* geom, const PointRow<Real>* prow,
                                                            const double* hdvs, const unsigned char* sun_table,
                                                            Vec4<Real>* rayleigh, Vec4<Real>* mie) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  FirstOrderSmem<Real>* sm = reinterpret_cast<FirstOrderSmem<Real>*>(smem_raw);
  const int b = blockIdx.y;
  const long long row = blockIdx.x;
  const long long nrows = d.rows();
  const AtmoParams& P = params[b];
  const int S = d.S;
  const int ncell = d.n2 * d.n3;
  const RowInfo ri = rowinfo[b * nrows + row];
  CellGeom<Real>* cg = reinterpret_cast<CellGeom<Real>*>(
      smem_raw + ((sizeof(FirstOrderSmem<Real>) * S + 15) & ~size_t(15)));
  if (CELLS) {
    const PointRow<Real>* pr = prow + ((long long)b * d.n0 + row / d.n1) * d.n2;
    for (int c = threadIdx.x; c < ncell; c += blockDim.x) {
      const int k = c / d.n3, a = c - k * d.n3;
      cg[c] = cell_geom<Real>(ri.sv, ri.cv, node_light(ri.sv, ri.cv, pr[k].ss, pr[k].cs, hdvs[a]));
    }
  }
  const RowSample<Real>* rs = rows + (b * nrows + row) * S;
  for (int s = threadIdx.x; s < S; s += blockDim.x) {
    RowSample<Real> v = rs[s];
    sm[s].tau[0] = v.tau[0];
    sm[s].tau[1] = v.tau[1];
    sm[s].tau[2] = v.tau[2];
    sm[s].er = v.er;
    sm[s].em = v.em;
    sm[s].q = v.q;
    sm[s].us = v.us;
  }
  __syncthreads();

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const Real Hh2 = std::is_same<Real, float>::value ? (Real)P.f_Hh2 : (Real)P.Hh2;
  // climbing rays from the top rows of the climbing table, where its
  // interpolation fails for atmospheres dense at the top, are integrated
  // directly (AtmoParams::f_sun_qlim)
  const Real qlim = (Real)P.f_sun_qlim;
  constexpr int NP = Bulk<Real>::kSunNP;
  const Real* hp = Bulk<Real>::hpr(P);
  Real hc[NP];
#pragma unroll
  for (int c = 0; c < NP; c++) hc[c] = hp[c];
  const Real alpha = Bulk<Real>::alpha(P), beta = Bulk<Real>::beta(P);
  const Real ratio = Bulk<Real>::hratio(P);
  Real rext[3], mext[3];
#pragma unroll
  for (int c = 0; c < 3; c++) {
    rext[c] = Bulk<Real>::ray_ext(P, c);
    mext[c] = Bulk<Real>::mie_ext(P, c);
  }
  const Real inv_steps = Real(1) / Real(S);
  const RowR<Real> rw = row_r<Real>(ri);
  const Real rr = rw.r, D0 = rw.D[0], D1 = rw.D[1], D2 = rw.D[2];
  const PhaseCS<Real> phase_ray(Bulk<Real>::phase_ray(P));
  const long long node0 = (b * nrows + row) * ncell;
  const unsigned char* tab = sun_table ? sun_table + (size_t)b * kSunTableBytes : nullptr;

  for (int cell = warp; cell < ncell; cell += WARPS) {
    const CellGeom<Real> g = CELLS ? cg[cell] : geom[node0 + cell];
    const Real b0 = rr * g.lx;  // x.l, x = (r, 0, 0)
    const Real Dl = D0 * g.lx + D1 * g.ly + D2 * g.lz;
    Real accR[3] = {0, 0, 0}, accM[3] = {0, 0, 0};
    for (int s = lane; s < S; s += 32) {
      const Real q = sm[s].q;
      const Real bp = fma(sm[s].us, Dl, b0);  // p_s.l
      if (sun_visible<Real>(P, d, ri, bp, q, cell, s)) {
        // exit of the sun ray from the top sphere, cancellation-free
        const Real ctop = q - Hh2;
        const Real disc = fmax(bp * bp - ctop, Real(0));
        const Real root = Bulk<Real>::sqrt(disc);
        Real texit = bp >= Real(0) ? Bulk<Real>::div(-ctop, bp + root) : root - bp;
        texit = fmax(texit, Real(0));
        Real odr, odm;
        if (std::is_same<Real, float>::value && tab && (bp < Real(0) || q < qlim)) {
          const float2 od = bp >= Real(0) ? sun_lookup(tab, P, (float)q, (float)texit)
                                          : sun_lookup_desc(tab + kSunClimbBytes, P, (float)q, (float)bp,
                                                            (float)texit);
          odr = (Real)od.x;
          odm = (Real)od.y;
        } else {
          const Real dt = texit * inv_steps;
          Real sr, smie;
          sun_sums<Real, NP>(q, bp, dt, S, hc, alpha, beta, ratio, sr, smie);
          odr = dt * sr;
          odm = dt * smie;
        }
#pragma unroll
        for (int c = 0; c < 3; c++) {
          const Real tau = sm[s].tau[c] + (rext[c] * odr + mext[c] * odm);
          const Real T = exp_neg(tau);
          accR[c] = fma(T, sm[s].er, accR[c]);
          accM[c] = fma(T, sm[s].em, accM[c]);
        }
      }
    }
#pragma unroll
    for (int c = 0; c < 3; c++) {
      accR[c] = warp_sum(accR[c]);
      accM[c] = warp_sum(accM[c]);
    }
    if (lane == 0) {
      const Real wR = rw.Ls;
      const Real phR = phase_ray(g.mu);
      Vec4<Real> o1, o2;
      o1.x = wR * phR * Bulk<Real>::src_ray(P, 0) * accR[0];
      o1.y = wR * phR * Bulk<Real>::src_ray(P, 1) * accR[1];
      o1.z = wR * phR * Bulk<Real>::src_ray(P, 2) * accR[2];
      o1.w = 0;
      o2.x = wR * Bulk<Real>::src_mie(P, 0) * accM[0];
      o2.y = wR * Bulk<Real>::src_mie(P, 1) * accM[1];
      o2.z = wR * Bulk<Real>::src_mie(P, 2) * accM[2];
      o2.w = 0;
      rayleigh[node0 + cell] = o1;
      mie[node0 + cell] = o2;
    }
  }
}

template <class Real>
int launch_first_order(const AtmoParams* params, const BuildDims& d, const RowInfo* rowinfo,
                       const RowSample<Real>* rows, const CellGeom<Real>* geom, const PointRow<Real>* prow,
                       const double* hdvs, const unsigned char* sun_table, Vec4<Real>* rayleigh, Vec4<Real>* mie,
                       cudaStream_t st) {
  constexpr int WARPS = 8;
  const bool cells = geom == nullptr;
  const size_t smem = first_order_smem<Real>(d, cells);
  auto kernel = cells ? k_first_order<Real, WARPS, true> : k_first_order<Real, WARPS, false>;
  // more than 48 KB (long rows, S > 1755 in FP32, > 877 in FP64) needs the opt-in
  if (smem > 48 * 1024 &&
      cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return -1;
  dim3 grid((unsigned)d.rows(), d.B);
  kernel<<<grid, WARPS * 32, smem, st>>>(params, d, rowinfo, rows, geom, prow, hdvs, sun_table, rayleigh, mie);
  return 0;
}

template int launch_first_order<float>(const AtmoParams*, const BuildDims&, const RowInfo*, const RowSample<float>*,
                                       const CellGeom<float>*, const PointRow<float>*, const double*,
                                       const unsigned char*, Vec4<float>*, Vec4<float>*, cudaStream_t);
template int launch_first_order<double>(const AtmoParams*, const BuildDims&, const RowInfo*,
                                        const RowSample<double>*, const CellGeom<double>*, const PointRow<double>*,
                                        const double*, const unsigned char*, Vec4<double>*, Vec4<double>*,
                                        cudaStream_t);

// Work census of the first order: count[0] = the (node, sample) pairs whose
// sun is above the horizon (sun-ray optical depths the reference integrates,
// each of S extinction samples), count[1] = those whose sun ray climbs
// (p_s.l >= 0; FP32 builds read them from the sun table).
template <class Real>
__global__ void k_first_order_census(const AtmoParams* params, BuildDims d, const RowInfo* rowinfo,
                                     const RowSample<Real>* rows, const CellGeom<Real>* geom,
                                     unsigned long long* count) {
  const int b = blockIdx.y;
  const long long row = blockIdx.x;
  const long long nrows = d.rows();
  const AtmoParams& P = params[b];
  const RowInfo ri = rowinfo[b * nrows + row];
  const RowSample<Real>* rs = rows + (b * nrows + row) * d.S;
  const int ncell = d.n2 * d.n3;
  const long long node0 = (b * nrows + row) * ncell;
  unsigned long long local = 0, climb = 0;
  for (long long t = threadIdx.x; t < (long long)ncell * d.S; t += blockDim.x) {
    const int cell = (int)(t / d.S), s = (int)(t % d.S);
    const CellGeom<Real> g = geom[node0 + cell];
    const Real Dl = (Real)ri.D[0] * g.lx + (Real)ri.D[1] * g.ly + (Real)ri.D[2] * g.lz;
    const Real bp = fma(rs[s].us, Dl, (Real)ri.r * g.lx);
    const bool lit = sun_visible<Real>(P, d, ri, bp, rs[s].q, cell, s);
    local += lit ? 1 : 0;
    climb += (lit && bp >= Real(0)) ? 1 : 0;
  }
  for (int o = 16; o > 0; o >>= 1) {
    local += __shfl_xor_sync(0xffffffffu, local, o);
    climb += __shfl_xor_sync(0xffffffffu, climb, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(count, local);
    atomicAdd(count + 1, climb);
  }
}

template <class Real>
void launch_first_order_census(const AtmoParams* params, const BuildDims& d, const RowInfo* rowinfo,
                               const RowSample<Real>* rows, const CellGeom<Real>* geom, unsigned long long* count,
                               cudaStream_t st) {
  dim3 grid((unsigned)d.rows(), d.B);
  k_first_order_census<Real><<<grid, 256, 0, st>>>(params, d, rowinfo, rows, geom, count);
}

template void launch_first_order_census<float>(const AtmoParams*, const BuildDims&, const RowInfo*,
                                               const RowSample<float>*, const CellGeom<float>*,
                                               unsigned long long*, cudaStream_t);
template void launch_first_order_census<double>(const AtmoParams*, const BuildDims&, const RowInfo*,
                                                const RowSample<double>*, const CellGeom<double>*,
                                                unsigned long long*, cudaStream_t);

}  // namespace sfsim
