// k_setup.cu -- node maps, transmittance and surface-base tables, per-row ray
// samples and per-height sphere directions of the atmosphere LUT build.
#include <type_traits>

#include "atmo_device.cuh"
#include "kernels.h"

namespace sfsim {

// ---------------------------------------------------------------------------
// Re-interpolation maps.  Every table that the reference writes is
// make-lookup-table of an interpolated function, so each node's value is the
// table interpolated at forward(backward(node)) (interpolate.clj:68-110,
// atmosphere_lut.clj:94-101).  These kernels store that coordinate per node.
// ---------------------------------------------------------------------------

// Per view row (i, j), once: the row's geometry (RowInfo) and its height and
// elevation coordinates, which every node and ray sample of the row shares.
template <class Real>
__global__ void k_row_info(const AtmoParams* params, BuildDims d, RowInfo* info, Remap2<Real>* rowmap) {
  const long long nrows = d.rows();
  const long long row = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const int b = blockIdx.y;
  if (row >= nrows) return;
  const AtmoParams& P = params[b];
  const int j = (int)(row % d.n1), i = (int)(row / d.n1);
  double r, sv, cv;
  int above;
  view_geometry(P, d, i, j, &r, &sv, &cv, &above);
  const d3 x = mk3(r, 0, 0), v = mk3(sv, cv, 0);
  const d3 e = above ? atmosphere_intersection(P, x, v) : surface_intersection(P, x, v);
  const d3 D = sub3(e, x);
  RowInfo ri;
  ri.r = r;
  ri.sv = sv;
  ri.cv = cv;
  ri.D[0] = D.x;
  ri.D[1] = D.y;
  ri.D[2] = D.z;
  ri.L = mag3(D);
  ri.Ls = ri.L / d.S;
  {
    const double c0 = dmul(dsub(r, P.R), dadd(r, P.R)), xD = dmul(r, D.x), DD = dot3(D, D);
    ri.qmin = DD > 0.0 ? c0 - xD * xD / DD : c0;
    ri.t = DD > 0.0 ? xD / DD : 0.0;
  }
  ri.f_r = (float)r;
  ri.f_sv = (float)sv;
  ri.f_cv = (float)cv;
  ri.f_D[0] = (float)D.x;
  ri.f_D[1] = (float)D.y;
  ri.f_D[2] = (float)D.z;
  ri.f_Ls = (float)ri.Ls;
  ri.above = above;
  info[b * nrows + row] = ri;
  Remap2<Real> m;
  split_coord<Real>(height_to_index(P, d.n0, mag3(x)), d.n0, &m.u[0], &m.s[0]);
  split_coord<Real>(elevation_to_index(P, d.n1, x, v, above), d.n1, &m.u[1], &m.s[1]);
  rowmap[b * nrows + row] = m;
}

// The height and elevation coordinates of a node are its row's (k_row_info);
// its light direction l = index-to-sun-direction(v, sin(k), a) has
// x.l = r sin(k) with x = (r, 0, 0), so its sun-elevation coordinate is the
// (i, k) one of k_point_rows, which also holds sin(k).
template <class Real>
__global__ void k_remap4(const AtmoParams* params, BuildDims d, const RowInfo* info, const Remap2<Real>* rowmap,
                         const PointRow<Real>* prow, const double* __restrict__ hdvs, Remap4<Real>* out,
                         CellGeom<Real>* geom) {
  const long long n4 = d.n4();
  const long long node = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const int b = blockIdx.y;
  if (node >= n4) return;
  int a = (int)(node % d.n3);
  int k = (int)((node / d.n3) % d.n2);
  const long long row = node / ((long long)d.n3 * d.n2);
  const int i = (int)(row / d.n1);
  const RowInfo& ri = info[b * d.rows() + row];
  const Remap2<Real> rm = rowmap[b * d.rows() + row];
  const PointRow<Real>& pk = prow[((long long)b * d.n0 + i) * d.n2 + k];
  const double sv = ri.sv, cv = ri.cv;
  const d3 v = mk3(sv, cv, 0);
  const d3 l = node_light(sv, cv, pk.ss, pk.cs, hdvs[a]);
  Remap4<Real> m;
  m.u[0] = rm.u[0];
  m.s[0] = rm.s[0];
  m.u[1] = rm.u[1];
  m.s[1] = rm.s[1];
  m.u[2] = pk.u2;
  m.s[2] = pk.s2;
  split_coord<Real>(sun_angle_to_index(d.n3, v, l), d.n3, &m.u[3], &m.s[3]);
  out[b * n4 + node] = m;
  geom[b * n4 + node] = cell_geom<Real>(sv, cv, l);
}

template <class Real>
__global__ void k_remapT(const AtmoParams* params, BuildDims d, Remap2<Real>* out) {
  const long long n = d.nT();
  const long long node = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const int b = blockIdx.y;
  if (node >= n) return;
  const AtmoParams& P = params[b];
  int j = (int)(node % d.nT1), i = (int)(node / d.nT1);
  double r = index_to_radius(P, d.nT0, (double)i), sv, cv;
  int above;
  index_to_elevation(P, d.nT1, r, (double)j, &sv, &cv, &above);
  d3 x = mk3(r, 0, 0), v = mk3(sv, cv, 0);
  Remap2<Real> m;
  split_coord<Real>(height_to_index(P, d.nT0, mag3(x)), d.nT0, &m.u[0], &m.s[0]);
  split_coord<Real>(elevation_to_index(P, d.nT1, x, v, above), d.nT1, &m.u[1], &m.s[1]);
  out[b * n + node] = m;
}

__host__ __device__ inline void surface_node(const AtmoParams& P, const BuildDims& d, int i, int k, d3* x, d3* l) {
  double r = index_to_radius(P, d.nE0, (double)i);
  double s = index_to_sin_sun_elevation(d.nE1, (double)k);
  double c = sqrt(dmax(0.0, 1 - sqr(s)));
  *x = mk3(r, 0, 0);
  *l = mk3(s, c, 0);
}

template <class Real>
__global__ void k_remapE(const AtmoParams* params, BuildDims d, Remap2<Real>* out) {
  const long long n = d.nE();
  const long long node = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const int b = blockIdx.y;
  if (node >= n) return;
  const AtmoParams& P = params[b];
  int k = (int)(node % d.nE1), i = (int)(node / d.nE1);
  d3 x, l;
  surface_node(P, d, i, k, &x, &l);
  Remap2<Real> m;
  split_coord<Real>(height_to_index(P, d.nE0, mag3(x)), d.nE0, &m.u[0], &m.s[0]);
  split_coord<Real>(sun_elevation_to_index(d.nE1, x, l), d.nE1, &m.u[1], &m.s[1]);
  out[b * n + node] = m;
}

// ---------------------------------------------------------------------------
// Transmittance table (atmosphere_lut.clj:74, atmosphere.clj:114-128)
// ---------------------------------------------------------------------------

template <class Real>
__global__ void k_transmittance(const AtmoParams* params, BuildDims d, Vec4<Real>* T) {
  const long long n = d.nT();
  const long long node = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const int b = blockIdx.y;
  if (node >= n) return;
  const AtmoParams& P = params[b];
  int j = (int)(node % d.nT1), i = (int)(node / d.nT1);
  double r = index_to_radius(P, d.nT0, (double)i), sv, cv;
  int above;
  index_to_elevation(P, d.nT1, r, (double)j, &sv, &cv, &above);
  d3 x = mk3(r, 0, 0), v = mk3(sv, cv, 0);
  d3 e = above ? atmosphere_intersection(P, x, v) : surface_intersection(P, x, v);
  Real tau[3];
  segment_depth<Real>(P, x, sub3(e, x), d.S, tau);
  Vec4<Real> o;
  o.x = exp_neg(tau[0]);
  o.y = exp_neg(tau[1]);
  o.z = exp_neg(tau[2]);
  o.w = 0;
  T[b * n + node] = o;
}

// ---------------------------------------------------------------------------
// Surface radiance of direct sun light E0 (atmosphere.clj:131-137)
// ---------------------------------------------------------------------------

template <class Real>
__global__ void k_surface_base(const AtmoParams* params, BuildDims d, Vec4<Real>* E0) {
  const long long n = d.nE();
  const long long node = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const int b = blockIdx.y;
  if (node >= n) return;
  const AtmoParams& P = params[b];
  int k = (int)(node % d.nE1), i = (int)(node / d.nE1);
  d3 x, l;
  surface_node(P, d, i, k, &x, &l);
  d3 normal = mul3(x, 1.0 / mag3(x));
  double cosine = dmax(0.0, dot3(normal, l));
  Vec4<Real> o;
  o.x = o.y = o.z = o.w = 0;
  if (cosine > 0.0) {
    d3 e = atmosphere_intersection(P, x, l);
    Real tau[3];
    segment_depth<Real>(P, x, sub3(e, x), d.S, tau);
    o.x = exp_neg(tau[0]) * (Real)(P.intensity[0] * cosine);
    o.y = exp_neg(tau[1]) * (Real)(P.intensity[1] * cosine);
    o.z = exp_neg(tau[2]) * (Real)(P.intensity[2] * cosine);
  }
  E0[b * n + node] = o;
}

// ---------------------------------------------------------------------------
// View rows: for every (height i, elevation j) of the 4-D space the ray from
// x to its extremity (atmosphere.clj:192-200) and its S midpoint samples.
// One thread per (row, sample).
// ---------------------------------------------------------------------------

// Sample s of a row, everything but the optical depth from the row's node.
// The sample's coordinates are generic (between nodes), so the FP64 forms
// are reduced where that moves them by rounding only: the point (r + su D.x,
// su D.y, su D.z) without adding x's zero components, the atmosphere's
// horizon distance P.Hh in the height coordinate, and rs = p.v in the
// elevation coordinate (elevation-to-index forms |p| ((p.v) / |p|)).
template <class Real>
__device__ inline RowSample<Real> view_sample(const AtmoParams& P, const BuildDims& d, const RowInfo& ri, int s) {
  // sample point as integral-ray forms it (ray.clj:22-24)
  const double su = (0.5 + s) * d.inv_S;
  const d3 p = mk3(dadd(ri.r, dmul(ri.D[0], su)), dmul(ri.D[1], su), dmul(ri.D[2], su));
  const double pr = mag3(p);
  const double h = pr - P.R;
  RowSample<Real> o;
  if (std::is_same<Real, float>::value) {
    // the densities exp(-h/H) as the FP32 integrands form them
    o.er = (Real)Bulk<float>::exp2((float)h * P.f_kr);
    o.em = (Real)Bulk<float>::exp2((float)h * P.f_km);
    o.inv_r = (Real)__frcp_rn((float)pr);
  } else {
    o.er = (Real)exp(-(h / P.ray_scale));
    o.em = (Real)exp(-(h / P.mie_scale));
    o.inv_r = (Real)(1.0 / pr);
  }
  o.q = (Real)(h * (pr + P.R));
  o.us = (Real)su;
  // height-to-index and elevation-to-index (atmosphere.clj:239-253, 273-288)
  const double rho = horizon_distance(P, pr);
  split_coord<Real>(dmul((double)(d.n0 - 1), rho / P.Hh), d.n0, &o.u0, &o.s0);
  const double rs = dadd(dmul(p.x, ri.sv), dmul(p.y, ri.cv));
  const double Delta = dsub(sqr(rs), sqr(rho));
  double idx;
  if (ri.above)
    idx = dsub(0.5, limit_quot(dsub(rs, sqrt(dmax(0.0, dadd(Delta, P.Hh2)))), dadd(dadd(rho, rho), dmul(2.0, P.Hh)),
                               -0.5, 0.0));
  else
    idx = dadd(0.5, limit_quot(dadd(rs, sqrt(dmax(0.0, Delta))), dadd(rho, rho), -0.5, 0.0));
  split_coord<Real>(dmul((double)(d.n1 - 1), idx), d.n1, &o.u1, &o.s1);
  o.pad = 0;
  return o;
}

// T(x, p_s) by the nested midpoint sums over x -> p_s = x + su D (S samples).
// The segment's height form comes from the row's (qmin and t are the same
// for every su up to rounding; u* scales as t / su), and its sample step in
// distance is su L / S.
template <class Real>
__device__ inline void view_depth(const AtmoParams& P, const BuildDims& d, const RowInfo& ri, int s, Real tau[3]) {
  if (!(ri.L > 0.0)) {
    tau[0] = tau[1] = tau[2] = 0;
    return;
  }
  const double du = d.inv_S, su = (0.5 + s) * du;
  const double c0 = dmul(dsub(ri.r, P.R), dadd(ri.r, P.R));
  const double DD = su * su * (ri.D[0] * ri.D[0] + ri.D[1] * ri.D[1] + ri.D[2] * ri.D[2]);
  QForm f;
  f.C = DD;
  if (DD > 0.0 && fabs(ri.qmin) < c0) {
    f.A = ri.qmin;
    f.B = 0.0;
    f.w0 = 0.5 * du + ri.t / su;
  } else {
    f.A = c0;
    f.B = 2.0 * (su * (ri.r * ri.D[0]));
    f.w0 = 0.5 * du;
  }
  Real sr, sm;
  optical_sums_w<Real, 5>((Real)f.A, (Real)f.B, (Real)f.C, (Real)f.w0, (Real)du, d.S, Bulk<Real>::hpoly(P),
                          Bulk<Real>::alpha(P), Bulk<Real>::beta(P), Bulk<Real>::kr(P), Bulk<Real>::km(P), sr, sm);
  const Real a = (Real)(su * ri.Ls);
#pragma unroll
  for (int ch = 0; ch < 3; ch++) tau[ch] = a * (Bulk<Real>::ray_ext(P, ch) * sr + Bulk<Real>::mie_ext(P, ch) * sm);
}

template <class Real>
__global__ void k_view_rows(const AtmoParams* params, BuildDims d, const RowInfo* info, RowSample<Real>* samples) {
  const long long nrows = d.rows();
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const int b = blockIdx.y;
  if (t >= nrows * d.S) return;
  const AtmoParams& P = params[b];
  const int s = (int)(t % d.S);
  const long long row = t / d.S;
  const RowInfo& ri = info[b * nrows + row];
  RowSample<Real> o = view_sample<Real>(P, d, ri, s);
  view_depth<Real>(P, d, ri, s, o.tau);
  samples[(b * nrows + row) * d.S + s] = o;
}

// The same samples with the optical depth from the row's node x to each
// p_s by one prefix scan over the row (SFSIM_ATMO_SCAN_RAYS), instead of S
// samples between x and every p_s.  With cells [n du, (n + 1) du] of the
// row parameter u (du = 1/S) and rho_n the density at the midpoint u_n of
// cell n (the sample points themselves),
//   tau(x, p_s) = L du (sum_{n<s} rho_n + rho((s + 1/4) du) / 2):
// the midpoint rule on the whole cells before p_s and on the half cell up
// to it.  The densities are the integrand of the nested sums: the row's
// height form q(u) (segment_q_form) in Real.  One warp per row; lane l takes
// samples l, l + 32, ...; each 32 samples are one shuffle scan, carried on
// to the next 32.
template <class Real>
__global__ void k_view_rows_scan(const AtmoParams* params, BuildDims d, const RowInfo* info,
                                 RowSample<Real>* samples) {
  const long long nrows = d.rows();
  const int lane = threadIdx.x & 31;
  const long long row = blockIdx.x * (long long)(blockDim.x >> 5) + (threadIdx.x >> 5);
  const int b = blockIdx.y;
  if (row >= nrows) return;  // whole warps
  const AtmoParams& P = params[b];
  const RowInfo& ri = info[b * nrows + row];
  const double du = 1.0 / d.S;
  const double c0 = dmul(dsub(ri.r, P.R), dadd(ri.r, P.R));
  const d3 D = mk3(ri.D[0], ri.D[1], ri.D[2]);
  const QForm f = segment_q_form(c0, dmul(ri.r, D.x), dot3(D, D), du);
  const Real A = (Real)f.A, B = (Real)f.B, C = (Real)f.C, w0 = (Real)f.w0, dur = (Real)du;
  const Real* hp = Bulk<Real>::hpoly(P);
  const Real al = Bulk<Real>::alpha(P), be = Bulk<Real>::beta(P), kr = Bulk<Real>::kr(P), km = Bulk<Real>::km(P);
  const Real Ls = (Real)(ri.L * du);
  Real carry_r = 0, carry_m = 0;
  for (int s0 = 0; s0 < d.S; s0 += 32) {
    const int s = s0 + lane;
    Real rr = 0, rm = 0, qr = 0, qm = 0;
    if (s < d.S) {
      // w of the sample's midpoint (as optical_sums_w forms it) and of the
      // half cell's midpoint (s + 1/4) du
      const Real wm = fma(Real(s), dur, w0);
      const Real wq = fma(Real(s) - Real(0.25), dur, w0);
      const Real hm = height_from_q<Real, 5>(fma(wm, fma(wm, C, B), A), hp, al, be);
      const Real hq = height_from_q<Real, 5>(fma(wq, fma(wq, C, B), A), hp, al, be);
      rr = Bulk<Real>::exp2(hm * kr);
      rm = Bulk<Real>::exp2(hm * km);
      qr = Bulk<Real>::exp2(hq * kr);
      qm = Bulk<Real>::exp2(hq * km);
    }
    // inclusive scan over the 32 lanes
    Real ir = rr, im = rm;
#pragma unroll
    for (int k = 1; k < 32; k <<= 1) {
      const Real ur = __shfl_up_sync(0xffffffffu, ir, k), um = __shfl_up_sync(0xffffffffu, im, k);
      if (lane >= k) {
        ir += ur;
        im += um;
      }
    }
    Real er = __shfl_up_sync(0xffffffffu, ir, 1), em = __shfl_up_sync(0xffffffffu, im, 1);
    if (lane == 0) er = em = 0;
    if (s < d.S) {
      RowSample<Real> o = view_sample<Real>(P, d, ri, s);
      const Real sr = carry_r + er + Real(0.5) * qr, sm = carry_m + em + Real(0.5) * qm;
#pragma unroll
      for (int ch = 0; ch < 3; ch++) o.tau[ch] = Ls * (Bulk<Real>::ray_ext(P, ch) * sr + Bulk<Real>::mie_ext(P, ch) * sm);
      samples[(b * nrows + row) * d.S + s] = o;
    }
    carry_r += __shfl_sync(0xffffffffu, ir, 31);
    carry_m += __shfl_sync(0xffffffffu, im, 31);
  }
}

// ---------------------------------------------------------------------------
// Sphere directions of point scatter per height row (atmosphere.clj:203-222,
// sphere.clj:62-105): the direction in world space, where it ends, whether
// that end is on the ground, the elevation coordinate of the dS lookup and,
// for ground ends, T(x, g) * brightness / pi and the ground point's height
// coordinate in the surface-radiance space.
// ---------------------------------------------------------------------------

template <class Real>
__global__ void k_sphere_setup(const AtmoParams* params, BuildDims d, const DirLocal* dirs,
                               SphereDir<Real>* out) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const int b = blockIdx.y;
  if (t >= (long long)d.n0 * d.P) return;
  const AtmoParams& P = params[b];
  const int w = (int)(t % d.P), i = (int)(t / d.P);
  double r = index_to_radius(P, d.n0, (double)i);
  d3 x = mk3(r, 0, 0);
  d3 n = mul3(x, 1.0 / mag3(x));
  d3 o1 = orthogonal(n);
  d3 o2 = cross3(n, o1);
  d3 omega = to_world(n, o1, o2, dirs[w]);
  d3 g = ray_extremity(P, x, omega);
  int surface = surface_point(P, g);
  SphereDir<Real> o;
  o.w[0] = (Real)omega.x;
  o.w[1] = (Real)omega.y;
  o.w[2] = (Real)omega.z;
  o.weight = (Real)dirs[w].w;
  o.surface = surface;
  o.pad = 0;
  split_coord<Real>(elevation_to_index(P, d.n1, x, omega, !surface), d.n1, &o.u1, &o.s1);
  if (surface) {
    Real tau[3];
    segment_depth<Real>(P, x, sub3(g, x), d.S, tau);
    double gr = mag3(g);
    for (int c = 0; c < 3; c++) o.ground[c] = exp_neg(tau[c]) * (Real)(P.brightness[c] / M_PI);
    o.tR = (Real)(mag3(sub3(g, x)) / P.R);
    split_coord<Real>(height_to_index(P, d.nE0, gr), d.nE0, &o.uE0, &o.sE0);
  } else {
    for (int c = 0; c < 3; c++) o.ground[c] = 0;
    o.tR = 0;
    o.uE0 = 0;
    o.sE0 = 0;
  }
  out[((long long)b * d.n0 + i) * d.P + w] = o;
}

// The sphere directions of one height row split into those that end in the
// sky and those that end on the ground (the latter with an exactly-zero
// ground height coordinate first), order kept within each part, and
// each part filled to a multiple of kDirBlock with zero-weight entries, so
// that point scatter runs both parts in whole blocks of directions without
// a branch per direction.  One warp per row.
template <class Real>
__global__ void k_sphere_partition(BuildDims d, const SphereDir<Real>* sdirs, SphereDir<Real>* pdirs,
                                   int2* pcount, unsigned char* dimage) {
  const int i = blockIdx.x, b = blockIdx.y, lane = threadIdx.x;
  const long long row = (long long)b * d.n0 + i;
  const SphereDir<Real>* src = sdirs + row * d.P;
  SphereDir<Real>* dst = pdirs + row * dir_row(d.P);
  // three groups, order kept within each: sky, ground with the ground
  // point's height coordinate exactly 0 (most of them: only its lower E row
  // has weight), other ground
  int nsky = 0, nflat = 0;
  for (int t0 = 0; t0 < d.P; t0 += 32) {
    const int t = t0 + lane;
    const bool in = t < d.P;
    nsky += __popc(__ballot_sync(0xffffffffu, in && !src[t].surface));
    nflat += __popc(__ballot_sync(0xffffffffu, in && src[t].surface && src[t].sE0 == Real(0)));
  }
  const int sky_end = (nsky + kDirBlock - 1) / kDirBlock * kDirBlock;
  const int nground = d.P - nsky;
  const int used = sky_end + (nground + kDirBlock - 1) / kDirBlock * kDirBlock;
  const unsigned below = (1u << lane) - 1u;
  int s = 0, f = 0, g = 0;
  for (int t0 = 0; t0 < d.P; t0 += 32) {
    const int t = t0 + lane;
    const bool in = t < d.P;
    const bool sky = in && !src[t].surface;
    const bool flat = in && !sky && src[t].sE0 == Real(0);
    const unsigned bs = __ballot_sync(0xffffffffu, sky), bf = __ballot_sync(0xffffffffu, flat);
    const unsigned bg = __ballot_sync(0xffffffffu, in && !sky && !flat);
    if (in) {
      SphereDir<Real> e = src[t];
      e.pad = 0;
      const int pos = sky ? s + __popc(bs & below)
                          : (flat ? sky_end + f + __popc(bf & below) : sky_end + nflat + g + __popc(bg & below));
      dst[pos] = e;
    }
    s += __popc(bs);
    f += __popc(bf);
    g += __popc(bg);
  }
  SphereDir<Real> z;
  for (int c = 0; c < 3; c++) z.w[c] = z.ground[c] = 0;
  z.tR = 0;
  z.weight = z.s1 = z.sE0 = 0;
  z.u1 = z.uE0 = 0;
  z.pad = 1;
  for (int t = nsky + lane; t < sky_end; t += 32) {
    z.surface = 0;
    dst[t] = z;
  }
  for (int t = sky_end + nground + lane; t < used; t += 32) {
    z.surface = 1;
    dst[t] = z;
  }
  if (lane == 0) pcount[row] = make_int2(sky_end, used);
  // point scatter's shared-memory image of the list: each field as an array
  __syncwarp();
  Real* img = reinterpret_cast<Real*>(dimage + row * dir_image_stride(d, sizeof(Real)));
  int* img_u = reinterpret_cast<int*>(img + kDirFields * used);
  for (int t = lane; t < used; t += 32) {
    const SphereDir<Real> e = dst[t];
    const Real f[kDirFields] = {e.w[0],      e.w[1],      e.w[2],      e.weight, e.tR,
                                e.ground[0], e.ground[1], e.ground[2], e.sE0};
#pragma unroll
    for (int c = 0; c < kDirFields; c++) img[c * used + t] = f[c];
    img_u[t] = e.uE0;
  }
}

// Point-scatter constants per (height i, sun elevation k): the coordinates
// of ray-scatter-forward (atmosphere.clj:203-222) at x = (r_i, 0, 0) with the
// sun at elevation k, and beta_c(x) (atmosphere.clj:42-47, 140-151), in FP64
// once here instead of in every thread of the point-scatter blocks.
template <class Real>
__global__ void k_point_rows(const AtmoParams* params, BuildDims d, PointRow<Real>* out, double* hdvs) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int b = blockIdx.y;
  if (b == 0) {
    // v.l of heading a as index_to_sun_direction forms it, for every atmosphere
    const int nt = gridDim.x * blockDim.x;
    for (int a = t; a < d.n3; a += nt) hdvs[a] = dsub(dmul(2.0, (double)a / (d.n3 - 1)), 1.0);
  }
  if (t >= d.n0 * d.n2) return;
  const AtmoParams& P = params[b];
  const int i = t / d.n2, k = t % d.n2;
  const double r = index_to_radius(P, d.n0, (double)i);
  const double ss = index_to_sin_sun_elevation(d.n2, (double)k);
  PointRow<Real> o;
  o.ss = ss;
  o.cs = sqrt(dmax(0.0, dsub(1.0, sqr(ss))));
  o.gA = (Real)(r * ss / P.R);
  split_coord<Real>(height_to_index(P, d.n0, r), d.n0, &o.u0, &o.s0);
  split_coord<Real>(sun_elevation_to_index(d.n2, mk3(r, 0, 0), mk3(ss, 0, 0)), d.n2, &o.u2, &o.s2);
  const double h = r - P.R;
  const double er = exp(-(h / P.ray_scale)), em = exp(-(h / P.mie_scale));
  for (int c = 0; c < 3; c++) {
    o.bR[c] = (Real)(P.ray_base[c] * er);
    o.bM[c] = (Real)(P.mie_base[c] * em);
  }
  out[(long long)b * d.n0 * d.n2 + t] = o;
}

// Surface-radiance constants per node (iE, kE), in FP64 as the per-node part
// of k_surface_radiance needs them (atmosphere.clj:225-230, 239-253).
template <class Real>
__global__ void k_surface_rows(const AtmoParams* params, BuildDims d, SurfRow<Real>* out) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const int b = blockIdx.y;
  if (t >= d.nE()) return;
  const AtmoParams& P = params[b];
  const int iE = (int)(t / d.nE1), kE = (int)(t % d.nE1);
  const double r = index_to_radius(P, d.nE0, (double)iE);
  const double ss = index_to_sin_sun_elevation(d.nE1, (double)kE);
  const d3 x = mk3(r, 0, 0), l = mk3(ss, sqrt(dmax(0.0, 1 - sqr(ss))), 0);
  SurfRow<Real> o;
  split_coord<Real>(height_to_index(P, d.n0, mag3(x)), d.n0, &o.u0, &o.s0);
  split_coord<Real>(sun_elevation_to_index(d.n2, x, l), d.n2, &o.u2, &o.s2);
  const double c0 = dmul(dsub(r, P.R), dadd(r, P.R));  // |x|^2 - R^2
  const Real rho = (Real)sqrt(dmax(0.0, c0));
  o.Hh2mq = (Real)dsub(P.Hh2, c0);
  o.den = rho + rho + Real(2) * (Real)P.Hh;
  o.rr = (Real)r;
  o.lx = (Real)l.x;
  o.ly = (Real)l.y;
  out[(long long)b * d.nE() + t] = o;
}

// The half-sphere directions of surface radiance in world coordinates at
// the height of row iE (x = (r, 0, 0), the frame of integral-half-sphere).
template <class Real>
__global__ void k_half_dirs(const AtmoParams* params, BuildDims d, const DirLocal* hdirs, HalfDir<Real>* out) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const int b = blockIdx.y;
  if (t >= (long long)d.nE0 * d.Ph) return;
  const AtmoParams& P = params[b];
  const int iE = (int)(t / d.Ph), w = (int)(t % d.Ph);
  const double r = index_to_radius(P, d.nE0, (double)iE);
  const d3 x = mk3(r, 0, 0);
  const d3 n = mul3(x, 1.0 / mag3(x));
  const d3 o1 = orthogonal(n);
  const d3 o2 = cross3(n, o1);
  const DirLocal qd = hdirs[w];
  const d3 omega = to_world(n, o1, o2, qd);
  HalfDir<Real> o;
  o.wx = (Real)omega.x;
  o.wy = (Real)omega.y;
  o.wgt = (Real)(qd.w * dot3(omega, n));
  out[(long long)b * d.nE0 * d.Ph + t] = o;
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------

static inline dim3 grid1(long long n, int block, int B) { return dim3((unsigned)((n + block - 1) / block), B); }

template <class Real>
void launch_setup_rows(const AtmoParams* params, const BuildDims& d, const SetupBuffers<Real>& o, cudaStream_t st) {
  const int blk = 128;
  k_row_info<Real><<<grid1(d.rows(), blk, d.B), blk, 0, st>>>(params, d, o.rowinfo, o.rowmap);
  k_point_rows<Real><<<grid1((long long)d.n0 * d.n2, blk, d.B), blk, 0, st>>>(params, d, o.prow, o.hdvs);
}

template <class Real>
void launch_node_maps(const AtmoParams* params, const BuildDims& d, const SetupBuffers<Real>& o, cudaStream_t st) {
  const int blk = 128;
  k_remap4<Real><<<grid1(d.n4(), blk, d.B), blk, 0, st>>>(params, d, o.rowinfo, o.rowmap, o.prow, o.hdvs,
                                                            o.remapS, o.geom);
}

template <class Real>
void launch_view_rows(const AtmoParams* params, const BuildDims& d, const SetupBuffers<Real>& o, cudaStream_t st) {
  const int blk = 128;
  if (d.scan_rays)
    k_view_rows_scan<Real><<<grid1(d.rows(), blk / 32, d.B), blk, 0, st>>>(params, d, o.rowinfo, o.rows);
  else
    k_view_rows<Real><<<grid1(d.rows() * d.S, blk, d.B), blk, 0, st>>>(params, d, o.rowinfo, o.rows);
}

template <class Real>
int launch_setup_aux(const AtmoParams* params, const BuildDims& d, const DirLocal* dirs,
                     const DirLocal* half_dirs, const SetupBuffers<Real>& o, cudaStream_t st) {
  const int blk = 128;
  k_remapT<Real><<<grid1(d.nT(), blk, d.B), blk, 0, st>>>(params, d, o.remapT);
  k_remapE<Real><<<grid1(d.nE(), blk, d.B), blk, 0, st>>>(params, d, o.remapE);
  // a build without iterations may ask for no sphere directions (sphere
  // steps below 2) or no half-sphere ones (ray steps below 4): nothing to launch
  if (d.P > 0)
    k_sphere_setup<Real><<<grid1((long long)d.n0 * d.P, blk, d.B), blk, 0, st>>>(params, d, dirs, o.sdirs);
  k_sphere_partition<Real><<<dim3(d.n0, d.B), 32, 0, st>>>(d, o.sdirs, o.pdirs, o.pcount, o.dimage);
  k_surface_rows<Real><<<grid1(d.nE(), blk, d.B), blk, 0, st>>>(params, d, o.erow);
  if (d.Ph > 0)
    k_half_dirs<Real><<<grid1((long long)d.nE0 * d.Ph, blk, d.B), blk, 0, st>>>(params, d, half_dirs, o.hdir);
  return 4 + (d.P > 0) + (d.Ph > 0);
}

template <class Real>
void launch_setup(const AtmoParams* params, const BuildDims& d, const DirLocal* dirs,
                  const DirLocal* half_dirs, const SetupBuffers<Real>& o, cudaStream_t st) {
  launch_setup_rows<Real>(params, d, o, st);
  launch_node_maps<Real>(params, d, o, st);
  launch_view_rows<Real>(params, d, o, st);
  launch_setup_aux<Real>(params, d, dirs, half_dirs, o, st);
}

template <class Real>
void launch_transmittance(const AtmoParams* params, const BuildDims& d, Vec4<Real>* T, cudaStream_t st) {
  const int blk = 128;
  k_transmittance<Real><<<grid1(d.nT(), blk, d.B), blk, 0, st>>>(params, d, T);
}

template <class Real>
void launch_surface_base(const AtmoParams* params, const BuildDims& d, Vec4<Real>* E0, cudaStream_t st) {
  const int blk = 128;
  k_surface_base<Real><<<grid1(d.nE(), blk, d.B), blk, 0, st>>>(params, d, E0);
}

template void launch_setup_rows<float>(const AtmoParams*, const BuildDims&, const SetupBuffers<float>&,
                                       cudaStream_t);
template void launch_setup_rows<double>(const AtmoParams*, const BuildDims&, const SetupBuffers<double>&,
                                        cudaStream_t);
template void launch_node_maps<float>(const AtmoParams*, const BuildDims&, const SetupBuffers<float>&,
                                      cudaStream_t);
template void launch_node_maps<double>(const AtmoParams*, const BuildDims&, const SetupBuffers<double>&,
                                       cudaStream_t);
template void launch_view_rows<float>(const AtmoParams*, const BuildDims&, const SetupBuffers<float>&,
                                      cudaStream_t);
template void launch_view_rows<double>(const AtmoParams*, const BuildDims&, const SetupBuffers<double>&,
                                       cudaStream_t);
template int launch_setup_aux<float>(const AtmoParams*, const BuildDims&, const DirLocal*, const DirLocal*,
                                     const SetupBuffers<float>&, cudaStream_t);
template int launch_setup_aux<double>(const AtmoParams*, const BuildDims&, const DirLocal*, const DirLocal*,
                                      const SetupBuffers<double>&, cudaStream_t);
template void launch_setup<float>(const AtmoParams*, const BuildDims&, const DirLocal*, const DirLocal*,
                                  const SetupBuffers<float>&, cudaStream_t);
template void launch_setup<double>(const AtmoParams*, const BuildDims&, const DirLocal*, const DirLocal*,
                                   const SetupBuffers<double>&, cudaStream_t);
template void launch_transmittance<float>(const AtmoParams*, const BuildDims&, Vec4<float>*, cudaStream_t);
template void launch_transmittance<double>(const AtmoParams*, const BuildDims&, Vec4<double>*, cudaStream_t);
template void launch_surface_base<float>(const AtmoParams*, const BuildDims&, Vec4<float>*, cudaStream_t);
template void launch_surface_base<double>(const AtmoParams*, const BuildDims&, Vec4<double>*, cudaStream_t);

}  // namespace sfsim
