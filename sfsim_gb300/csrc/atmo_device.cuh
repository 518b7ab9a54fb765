// atmo_device.cuh -- device math of the atmosphere lookup-table build.
//
// Two kinds of arithmetic live here:
//  * FP64 "islands": the table parameterisations, ray-sphere intersections and
//    horizon tests, written as the same IEEE double operations as the
//    reference (src/clj/sfsim/atmosphere.clj:70-384, sphere.clj:34-59,
//    util.clj:403-420), because radius-scale cancellation (r ~ 6.4e6 m) makes
//    them unusable in FP32.
//  * the bulk integrand in `Real` (float or double): optical-depth sums along
//    rays in the cancellation-free form q(t) = |p|^2 - R^2 = q0 + t (2b + t),
//    heights from q through a fitted polynomial h = q P(q), exponentials on
//    the SFU (ex2.approx) in FP32, compensated (Kahan) sums.
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <type_traits>

#include "atmo_params.h"

namespace sfsim {

// ---------------------------------------------------------------------------
// small vector helpers
// ---------------------------------------------------------------------------

struct d3 {
  double x, y, z;
};

// FP64 islands use separately rounded multiplies and adds, never fused: the
// reference (JVM doubles) rounds every operation, and at the horizon nodes
// the table maps take square roots of near-zero differences that amplify a
// one-ulp change into a visible one.
#ifdef __CUDA_ARCH__
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
#else
inline double dmul(double a, double b) { return a * b; }
inline double dadd(double a, double b) { return a + b; }
inline double dsub(double a, double b) { return a - b; }
#endif

__host__ __device__ __forceinline__ d3 mk3(double x, double y, double z) { return d3{x, y, z}; }
__host__ __device__ __forceinline__ d3 add3(d3 a, d3 b) { return d3{dadd(a.x, b.x), dadd(a.y, b.y), dadd(a.z, b.z)}; }
__host__ __device__ __forceinline__ d3 sub3(d3 a, d3 b) { return d3{dsub(a.x, b.x), dsub(a.y, b.y), dsub(a.z, b.z)}; }
__host__ __device__ __forceinline__ d3 mul3(d3 a, double s) { return d3{dmul(a.x, s), dmul(a.y, s), dmul(a.z, s)}; }
__host__ __device__ __forceinline__ double dot3(d3 a, d3 b) {
  return dadd(dadd(dmul(a.x, b.x), dmul(a.y, b.y)), dmul(a.z, b.z));
}
__host__ __device__ __forceinline__ double mag3(d3 a) { return sqrt(dot3(a, a)); }
__host__ __device__ __forceinline__ double sqr(double x) { return dmul(x, x); }
__host__ __device__ __forceinline__ double dmax(double a, double b) { return a >= b ? a : b; }
__host__ __device__ __forceinline__ double dmin(double a, double b) { return a <= b ? a : b; }

// ---------------------------------------------------------------------------
// FP64 islands (reference semantics)
// ---------------------------------------------------------------------------

// util.clj:403-420
__host__ __device__ inline double limit_quot(double a, double b, double lower, double upper) {
  if (a == 0.0) return a;
  if (b < 0) {
    a = -a;
    b = -b;
  }
  if (a < b * upper) {
    if (a > b * lower) return a / b;
    return lower;
  }
  return upper;
}

// core/limit-quot.glsl, the FP32 form of limit_quot the shaders use
__device__ __forceinline__ float limit_quot_f(float a, float b, float lower, float upper) {
  if (a == 0.0f) return 0.0f;
  if (b < 0) {
    a = -a;
    b = -b;
  }
  if (a < b * upper) {
    if (a > b * lower) return a / b;
    return lower;
  }
  return upper;
}

// sphere.clj:46-59; returns distance + length of the chosen branch pieces.
struct Isect {
  double distance, length;
};

__host__ __device__ inline Isect ray_sphere(double radius, d3 origin, d3 direction) {
  double direction_sqr = dot3(direction, direction);
  double od = dot3(direction, origin);
  double discriminant = dsub(sqr(od), dmul(direction_sqr, dsub(dot3(origin, origin), sqr(radius))));
  double middle = -(od / direction_sqr);
  Isect r;
  if (discriminant > 0) {
    double length2 = sqrt(discriminant) / direction_sqr;
    if (middle < length2) {
      r.distance = 0.0;
      r.length = dmax(0.0, dadd(middle, length2));
    } else {
      r.distance = dsub(middle, length2);
      r.length = dmul(2.0, length2);
    }
  } else {
    r.distance = dmax(0.0, middle);
    r.length = 0.0;
  }
  return r;
}

// atmosphere.clj:70-85
__host__ __device__ inline d3 atmosphere_intersection(const AtmoParams& P, d3 o, d3 d) {
  Isect i = ray_sphere(P.top, o, d);
  return add3(o, mul3(d, dadd(i.distance, i.length)));
}

__host__ __device__ inline d3 surface_intersection(const AtmoParams& P, d3 o, d3 d) {
  Isect i = ray_sphere(P.R, o, d);
  return add3(o, mul3(d, i.distance));
}

// atmosphere.clj:88-111
__host__ __device__ inline int surface_point(const AtmoParams& P, d3 point) {
  return dmul(2.0, dsub(mag3(point), P.R)) < P.H;
}

__host__ __device__ inline int is_above_horizon(const AtmoParams& P, d3 point, d3 direction) {
  double norm_point = mag3(point);
  double s = dot3(direction, point);
  double hd2 = dsub(sqr(norm_point), P.R2);
  return (s >= 0) || (sqr(s) <= hd2);
}

__host__ __device__ inline d3 ray_extremity(const AtmoParams& P, d3 o, d3 d) {
  if (is_above_horizon(P, o, d)) return atmosphere_intersection(P, o, d);
  return surface_intersection(P, o, d);
}

// atmosphere.clj:233-236
__host__ __device__ inline double horizon_distance(const AtmoParams& P, double radius) {
  return sqrt(dmax(0.0, dsub(sqr(radius), P.R2)));
}

// atmosphere.clj:239-253
__host__ __device__ inline double elevation_to_index(const AtmoParams& P, int size, d3 point, d3 direction,
                                                     int above) {
  double radius = mag3(point);
  double sin_elevation = dot3(point, direction) / radius;
  double rho = horizon_distance(P, radius);
  double rs = dmul(radius, sin_elevation);
  double Delta = dsub(sqr(rs), sqr(rho));
  double idx;
  if (above)
    idx = dsub(0.5, limit_quot(dsub(rs, sqrt(dmax(0.0, dadd(Delta, P.Hh2)))), dadd(dadd(rho, rho), dmul(2.0, P.Hh)),
                               -0.5, 0.0));
  else
    idx = dadd(0.5, limit_quot(dadd(rs, sqrt(dmax(0.0, Delta))), dadd(rho, rho), -0.5, 0.0));
  return dmul((double)(size - 1), idx);
}

// atmosphere.clj:256-270; direction = (sin, cos, 0)
__host__ __device__ inline void index_to_elevation(const AtmoParams& P, int size, double radius, double index,
                                                   double* sin_el, double* cos_el, int* above) {
  double horizon_dist = horizon_distance(P, radius);
  double scaled_index = index / (size - 1);
  double s;
  if (scaled_index < 0.5 || (scaled_index == 0.5 && dmul(2.0, radius) < dadd(P.R, P.top))) {
    double ground_dist = dmul(horizon_dist, dsub(1.0, dmul(2.0, scaled_index)));
    s = limit_quot(dsub(dsub(P.R2, sqr(radius)), sqr(ground_dist)), dmul(dmul(2.0, radius), ground_dist), -1.0, 1.0);
    *above = 0;
  } else {
    double sky_dist = dmul(dadd(horizon_dist, P.Hh), dsub(dmul(2.0, scaled_index), 1.0));
    s = limit_quot(dsub(dsub(P.top2, sqr(radius)), sqr(sky_dist)), dmul(dmul(2.0, radius), sky_dist), -1.0, 1.0);
    *above = 1;
  }
  *sin_el = s;
  *cos_el = sqrt(dsub(1.0, sqr(s)));
}

// atmosphere.clj:273-288
__host__ __device__ inline double height_to_index(const AtmoParams& P, int size, double radius) {
  return dmul((double)(size - 1), horizon_distance(P, radius) / horizon_distance(P, P.top));
}

__host__ __device__ inline double index_to_radius(const AtmoParams& P, int size, double index) {
  double horizon_dist = dmul(index / (size - 1), P.Hh);
  return sqrt(dadd(P.R2, sqr(horizon_dist)));
}

// atmosphere.clj:322-332
__host__ __device__ inline double sun_elevation_to_index(int size, d3 point, d3 light) {
  double sin_elevation = dot3(point, light) / mag3(point);
  return dmul((double)(size - 1),
              dmax(0.0, dsub(1.0, exp(dsub(dsub(0.0, dmul(3.0, sin_elevation)), 0.6))) / dsub(1.0, exp(-3.6))));
}

__host__ __device__ inline double index_to_sin_sun_elevation(int size, double index) {
  return dadd(log(dsub(1.0, dmul(index / (size - 1), dsub(1.0, exp(-3.6))))), 0.6) / -3.0;
}

// atmosphere.clj:368-384
__host__ __device__ inline double sun_angle_to_index(int size, d3 direction, d3 light) {
  return dmul((double)(size - 1), dadd(1.0, dot3(direction, light)) / 2.0);
}

__host__ __device__ inline d3 index_to_sun_direction(int size, d3 direction, double sin_sun, double index) {
  double dot_view_sun = dsub(dmul(2.0, index / (size - 1)), 1.0);
  double max_sun_1 = sqrt(dmax(0.0, dsub(1.0, sqr(sin_sun))));
  double sun_1 = limit_quot(dsub(dot_view_sun, dmul(direction.x, sin_sun)), direction.y, -max_sun_1, max_sun_1);
  double sun_2 = sqrt(dmax(0.0, dsub(dsub(1.0, sqr(sun_1)), sqr(sin_sun))));
  return mk3(sin_sun, sun_1, sun_2);
}

// index_to_sun_direction(n3, v, ss, a) for v = (sv, cv, 0), with its
// per-heading term dvs = 2 a / (n3 - 1) - 1 and per-sun-elevation bound
// cs = sqrt(max(0, 1 - ss^2)) precomputed by the same operations (so the
// same value); the light direction of every 4-D node.
__host__ __device__ inline d3 node_light(double sv, double cv, double ss, double cs, double dvs) {
  const double sun_1 = limit_quot(dsub(dvs, dmul(sv, ss)), cv, -cs, cs);
  return mk3(ss, sun_1, sqrt(dmax(0.0, dsub(dsub(1.0, sqr(sun_1)), sqr(ss)))));
}

// A node's light direction and v.l in Real, as the scattering kernels use them.
template <class Real>
__host__ __device__ inline CellGeom<Real> cell_geom(double sv, double cv, const d3& l) {
  CellGeom<Real> g;
  g.lx = (Real)l.x;
  g.ly = (Real)l.y;
  g.lz = (Real)l.z;
  g.mu = (Real)dot3(mk3(sv, cv, 0), l);
  return g;
}

// interpolate.clj:75-98 per dimension: i = clip(c), u = floor(i), s = i - u
template <class Real>
__host__ __device__ inline void split_coord(double c, int size, int* u, Real* s) {
  double i = dmin(dmax(c, 0.0), (double)(size - 1));
  double f = floor(i);
  *u = (int)f;
  *s = (Real)dsub(i, f);
}

template <class Real>
__device__ __forceinline__ void split_coord_r(Real c, int size, int* u, Real* s) {
  Real i = c < Real(0) ? Real(0) : c;
  Real hi = Real(size - 1);
  i = i > hi ? hi : i;
  Real f = floor(i);
  *u = (int)f;
  *s = i - f;
}

__host__ __device__ __forceinline__ int upper_index(int u, int size) { return u + 1 < size ? u + 1 : size - 1; }

__host__ __device__ inline d3 cross3(d3 a, d3 b) {
  return mk3(dsub(dmul(a.y, b.z), dmul(a.z, b.y)), dsub(dmul(a.z, b.x), dmul(a.x, b.z)),
             dsub(dmul(a.x, b.y), dmul(a.y, b.x)));
}

// quaternion.clj:166-171
__host__ __device__ inline d3 orthogonal(d3 n) {
  d3 rows[3] = {mk3(1, 0, 0), mk3(0, 1, 0), mk3(0, 0, 1)};
  int best = 0;
  double key = fabs(dot3(n, rows[0]));
  for (int i = 1; i < 3; i++) {
    double kk = fabs(dot3(n, rows[i]));
    if (kk < key) {
      key = kk;
      best = i;
    }
  }
  d3 c = cross3(n, rows[best]);
  return mul3(c, 1.0 / mag3(c));
}

// mulv (transpose (oriented-matrix n)) (vec3 x y z), matrix.clj:207-213
__host__ __device__ inline d3 to_world(d3 n, d3 o1, d3 o2, const DirLocal& q) {
  return mk3(dadd(dadd(dmul(n.x, q.x), dmul(o1.x, q.y)), dmul(o2.x, q.z)),
             dadd(dadd(dmul(n.y, q.x), dmul(o1.y, q.y)), dmul(o2.y, q.z)),
             dadd(dadd(dmul(n.z, q.x), dmul(o1.z, q.y)), dmul(o2.z, q.z)));
}

// Geometry of a 4-D node (ray-scatter-backward, atmosphere.clj:401-412).
struct NodeGeom {
  double r;
  double sv, cv;
  int above;
  d3 l;
};

__host__ __device__ inline void view_geometry(const AtmoParams& P, const BuildDims& d, int i, int j, double* r,
                                              double* sv, double* cv, int* above) {
  *r = index_to_radius(P, d.n0, (double)i);
  index_to_elevation(P, d.n1, *r, (double)j, sv, cv, above);
}

__host__ __device__ inline d3 light_direction(const BuildDims& d, double sv, double cv, int k, int a) {
  double sin_sun = index_to_sin_sun_elevation(d.n2, (double)k);
  return index_to_sun_direction(d.n3, mk3(sv, cv, 0.0), sin_sun, (double)a);
}

// ---------------------------------------------------------------------------
// Bulk arithmetic in Real
// ---------------------------------------------------------------------------

template <class Real>
struct Bulk;

template <>
struct Bulk<float> {
  static __device__ __forceinline__ float exp2(float x) {
    float r;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
  }
  static __device__ __forceinline__ float sqrt(float x) {
    float r;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
  }
  static __device__ __forceinline__ float rsqrt(float x) {
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
  }
  static __device__ __forceinline__ float div(float a, float b) { return __fdividef(a, b); }
  static __device__ __forceinline__ const float* hpoly(const AtmoParams& P) { return P.f_hpoly; }
  static constexpr int kSunNP = 4;  // the FP32 sun-ray loop uses the degree-3 fit
  static __device__ __forceinline__ const float* hpr(const AtmoParams& P) { return P.f_hpr4; }
  static __device__ __forceinline__ float hratio(const AtmoParams& P) { return P.f_hratio; }
  static __device__ __forceinline__ float alpha(const AtmoParams& P) { return P.f_alpha; }
  static __device__ __forceinline__ float beta(const AtmoParams& P) { return P.f_beta; }
  static __device__ __forceinline__ float kr(const AtmoParams& P) { return P.f_kr; }
  static __device__ __forceinline__ float km(const AtmoParams& P) { return P.f_km; }
  static __device__ __forceinline__ float ray_ext(const AtmoParams& P, int c) { return P.f_ray_ext[c]; }
  static __device__ __forceinline__ float mie_ext(const AtmoParams& P, int c) { return P.f_mie_ext[c]; }
  static __device__ __forceinline__ const float* phase_ray(const AtmoParams& P) { return P.f_phR; }
  static __device__ __forceinline__ const float* phase_mie(const AtmoParams& P) { return P.f_phM; }
  static __device__ __forceinline__ float src_ray(const AtmoParams& P, int c) { return P.f_srcR[c]; }
  static __device__ __forceinline__ float src_mie(const AtmoParams& P, int c) { return P.f_srcM[c]; }
  static __device__ __forceinline__ float sun_scale(const BuildDims& d) { return d.f_sun_scale; }
  static __device__ __forceinline__ float sun_scale_E(const BuildDims& d) { return d.f_sun_scale_E; }
};

template <>
struct Bulk<double> {
  static __device__ __forceinline__ double exp2(double x) { return ::exp2(x); }
  static __device__ __forceinline__ double sqrt(double x) { return ::sqrt(x); }
  static __device__ __forceinline__ double rsqrt(double x) { return 1.0 / ::sqrt(x); }
  static __device__ __forceinline__ double div(double a, double b) { return a / b; }
  static __device__ __forceinline__ const double* hpoly(const AtmoParams& P) { return P.d_hpoly; }
  static constexpr int kSunNP = 5;
  static __device__ __forceinline__ const double* hpr(const AtmoParams& P) { return P.d_hpr; }
  static __device__ __forceinline__ double hratio(const AtmoParams& P) { return P.d_hratio; }
  static __device__ __forceinline__ double alpha(const AtmoParams& P) { return P.d_alpha; }
  static __device__ __forceinline__ double beta(const AtmoParams& P) { return P.d_beta; }
  static __device__ __forceinline__ double kr(const AtmoParams& P) { return P.d_kr; }
  static __device__ __forceinline__ double km(const AtmoParams& P) { return P.d_km; }
  static __device__ __forceinline__ double ray_ext(const AtmoParams& P, int c) { return P.d_ray_ext[c]; }
  static __device__ __forceinline__ double mie_ext(const AtmoParams& P, int c) { return P.d_mie_ext[c]; }
  static __device__ __forceinline__ const double* phase_ray(const AtmoParams& P) { return P.d_phR; }
  static __device__ __forceinline__ const double* phase_mie(const AtmoParams& P) { return P.d_phM; }
  static __device__ __forceinline__ double src_ray(const AtmoParams& P, int c) { return P.d_srcR[c]; }
  static __device__ __forceinline__ double src_mie(const AtmoParams& P, int c) { return P.d_srcM[c]; }
  static __device__ __forceinline__ double sun_scale(const BuildDims& d) { return d.sun_scale; }
  static __device__ __forceinline__ double sun_scale_E(const BuildDims& d) { return d.sun_scale_E; }
};

// A view row's geometry in Real: the FP32 copies for FP32 kernels, so that
// they convert nothing on the (slow) FP64 pipe.
template <class Real>
struct RowR {
  Real r, sv, cv, D[3], Ls;
};
__device__ __forceinline__ void row_r(const RowInfo& ri, RowR<float>& o) {
  o.r = ri.f_r, o.sv = ri.f_sv, o.cv = ri.f_cv, o.Ls = ri.f_Ls;
  o.D[0] = ri.f_D[0], o.D[1] = ri.f_D[1], o.D[2] = ri.f_D[2];
}
__device__ __forceinline__ void row_r(const RowInfo& ri, RowR<double>& o) {
  o.r = ri.r, o.sv = ri.sv, o.cv = ri.cv, o.Ls = ri.Ls;
  o.D[0] = ri.D[0], o.D[1] = ri.D[1], o.D[2] = ri.D[2];
}
template <class Real>
__device__ __forceinline__ RowR<Real> row_r(const RowInfo& ri) {
  RowR<Real> o;
  row_r(ri, o);
  return o;
}

// Pairs of independent values with one instruction per operation: on
// sm_100+ FFMA2/FADD2/FMUL2 (each lane rounded as the scalar operation),
// plain pairs in FP64.
template <class Real>
struct Vec2Of;
template <>
struct Vec2Of<float> {
  using T = float2;
};
template <>
struct Vec2Of<double> {
  using T = double2;
};
template <class Real>
using V2 = typename Vec2Of<Real>::T;
__device__ __forceinline__ float2 mk2(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ double2 mk2(double a, double b) { return make_double2(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ double2 fma2(double2 a, double2 b, double2 c) {
  return make_double2(fma(a.x, b.x, c.x), fma(a.y, b.y, c.y));
}
__device__ __forceinline__ double2 add2(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 mul2(double2 a, double2 b) { return make_double2(a.x * b.x, a.y * b.y); }
// b - a, exactly rounded (a * -1 is exact, the FMA rounds once)
template <class V>
__device__ __forceinline__ V sub2(V b, V a) {
  return fma2(a, mk2(decltype(a.x)(-1), decltype(a.x)(-1)), b);
}

// Cornette-Shanks phase k (1 + mu^2) (a + b mu)^-3/2 from the host-computed
// coefficients {k, a, b} of AtmoParams.
template <class Real>
struct PhaseCS {
  Real k, a, b;
  __device__ __forceinline__ explicit PhaseCS(const Real* c) : k(c[0]), a(c[1]), b(c[2]) {}
  __device__ __forceinline__ Real operator()(Real mu) const {
    const Real r = Bulk<Real>::rsqrt(fma(b, mu, a));
    return k * fma(mu, mu, Real(1)) * (r * r * r);
  }
  __device__ __forceinline__ V2<Real> pair(V2<Real> mu) const {
    const V2<Real> t = fma2(mk2(b, b), mu, mk2(a, a));
    const V2<Real> r = mk2(Bulk<Real>::rsqrt(t.x), Bulk<Real>::rsqrt(t.y));
    return mul2(mul2(mk2(k, k), fma2(mu, mu, mk2(Real(1), Real(1)))), mul2(mul2(r, r), r));
  }
};

template <class Real>
__device__ __forceinline__ void kahan_add(Real& sum, Real& comp, Real x) {
  Real y = x - comp;
  Real t = sum + y;
  comp = (t - sum) - y;
  sum = t;
}

// Height above ground from q = |p|^2 - R^2: h = q / (R + sqrt(R^2 + q)),
// evaluated as q * P(z), z = q alpha + beta, P fitted on the host over the
// atmosphere's range of q (Chebyshev interpolation, relative error < 1e-9).
template <class Real, int NP>
__device__ __forceinline__ Real height_from_q(Real q, const Real* c, Real alpha, Real beta) {
  Real z = fma(q, alpha, beta);
  Real p = c[NP - 1];
#pragma unroll
  for (int k = NP - 2; k >= 0; k--) p = fma(p, z, c[k]);
  return q * p;
}

// Sums of exp(-h/H_rayleigh) and exp(-h/H_mie) over the midpoint samples of
// the sun ray, in the form the first-order kernel needs most often.  With
// t_n = (n + 1/2) dt, q(t_n) = A + n (B + n C), A = q0 + dt (b + dt/4),
// B = dt (2b + dt), C = dt^2, so each sample costs two FMAs for q, one for
// z = q alpha + beta, the Horner steps of Pr (which carries -log2(e)/H_r),
// one multiply for the Rayleigh exponent and one for the Mie exponent
// (ratio = H_r/H_m), two SFU exponentials and two adds into four partial
// sums per component.
template <class Real, int NP>
__device__ __forceinline__ void sun_sums(Real q0, Real b, Real dt, int steps, const Real* pr, Real alpha, Real beta,
                                         Real ratio, Real& sum_r, Real& sum_m) {
  const Real A = fma(dt, fma(Real(0.25), dt, b), q0);
  const Real B = dt * fma(Real(2), b, dt);
  const Real C = dt * dt;
  // sample n = 4m + u: q = A_u + f (B_u + f C) with f = 4m, A_u = A + u (B + u C),
  // B_u = B + 2 u C, so the counter f advances once per four samples
  Real Au[4], Bu[4];
#pragma unroll
  for (int u = 0; u < 4; u++) {
    Au[u] = fma(Real(u), fma(Real(u), C, B), A);
    Bu[u] = fma(Real(2 * u), C, B);
  }
  Real sr[4] = {0, 0, 0, 0}, sm[4] = {0, 0, 0, 0};
  Real f = 0;
  int n = 0;
  if constexpr (std::is_same<Real, float>::value) {
    // samples u = 0, 1 and u = 2, 3 as pairs of FP32 lanes (FFMA2/FMUL2/
    // FADD2, each lane rounded as the scalar operation): the same values
    // in half the instructions
    float2 A2[2], B2[2], pr2[NP], s_r[2], s_m[2];
    const float2 C2 = make_float2(C, C), al2 = make_float2(alpha, alpha), be2 = make_float2(beta, beta);
    const float2 ra2 = make_float2(ratio, ratio), four = make_float2(4.0f, 4.0f);
#pragma unroll
    for (int k = 0; k < NP; k++) pr2[k] = make_float2(pr[k], pr[k]);
#pragma unroll
    for (int h = 0; h < 2; h++) {
      A2[h] = make_float2(Au[2 * h], Au[2 * h + 1]);
      B2[h] = make_float2(Bu[2 * h], Bu[2 * h + 1]);
      s_r[h] = make_float2(0.0f, 0.0f);
      s_m[h] = make_float2(0.0f, 0.0f);
    }
    float2 f2 = make_float2(0.0f, 0.0f);
    for (; n + 4 <= steps; n += 4) {
#pragma unroll
      for (int h = 0; h < 2; h++) {
        const float2 q = __ffma2_rn(f2, __ffma2_rn(f2, C2, B2[h]), A2[h]);
        const float2 z = __ffma2_rn(q, al2, be2);
        float2 p = pr2[NP - 1];
#pragma unroll
        for (int k = NP - 2; k >= 0; k--) p = __ffma2_rn(p, z, pr2[k]);
        const float2 xr = __fmul2_rn(q, p);
        const float2 xm = __fmul2_rn(xr, ra2);
        s_r[h] = __fadd2_rn(s_r[h], make_float2(Bulk<float>::exp2(xr.x), Bulk<float>::exp2(xr.y)));
        s_m[h] = __fadd2_rn(s_m[h], make_float2(Bulk<float>::exp2(xm.x), Bulk<float>::exp2(xm.y)));
      }
      f2 = __fadd2_rn(f2, four);
    }
    sr[0] = s_r[0].x, sr[1] = s_r[0].y, sr[2] = s_r[1].x, sr[3] = s_r[1].y;
    sm[0] = s_m[0].x, sm[1] = s_m[0].y, sm[2] = s_m[1].x, sm[3] = s_m[1].y;
  } else {
    for (; n + 4 <= steps; n += 4) {
#pragma unroll
      for (int u = 0; u < 4; u++) {
        const Real q = fma(f, fma(f, C, Bu[u]), Au[u]);
        const Real z = fma(q, alpha, beta);
        Real p = pr[NP - 1];
#pragma unroll
        for (int k = NP - 2; k >= 0; k--) p = fma(p, z, pr[k]);
        const Real xr = q * p;
        sr[u] += Bulk<Real>::exp2(xr);
        sm[u] += Bulk<Real>::exp2(xr * ratio);
      }
      f += Real(4);
    }
  }
  for (; n < steps; n++) {
    const Real fn = Real(n);
    const Real q = fma(fn, fma(fn, C, B), A);
    const Real z = fma(q, alpha, beta);
    Real p = pr[NP - 1];
#pragma unroll
    for (int k = NP - 2; k >= 0; k--) p = fma(p, z, pr[k]);
    const Real xr = q * p;
    sr[0] += Bulk<Real>::exp2(xr);
    sm[0] += Bulk<Real>::exp2(xr * ratio);
  }
  sum_r = (sr[0] + sr[1]) + (sr[2] + sr[3]);
  sum_m = (sm[0] + sm[1]) + (sm[2] + sm[3]);
}

// Same sums for a segment parameterised by u in [0, 1], with the height
// coordinate written as q = A + w (B + w C) in w = u - u0: the samples are
// w_n = w0 + n du.
template <class Real, int NP>
__device__ __forceinline__ void optical_sums_w(Real A, Real B, Real C, Real w0, Real du, int steps, const Real* c,
                                               Real alpha, Real beta, Real kr, Real km, Real& sum_r, Real& sum_m) {
  Real sr = 0, cr = 0, sm = 0, cm = 0;
  Real fn = 0;
  for (int n = 0; n < steps; n++) {
    Real w = fma(fn, du, w0);
    Real q = fma(w, fma(w, C, B), A);
    Real h = height_from_q<Real, NP>(q, c, alpha, beta);
    Real er = Bulk<Real>::exp2(h * kr);
    Real em = Bulk<Real>::exp2(h * km);
    kahan_add(sr, cr, er);
    kahan_add(sm, cm, em);
    fn += Real(1);
  }
  sum_r = sr;
  sum_m = sm;
}

// q(u) = c0 + u (two_xd + u dd) with two_xd = 2 x.D, dd = D.D.
template <class Real, int NP>
__device__ __forceinline__ void optical_sums_u(Real c0, Real two_xd, Real dd, Real du, int steps, const Real* c,
                                               Real alpha, Real beta, Real kr, Real km, Real& sum_r, Real& sum_m) {
  optical_sums_w<Real, NP>(c0, two_xd, dd, Real(0.5) * du, du, steps, c, alpha, beta, kr, km, sum_r, sum_m);
}

// The height form of the segment x -> x + D from its FP64 invariants c0 =
// |x|^2 - R^2, x.D and D.D.  Plain: q = c0 + u (2 x.D + u D.D).  About the
// closest approach u* = -x.D / D.D: q = qmin + D.D (u - u*)^2 with qmin = c0 -
// (x.D)^2 / D.D computed in FP64.  A grazing segment (|qmin| < c0) takes the
// second form: the plain one rounds c0 and x.D to Real, an error of about
// 1e-7 c0 in q at every sample, which near the tangent point is a height
// offset of millimetres where the density is largest (a systematic 1e-5 in
// the optical depth of a Mie-dense grazing ray); about u* the samples keep
// their heights to 1e-7 of the height above qmin, and rounding u* only shifts
// all samples together.  Steeper segments keep the plain form, which does not
// cancel there.
struct QForm {
  double A, B, C, w0;
};
__device__ __forceinline__ QForm segment_q_form(double c0, double xD, double DD, double du) {
  QForm f;
  f.C = DD;
  const double qmin = DD > 0.0 ? c0 - xD * xD / DD : c0;
  if (DD > 0.0 && fabs(qmin) < c0) {
    f.A = qmin;
    f.B = 0.0;
    f.w0 = 0.5 * du + xD / DD;  // u_0 - u* with u_0 = du / 2
  } else {
    f.A = c0;
    f.B = 2.0 * xD;
    f.w0 = 0.5 * du;
  }
  return f;
}

// Optical depth (RGB) of a segment from x to x + D with `steps` midpoint
// samples (ray.clj:19-30 with atmosphere.clj:114-125), from the segment's
// FP64 invariants: c0 = |x|^2 - R^2, x.D, D.D and L = |D| (a view row's
// sample segments are the row's segment scaled).
template <class Real>
__device__ inline void segment_depth_q(const AtmoParams& P, double c0, double xD, double DD, double L, int steps,
                                       Real tau[3]) {
  if (!(L > 0.0)) {
    tau[0] = tau[1] = tau[2] = 0;
    return;
  }
  const double du = 1.0 / steps;
  const QForm f = segment_q_form(c0, xD, DD, du);
  Real sr, sm;
  optical_sums_w<Real, 5>((Real)f.A, (Real)f.B, (Real)f.C, (Real)f.w0, (Real)du, steps, Bulk<Real>::hpoly(P),
                          Bulk<Real>::alpha(P), Bulk<Real>::beta(P), Bulk<Real>::kr(P), Bulk<Real>::km(P), sr, sm);
  Real a = (Real)(L / steps);
#pragma unroll
  for (int ch = 0; ch < 3; ch++) tau[ch] = a * (Bulk<Real>::ray_ext(P, ch) * sr + Bulk<Real>::mie_ext(P, ch) * sm);
}

// The same for x and D in FP64.
template <class Real>
__device__ inline void segment_depth(const AtmoParams& P, d3 x, d3 D, int steps, Real tau[3]) {
  const double c0 = (mag3(x) - P.R) * (mag3(x) + P.R);
  segment_depth_q<Real>(P, c0, dot3(x, D), dot3(D, D), mag3(D), steps, tau);
}

template <class Real>
__device__ __forceinline__ Real exp_neg(Real tau) {
  return Bulk<Real>::exp2(tau * Real(-1.4426950408889634));
}

// ---------------------------------------------------------------------------
// Table gathers
// ---------------------------------------------------------------------------

// Index of a 4-D texel.
__device__ __forceinline__ long long idx4(const BuildDims& d, int i, int j, int k, int a) {
  return (((long long)i * d.n1 + j) * d.n2 + k) * d.n3 + a;
}

template <class Real>
__device__ __forceinline__ void ld3(const Vec4<Real>* t, long long i, Real o[3]) {
  Vec4<Real> v = t[i];
  o[0] = v.x;
  o[1] = v.y;
  o[2] = v.z;
}

template <class Real>
__device__ __forceinline__ void mix3(const Real* a, const Real* b, Real s, Real* o) {
#pragma unroll
  for (int c = 0; c < 3; c++) o[c] = a[c] * (Real(1) - s) + b[c] * s;
}

// Clamped quadrilinear interpolation of a 4-D table (interpolate.clj:87-98:
// the innermost dimension is mixed first).  With SKIP, a dimension whose
// fraction is exactly 0 gives its upper corners weight 0, and
// mix3(a, b, 0) = a exactly for finite b, so those corners are not loaded:
// for the re-interpolation maps, which are integers in most dimensions of
// most nodes (elsewhere the tests cost more than they save).
template <class Real, bool SKIP = false>
__device__ inline void interp4(const Vec4<Real>* t, const BuildDims& d, const int* u, const Real* s, Real out[3]) {
  const int v[4] = {upper_index(u[0], d.n0), upper_index(u[1], d.n1), upper_index(u[2], d.n2),
                    upper_index(u[3], d.n3)};
  const bool two[4] = {!SKIP || s[0] != Real(0), !SKIP || s[1] != Real(0), !SKIP || s[2] != Real(0),
                       !SKIP || s[3] != Real(0)};
  Real rh[2][3];
#pragma unroll
  for (int h = 0; h < 2; h++) {
    Real re[2][3];
    if (h == 1 && !two[0]) {
#pragma unroll
      for (int c = 0; c < 3; c++) rh[1][c] = rh[0][c];
      continue;
    }
#pragma unroll
    for (int e = 0; e < 2; e++) {
      Real rk[2][3];
      if (e == 1 && !two[1]) {
#pragma unroll
        for (int c = 0; c < 3; c++) re[1][c] = re[0][c];
        continue;
      }
#pragma unroll
      for (int k = 0; k < 2; k++) {
        Real A[3], B[3];
        if (k == 1 && !two[2]) {
#pragma unroll
          for (int c = 0; c < 3; c++) rk[1][c] = rk[0][c];
          continue;
        }
        const int ih = h ? v[0] : u[0], ie = e ? v[1] : u[1], ik = k ? v[2] : u[2];
        ld3(t, idx4(d, ih, ie, ik, u[3]), A);
        if (two[3]) {
          ld3(t, idx4(d, ih, ie, ik, v[3]), B);
        } else {
#pragma unroll
          for (int c = 0; c < 3; c++) B[c] = A[c];
        }
        mix3(A, B, s[3], rk[k]);
      }
      mix3(rk[0], rk[1], s[2], re[e]);
    }
    mix3(re[0], re[1], s[1], rh[h]);
  }
  mix3(rh[0], rh[1], s[0], out);
}

template <class Real>
__device__ inline void interp2(const Vec4<Real>* t, int n0, int n1, const int* u, const Real* s, Real out[3]) {
  const int v0 = upper_index(u[0], n0), v1 = upper_index(u[1], n1);
  Real A[3], B[3], lo[3], hi[3];
  ld3(t, (long long)u[0] * n1 + u[1], A);
  ld3(t, (long long)u[0] * n1 + v1, B);
  mix3(A, B, s[1], lo);
  ld3(t, (long long)v0 * n1 + u[1], A);
  ld3(t, (long long)v0 * n1 + v1, B);
  mix3(A, B, s[1], hi);
  mix3(lo, hi, s[0], out);
}

// (1 - exp(-3 s - 0.6)) / (1 - exp(-3.6)) clamped at 0, times (size - 1)
// (sun-elevation-to-index, atmosphere.clj:322-326) in Real.
template <class Real>
__device__ __forceinline__ Real sun_elevation_index_r(Real sin_el, Real scale) {
  const Real e = Bulk<Real>::exp2((Real(3) * sin_el + Real(0.6)) * Real(-1.4426950408889634));
  const Real r = (Real(1) - e) * scale;
  return r > Real(0) ? r : Real(0);
}

// sun_elevation_index_r for two values: the same operations per lane.
template <class Real>
__device__ __forceinline__ V2<Real> sun_elevation_index_r2(V2<Real> sin_el, Real scale) {
  const V2<Real> z = mul2(fma2(mk2(Real(3), Real(3)), sin_el, mk2(Real(0.6), Real(0.6))),
                          mk2(Real(-1.4426950408889634), Real(-1.4426950408889634)));
  const V2<Real> e = mk2(Bulk<Real>::exp2(z.x), Bulk<Real>::exp2(z.y));
  const V2<Real> r = mul2(sub2(mk2(Real(1), Real(1)), e), mk2(scale, scale));
  return mk2(r.x > Real(0) ? r.x : Real(0), r.y > Real(0) ? r.y : Real(0));
}

}  // namespace sfsim
