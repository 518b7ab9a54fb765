// atmo_params.h -- parameters and buffer records shared by the host driver and
// the CUDA kernels of the atmosphere lookup-table build.
#pragma once

#include <cstddef>
#include <cstdint>

#ifdef __CUDACC__
#define SFSIM_HD __host__ __device__
#else
#define SFSIM_HD
#endif

namespace sfsim {

constexpr int kMaxHPoly = 8;  // coefficients of the height-from-q polynomial

// One atmosphere.  Geometry in FP64; the bulk constants also as float so the
// FP32 kernels read them without conversions.
struct AtmoParams {
  // geometry
  double R, H, top;        // ground radius, atmosphere height, top radius
  double R2, top2;         // squares
  double Hh, Hh2;          // horizon distance at the top: sqrt(top^2 - R^2), and its square
  // components; mie is scatter[0], rayleigh scatter[1] (atmosphere_lut.clj:63)
  double mie_base[3], mie_scale, mie_quot, mie_g;
  double ray_base[3], ray_scale, ray_quot, ray_g;
  double brightness[3], intensity[3];
  // bulk constants
  double d_mie_ext[3], d_ray_ext[3];  // base / quotient
  double d_km, d_kr;                  // -log2(e) / scale height
  double d_hpoly[kMaxHPoly];          // h(q) = q * P(q * alpha + beta)
  double d_alpha, d_beta;
  double d_hpr[kMaxHPoly];            // -log2(e)/H_rayleigh * h(q) = q * Pr(z)
  double d_hratio;                    // H_rayleigh / H_mie
  float f_mie_ext[3], f_ray_ext[3];
  float f_mie_base[3], f_ray_base[3];
  float f_km, f_kr;
  float f_hpoly[kMaxHPoly];
  float f_alpha, f_beta;
  float f_hpr[kMaxHPoly];
  float f_hpr4[4];                    // degree-3 fit of the same, for the FP32 sun-ray loop
  float f_hratio;
  float f_R, f_Hh2, f_mie_g;
  float f_bright_pi[3];               // brightness / pi
  float f_intensity[3];
  // Cornette-Shanks phase as k (1 + mu^2) (a + b mu)^-3/2: {k, a, b} with
  // k = 3 (1 - g^2) / (8 pi (2 + g^2)), a = 1 + g^2, b = -2 g
  double d_phR[3], d_phM[3];
  float f_phR[3], f_phM[3];
  // intensity * scatter base, the first-order source factors
  double d_srcR[3], d_srcM[3];
  float f_srcR[3], f_srcM[3];
  float f_top, f_Hh;
  // descending sun-ray table of the FP32 first order: atmosphere height and
  // the distance scale s of its asinh coordinate (and 1 / s)
  float f_H, f_desc_s, f_desc_inv_s;
  // climbing sun rays from q >= f_sun_qlim are integrated directly (the top
  // rows of the climbing table where the density at the top matters)
  float f_sun_qlim;
  int hpoly_n;                        // number of coefficients
};

// Shapes, steps and sizes shared by every atmosphere of one batched build.
struct BuildDims {
  int B;                   // atmospheres
  int nT0, nT1;            // transmittance [height][elevation]
  int nE0, nE1;            // surface radiance [height][sun elevation]
  int n0, n1, n2, n3;      // ray scatter [height][elevation][sun elevation][sun heading]
  int S;                   // ray steps
  int sphere_steps;        // point-scatter sphere steps
  int P;                   // directions of integral-sphere(sphere_steps)
  int Ph;                  // directions of integral-half-sphere(ray_steps)
  int iterations;
  double inv_S;            // 1 / S, the view rays' step in their parameter
  int scan_rays;           // view-ray transmittances by prefix scan (SFSIM_ATMO_SCAN_RAYS)
  // (size - 1) / (1 - exp(-3.6)) of the sun-elevation axes of the ray-scatter
  // space (n2) and of the surface-radiance space (nE1)
  double sun_scale, sun_scale_E;
  float f_sun_scale, f_sun_scale_E;
  SFSIM_HD long long nT() const { return (long long)nT0 * nT1; }
  SFSIM_HD long long nE() const { return (long long)nE0 * nE1; }
  SFSIM_HD long long n4() const { return (long long)n0 * n1 * n2 * n3; }
  SFSIM_HD long long rows() const { return (long long)n0 * n1; }
};

// A sample direction of a spherical integral in the local frame
// (cos theta, sin theta cos phi, sin theta sin phi) with its quadrature weight.
struct DirLocal {
  double x, y, z, w;
};

// Interpolation coordinate of one table dimension: lower index and fraction.
template <class Real>
struct alignas(2 * sizeof(Real) >= 8 ? 2 * sizeof(Real) : 8) Coord {
  int u;
  Real s;
};

// Re-interpolation coordinates of a 4-D node (forward of backward of the node).
template <class Real>
struct Remap4 {
  int u[4];
  Real s[4];
};

template <class Real>
struct Remap2 {
  int u[2];
  Real s[2];
};

template <class Real>
struct alignas(4 * sizeof(Real)) Vec4 {
  Real x, y, z, w;
};

// Light direction and view-light cosine of a 4-D node, computed once in FP64
// (index-to-sun-direction, atmosphere.clj:375-384) and stored in Real.
template <class Real>
struct alignas(4 * sizeof(Real)) CellGeom {
  Real lx, ly, lz, mu;
};

// Per view row (height i, elevation j) of the 4-D space, FP64, with FP32
// copies for the FP32 kernels.
struct RowInfo {
  double r;            // |x|, x = (r, 0, 0)
  double sv, cv;       // view direction (sv, cv, 0)
  double D[3];         // ray segment from x to its extremity
  double L;            // |D|
  double Ls;           // L / ray steps
  // the height form of the segment x -> x + D about its closest approach
  // (segment_q_form): qmin = c0 - (x.D)^2 / D.D and t = x.D / D.D (0 when
  // D.D = 0); a sample segment x -> x + su D has the same qmin and t / su
  double qmin, t;
  float f_r, f_sv, f_cv, f_D[3], f_Ls;
  int above;           // above-horizon flag of the node
};

// Per (height i, sun elevation k) of the 4-D space, from FP64: the height
// and sun-elevation coordinates of the dS lookups at x = (r_i, 0, 0) (also
// those of every node (i, ., k, .), whose light direction has x.l = r_i sin),
// and the scattering coefficients beta(x) point scatter multiplies its sums
// with.
template <class Real>
struct PointRow {
  double ss;  // sin of the sun elevation of index k (index-to-sin-sun-elevation)
  double cs;  // sqrt(max(0, 1 - ss^2)), the bound of index-to-sun-direction's second component
  int u0, u2;
  Real s0, s2;
  Real bR[3], bM[3];
  Real gA;    // r ss / R: with x = (r, 0, 0), a ground point g = x + t omega (|g| = R) has
              // g.l / |g| = gA + (t / R) (omega . l), since l has first component ss
};

// Per node (height iE, sun elevation kE) of the surface-radiance space, from
// FP64: the dS lookup's height and sun-elevation coordinates at x = (r, 0, 0)
// and the terms of the elevation coordinate of (x, w) (atmosphere.clj:239-253):
// H^2 - q, 2 rho + 2 H, r; and the light direction (lx, ly, 0).
template <class Real>
struct SurfRow {
  int u0, u2;
  Real s0, s2;
  Real Hh2mq, den, rr, lx, ly;
};

// A direction of the surface-radiance half-sphere integral in world
// coordinates at the height of row iE: its first two components and its
// quadrature weight times w.n.
template <class Real>
struct HalfDir {
  Real wx, wy, wgt;
};

// Per view row and ray sample s (p_s = x + D (s + 1/2)/S).
template <class Real>
struct RowSample {
  Real tau[3];         // optical depth from x to p_s (RGB)
  Real er, em;         // exp(-h/H_rayleigh), exp(-h/H_mie) at p_s
  Real q;              // |p_s|^2 - R^2
  Real us;             // (s + 1/2)/S
  Real inv_r;          // 1/|p_s|
  int u0, u1;          // height and elevation coordinates of p_s in the 4-D space
  Real s0, s1;
  Real pad;
};

// Per height row i and sphere direction of point scatter.
template <class Real>
struct SphereDir {
  Real w[3];           // direction omega in world coordinates
  Real weight;         // quadrature weight (ring factor * 2 pi / ring steps)
  Real tR;             // ground distance / R (surface directions): the ground point's sin of the
                       // sun elevation is gA + tR (omega . l), gA of the (height, sun elevation) row
  Real ground[3];      // T(x, g) * brightness / pi (surface directions)
  int surface;         // 1: the direction ends on the ground
  int u1;              // elevation coordinate of (x, omega, !surface)
  int uE0;             // height coordinate of the ground point in the surface space
  int pad;             // 1: a zero-weight filler of the partitioned lists
  Real s1, sE0;
};

}  // namespace sfsim
