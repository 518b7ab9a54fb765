// atmo_api.cu -- C ABI of the atmosphere LUT builder (include/sfsim_atmo.h):
// validation, parameter set-up, the device workspace and the order loop of
// generate-atmosphere-luts (src/clj/sfsim/atmosphere_lut.clj:43-105).
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/sfsim_atmo.h"
#include "../../include/sfsim_noise.h"
#include "atmo_device.cuh"
#include "kernels.h"

namespace sfsim {
template <class Real>
size_t point_scatter_smem(const BuildDims& d, bool first);
template <class Real>
size_t ray_scatter_smem(const BuildDims& d);
}

using namespace sfsim;

namespace {

constexpr size_t kMaxSmem = 227 * 1024;

thread_local std::string g_last_error;
std::mutex g_mutex;
bool g_timing = false;
int g_launches = 0;
constexpr int kStages = 10;
double g_stage_ms[kStages];
// stage names of the timings and of the NVTX ranges
const char* const kStageNames[kStages] = {"set-up",    "transmittance",    "surface base", "first order",
                                          "reserved",  "point scatter",    "surface radiance",
                                          "ray scatter", "accumulate", "output"};
int g_have_timings = 0;
// bytes the last build copied host -> device and device -> host
unsigned long long g_h2d_bytes = 0, g_d2h_bytes = 0;

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

#define CUDA_TRY(expr)                                                                              \
  do {                                                                                              \
    cudaError_t _e = (expr);                                                                        \
    if (_e != cudaSuccess) return fail(SFSIM_ATMO_ECUDA, std::string(#expr) + ": " + cudaGetErrorString(_e)); \
  } while (0)

// ---------------------------------------------------------------------------
// configuration
// ---------------------------------------------------------------------------

int validate(const sfsim_atmo_config* c) {
  if (!c) return fail(SFSIM_ATMO_ENULL, "config is NULL");
  if (!(c->radius > 0) || !(c->height > 0) || !std::isfinite(c->radius) || !std::isfinite(c->height))
    return fail(SFSIM_ATMO_EINVAL, "radius and height must be positive and finite");
  const sfsim_atmo_component* comps[2] = {&c->mie, &c->rayleigh};
  for (int i = 0; i < 2; i++) {
    const sfsim_atmo_component* k = comps[i];
    if (!(k->scatter_scale > 0) || !(k->scatter_quotient > 0) || !std::isfinite(k->scatter_g) ||
        std::fabs(k->scatter_g) >= 1.0)
      return fail(SFSIM_ATMO_EINVAL, "component scale and quotient must be positive and |g| < 1");
    for (int ch = 0; ch < 3; ch++)
      if (!(k->scatter_base[ch] >= 0) || !std::isfinite(k->scatter_base[ch]))
        return fail(SFSIM_ATMO_EINVAL, "scatter base must be finite and non-negative");
  }
  for (int ch = 0; ch < 3; ch++)
    if (!std::isfinite(c->brightness[ch]) || !std::isfinite(c->intensity[ch]))
      return fail(SFSIM_ATMO_EINVAL, "brightness and intensity must be finite");
  for (int i = 0; i < 2; i++)
    if (c->transmittance_shape[i] < 2 || c->surface_radiance_shape[i] < 2)
      return fail(SFSIM_ATMO_ESHAPE, "every table dimension needs at least 2 nodes");
  for (int i = 0; i < 4; i++)
    if (c->ray_scatter_shape[i] < 2) return fail(SFSIM_ATMO_ESHAPE, "every table dimension needs at least 2 nodes");
  if (c->ray_steps < 1 || c->ray_steps > 4096) return fail(SFSIM_ATMO_EINVAL, "ray_steps must be in [1, 4096]");
  if (c->iterations < 0 || c->iterations > 64) return fail(SFSIM_ATMO_EINVAL, "iterations must be in [0, 64]");
  if (c->sphere_steps < 0 || c->sphere_steps > 1024)
    return fail(SFSIM_ATMO_EINVAL, "sphere_steps must be in [0, 1024]");
  if (c->iterations > 0 && c->sphere_steps < 2)
    return fail(SFSIM_ATMO_EINVAL, "sphere_steps must be in [2, 1024] when there are iterations");
  if (c->iterations > 0 && c->ray_steps < 4)
    return fail(SFSIM_ATMO_EINVAL, "ray_steps must be at least 4 (surface radiance uses ray_steps/4 rings)");
  if (c->precision != SFSIM_ATMO_FP32 && c->precision != SFSIM_ATMO_FP64)
    return fail(SFSIM_ATMO_EINVAL, "precision must be SFSIM_ATMO_FP32 or SFSIM_ATMO_FP64");
  if (c->flags & ~SFSIM_ATMO_SCAN_RAYS) return fail(SFSIM_ATMO_EINVAL, "flags has an unknown bit");
  long long n4 = 1;
  for (int i = 0; i < 4; i++) n4 *= c->ray_scatter_shape[i];
  if (n4 > (1LL << 31)) return fail(SFSIM_ATMO_ETOOBIG, "ray-scatter table exceeds 2^31 nodes");
  return 0;
}

bool same_layout(const sfsim_atmo_config& a, const sfsim_atmo_config& b) {
  return memcmp(a.transmittance_shape, b.transmittance_shape, sizeof(a.transmittance_shape)) == 0 &&
         memcmp(a.surface_radiance_shape, b.surface_radiance_shape, sizeof(a.surface_radiance_shape)) == 0 &&
         memcmp(a.ray_scatter_shape, b.ray_scatter_shape, sizeof(a.ray_scatter_shape)) == 0 &&
         a.ray_steps == b.ray_steps && a.sphere_steps == b.sphere_steps && a.iterations == b.iterations &&
         a.precision == b.precision && a.flags == b.flags;
}

// Directions of spherical-integral (sphere.clj:62-93): theta rings at
// midpoints, ceil(sin theta * phi_steps) phi midpoints per ring, weight
// (cos(theta - d) - cos(theta + d)) * 2 pi / ring steps.
void sphere_directions(int theta_steps, int phi_steps, double range, std::vector<DirLocal>& out) {
  out.clear();
  if (theta_steps <= 0) return;
  const double delta2 = range / theta_steps / 2;
  for (int k = 0; k < theta_steps; k++) {
    const double theta = range * ((0.5 + k) / theta_steps);
    const double factor = std::cos(theta - delta2) - std::cos(theta + delta2);
    const int ringsteps = (int)std::ceil(std::sin(theta) * phi_steps);
    const double weight = (2 * M_PI) / ringsteps;
    for (int i = 0; i < ringsteps; i++) {
      const double phi = 2 * M_PI * ((0.5 + i) / ringsteps);
      out.push_back(DirLocal{std::cos(theta), std::sin(theta) * std::cos(phi), std::sin(theta) * std::sin(phi),
                             factor * weight});
    }
  }
}

// h(q) = q / (R + sqrt(R^2 + q)) = q * f(q); f is interpolated at 5
// Chebyshev nodes over q in [-0.01, 1.05] * (top^2 - R^2) and stored as a
// polynomial in z = q * alpha + beta, z in [-1, 1].
// Chebyshev interpolant of f(q) = 1/(R + sqrt(R^2 + q)) with N nodes on
// [qlo, qhi], as monomial coefficients in z = q alpha + beta; returns the
// largest relative error on a fine grid.
double chebyshev_height_fit(const AtmoParams& P, int N, double qlo, double qhi, double* mono) {
  const double alpha = 2.0 / (qhi - qlo), beta = -(qhi + qlo) / (qhi - qlo);
  auto f = [&](double q) { return 1.0 / (P.R + std::sqrt(P.R2 + q)); };
  double cheb[8] = {};
  for (int j = 0; j < N; j++) {
    double s = 0;
    for (int k = 0; k < N; k++) {
      const double t = M_PI * (k + 0.5) / N;
      s += f((std::cos(t) - beta) / alpha) * std::cos(j * t);
    }
    cheb[j] = s * (j == 0 ? 1.0 : 2.0) / N;
  }
  double T[8][8] = {};
  T[0][0] = 1;
  T[1][1] = 1;
  for (int j = 2; j < N; j++)
    for (int k = 0; k < N; k++) T[j][k] = (k > 0 ? 2 * T[j - 1][k - 1] : 0) - T[j - 2][k];
  for (int k = 0; k < N; k++) {
    mono[k] = 0;
    for (int j = 0; j < N; j++) mono[k] += cheb[j] * T[j][k];
  }
  double worst = 0;
  for (int k = 0; k <= 1000; k++) {
    const double q = qlo + (qhi - qlo) * k / 1000.0;
    const double z = q * alpha + beta;
    double p = mono[N - 1];
    for (int m = N - 2; m >= 0; m--) p = p * z + mono[m];
    worst = std::fmax(worst, std::fabs(p / f(q) - 1));
  }
  return worst;
}

int fit_height_polynomial(AtmoParams& P) {
  constexpr int N = 5;
  const double qlo = -0.01 * P.Hh2, qhi = 1.05 * P.Hh2;
  const double alpha = 2.0 / (qhi - qlo), beta = -(qhi + qlo) / (qhi - qlo);
  auto f = [&](double q) { return 1.0 / (P.R + std::sqrt(P.R2 + q)); };
  double cheb[N];
  for (int j = 0; j < N; j++) {
    double s = 0;
    for (int k = 0; k < N; k++) {
      const double t = M_PI * (k + 0.5) / N;
      const double z = std::cos(t);
      s += f((z - beta) / alpha) * std::cos(j * t);
    }
    cheb[j] = s * (j == 0 ? 1.0 : 2.0) / N;
  }
  // Chebyshev -> monomial in z
  double T[N][N] = {};
  T[0][0] = 1;
  T[1][1] = 1;
  for (int j = 2; j < N; j++)
    for (int k = 0; k < N; k++) T[j][k] = (k > 0 ? 2 * T[j - 1][k - 1] : 0) - T[j - 2][k];
  double mono[N] = {};
  for (int j = 0; j < N; j++)
    for (int k = 0; k < N; k++) mono[k] += cheb[j] * T[j][k];
  double worst = 0;
  for (int k = 0; k <= 1000; k++) {
    const double q = qlo + (qhi - qlo) * k / 1000.0;
    const double z = q * alpha + beta;
    double p = mono[N - 1];
    for (int m = N - 2; m >= 0; m--) p = p * z + mono[m];
    worst = std::fmax(worst, std::fabs(p / f(q) - 1));
  }
  if (worst > 1e-8) return fail(SFSIM_ATMO_EINVAL, "atmosphere too thick for the height polynomial");
  for (int k = 0; k < kMaxHPoly; k++) {
    P.d_hpoly[k] = k < N ? mono[k] : 0.0;
    P.f_hpoly[k] = (float)P.d_hpoly[k];
  }
  P.hpoly_n = N;
  const double kr = -1.4426950408889634 / P.ray_scale;
  for (int k = 0; k < kMaxHPoly; k++) {
    P.d_hpr[k] = P.d_hpoly[k] * kr;
    P.f_hpr[k] = (float)P.d_hpr[k];
  }
  {
    double mono4[8];
    if (chebyshev_height_fit(P, 4, qlo, qhi, mono4) > 1e-7)
      return fail(SFSIM_ATMO_EINVAL, "atmosphere too thick for the degree-3 height polynomial");
    for (int k = 0; k < 4; k++) P.f_hpr4[k] = (float)(mono4[k] * kr);
  }
  P.d_hratio = P.ray_scale / P.mie_scale;
  P.f_hratio = (float)P.d_hratio;
  P.d_alpha = alpha;
  P.d_beta = beta;
  P.f_alpha = (float)alpha;
  P.f_beta = (float)beta;
  return 0;
}

int make_params(const sfsim_atmo_config& c, AtmoParams& P) {
  memset(&P, 0, sizeof(P));
  P.R = c.radius;
  P.H = c.height;
  P.top = c.radius + c.height;
  P.R2 = c.radius * c.radius;
  P.top2 = P.top * P.top;
  P.Hh = std::sqrt(P.top2 - P.R2);
  P.Hh2 = P.Hh * P.Hh;
  for (int ch = 0; ch < 3; ch++) {
    P.mie_base[ch] = c.mie.scatter_base[ch];
    P.ray_base[ch] = c.rayleigh.scatter_base[ch];
    P.brightness[ch] = c.brightness[ch];
    P.intensity[ch] = c.intensity[ch];
    P.d_mie_ext[ch] = c.mie.scatter_base[ch] / c.mie.scatter_quotient;
    P.d_ray_ext[ch] = c.rayleigh.scatter_base[ch] / c.rayleigh.scatter_quotient;
    P.f_mie_ext[ch] = (float)P.d_mie_ext[ch];
    P.f_ray_ext[ch] = (float)P.d_ray_ext[ch];
    P.f_mie_base[ch] = (float)P.mie_base[ch];
    P.f_ray_base[ch] = (float)P.ray_base[ch];
    P.f_bright_pi[ch] = (float)(c.brightness[ch] / M_PI);
    P.f_intensity[ch] = (float)c.intensity[ch];
  }
  P.mie_scale = c.mie.scatter_scale;
  P.mie_quot = c.mie.scatter_quotient;
  P.mie_g = c.mie.scatter_g;
  P.ray_scale = c.rayleigh.scatter_scale;
  P.ray_quot = c.rayleigh.scatter_quotient;
  P.ray_g = c.rayleigh.scatter_g;
  const double log2e = 1.4426950408889634;
  P.d_km = -log2e / P.mie_scale;
  P.d_kr = -log2e / P.ray_scale;
  P.f_km = (float)P.d_km;
  P.f_kr = (float)P.d_kr;
  P.f_R = (float)P.R;
  P.f_Hh2 = (float)P.Hh2;
  P.f_mie_g = (float)P.mie_g;
  P.f_top = (float)P.top;
  P.f_Hh = (float)P.Hh;
  P.f_H = (float)P.H;
  // the descending sun rays' distance to their perigee is tabulated in
  // asinh(d / s): about linear within s of the perigee, where the Mie density
  // peak lies (it spans sqrt(2 R H_mie)), logarithmic beyond
  P.f_desc_s = (float)(1.2 * std::sqrt(2.0 * P.R * P.mie_scale));
  P.f_desc_inv_s = 1.0f / P.f_desc_s;
  // Near the top of the climbing sun-ray table the sums fall to zero like
  // sqrt(q_top - q), which bilinear interpolation follows badly: a numpy model
  // put the optical-depth error of the last row at about 0.18 times the
  // Rayleigh density at the top relative to the ground (2.2e-3 in a 35 km
  // atmosphere), 1e-5 eight rows down.  Where that density exceeds 2e-5 the
  // rays starting in the top eight rows are integrated directly; elsewhere
  // (the 100 km atmospheres) the whole table is read.
  {
    const double top_density = std::exp(-P.H / P.ray_scale);
    const double x = (double)(kSunNR - 9) / (double)(kSunNR - 1);
    P.f_sun_qlim = top_density > 2e-5 ? (float)(P.Hh2 * x * x) : 3.0e38f;
  }
  const double gs[2] = {P.ray_g, P.mie_g};
  for (int m = 0; m < 2; m++) {
    const double g = gs[m];
    double* ph = m ? P.d_phM : P.d_phR;
    float* fph = m ? P.f_phM : P.f_phR;
    ph[0] = 3.0 * (1.0 - g * g) / (8.0 * M_PI * (2.0 + g * g));
    ph[1] = 1.0 + g * g;
    ph[2] = -2.0 * g;
    for (int k = 0; k < 3; k++) fph[k] = (float)ph[k];
  }
  for (int ch = 0; ch < 3; ch++) {
    P.d_srcR[ch] = P.intensity[ch] * P.ray_base[ch];
    P.d_srcM[ch] = P.intensity[ch] * P.mie_base[ch];
    P.f_srcR[ch] = (float)P.d_srcR[ch];
    P.f_srcM[ch] = (float)P.d_srcM[ch];
  }
  return fit_height_polynomial(P);
}

BuildDims make_dims(const sfsim_atmo_config& c, int B) {
  BuildDims d;
  d.B = B;
  d.nT0 = c.transmittance_shape[0];
  d.nT1 = c.transmittance_shape[1];
  d.nE0 = c.surface_radiance_shape[0];
  d.nE1 = c.surface_radiance_shape[1];
  d.n0 = c.ray_scatter_shape[0];
  d.n1 = c.ray_scatter_shape[1];
  d.n2 = c.ray_scatter_shape[2];
  d.n3 = c.ray_scatter_shape[3];
  d.S = c.ray_steps;
  d.sphere_steps = c.sphere_steps;
  d.iterations = c.iterations;
  d.scan_rays = (c.flags & SFSIM_ATMO_SCAN_RAYS) ? 1 : 0;
  d.inv_S = 1.0 / c.ray_steps;
  std::vector<DirLocal> v;
  sphere_directions(c.sphere_steps >> 1, c.sphere_steps, M_PI, v);
  d.P = (int)v.size();
  sphere_directions(c.ray_steps >> 2, c.ray_steps, M_PI / 2, v);
  d.Ph = (int)v.size();
  d.sun_scale = (d.n2 - 1) / (1 - std::exp(-3.6));
  d.sun_scale_E = (d.nE1 - 1) / (1 - std::exp(-3.6));
  d.f_sun_scale = (float)d.sun_scale;
  d.f_sun_scale_E = (float)d.sun_scale_E;
  return d;
}

template <class Real>
int check_smem(const BuildDims& d) {
  if (point_scatter_smem<Real>(d, true) > kMaxSmem)
    return fail(SFSIM_ATMO_ESHAPE, "elevation x heading slab of point scatter exceeds shared memory");
  if (ray_scatter_smem<Real>(d) > kMaxSmem)
    return fail(SFSIM_ATMO_ESHAPE, "sun elevation x heading plane of ray scatter exceeds shared memory");
  if (first_order_smem<Real>(d, false) > kMaxSmem)
    return fail(SFSIM_ATMO_ESHAPE, "the view rows' samples of the first order exceed shared memory");
  return 0;
}

// ---------------------------------------------------------------------------
// device workspace: one allocation per device, grown on demand
// ---------------------------------------------------------------------------

struct Arena {
  void* base = nullptr;
  size_t size = 0;
};

constexpr int kMaxDevices = 64;
Arena g_arena[kMaxDevices];
cudaStream_t g_stream[kMaxDevices];
cudaEvent_t g_events[kMaxDevices][2 * 512];
// host-output builds: a second stream copies the transmittance and Mie
// tables to the host while the scattering iterations still run
cudaStream_t g_copy_stream[kMaxDevices];
cudaEvent_t g_early_done[kMaxDevices];
// each iteration's surface radiance and accumulation run on a side stream
// beside point and ray scatter (run_build)
cudaStream_t g_side_stream[kMaxDevices];
cudaEvent_t g_side_fork[kMaxDevices], g_side_sr[kMaxDevices], g_side_rs[kMaxDevices], g_side_acc[kMaxDevices],
    g_side_setup[kMaxDevices], g_side_sun[kMaxDevices], g_side_rows[kMaxDevices];

struct Carver {
  char* base;
  size_t off = 0;
  template <class T>
  T* take(size_t count) {
    off = (off + 255) & ~size_t(255);
    T* p = reinterpret_cast<T*>(base ? base + off : nullptr);
    off += count * sizeof(T);
    return p;
  }
};

template <class Real>
struct Work {
  AtmoParams* params;
  DirLocal* dirs;
  DirLocal* hdirs;
  SetupBuffers<Real> setup;
  Vec4<Real>*T, *E0, *dE[2], *Eacc[2];
  Vec4<Real>*S1R, *M, *dS[2], *Sacc[2];
  Real* J;
  Real* hrows;  // point scatter's heading rows per (height, sun elevation)
  float *oT, *oE, *oS, *oM;  // device outputs when the caller passes host buffers
  unsigned char* sun;        // sun-ray optical-depth tables, kSunTableBytes per atmosphere (FP32 builds), or NULL
};

// The sun-ray tables cost kSunTableLen nodes of S samples per atmosphere;
// integrating the lit sun rays directly costs S samples for each lit
// (node, ray sample) pair, about a third of all pairs.  Small builds (the
// 8x16x8x4 case) integrate directly, larger ones (the production and sweep
// tables) read the tables.
inline bool sun_tables_pay(const BuildDims& d) { return (double)d.n4() * d.S / 3.0 > (double)kSunTableLen; }

template <class Real>
size_t carve(Work<Real>& w, char* base, const BuildDims& d, bool outputs, bool sun_table = true) {
  Carver c{base};
  const long long B = d.B;
  w.params = c.take<AtmoParams>(B);
  w.dirs = c.take<DirLocal>(d.P + 1);
  w.hdirs = c.take<DirLocal>(d.Ph + 1);
  w.setup.remapS = c.take<Remap4<Real>>(B * d.n4());
  w.setup.geom = c.take<CellGeom<Real>>(B * d.n4());
  w.setup.remapT = c.take<Remap2<Real>>(B * d.nT());
  w.setup.remapE = c.take<Remap2<Real>>(B * d.nE());
  w.setup.rowinfo = c.take<RowInfo>(B * d.rows());
  w.setup.rowmap = c.take<Remap2<Real>>(B * d.rows());
  w.setup.rows = c.take<RowSample<Real>>(B * d.rows() * d.S);
  w.setup.sdirs = c.take<SphereDir<Real>>(B * d.n0 * (long long)(d.P + 1));
  w.setup.pdirs = c.take<SphereDir<Real>>(B * d.n0 * (long long)dir_row(d.P));
  w.setup.dimage = c.take<unsigned char>(B * d.n0 * dir_image_stride(d, sizeof(Real)));
  w.setup.pcount = c.take<int2>(B * d.n0);
  w.setup.prow = c.take<PointRow<Real>>(B * d.n0 * d.n2);
  w.setup.hdvs = c.take<double>(d.n3);
  w.setup.erow = c.take<SurfRow<Real>>(B * d.nE());
  w.setup.hdir = c.take<HalfDir<Real>>(B * d.nE0 * (long long)d.Ph);
  w.T = c.take<Vec4<Real>>(B * d.nT());
  w.E0 = c.take<Vec4<Real>>(B * d.nE());
  for (int i = 0; i < 2; i++) {
    w.dE[i] = c.take<Vec4<Real>>(B * d.nE());
    w.Eacc[i] = c.take<Vec4<Real>>(B * d.nE());
  }
  w.S1R = c.take<Vec4<Real>>(B * d.n4());
  w.M = c.take<Vec4<Real>>(B * d.n4());
  w.J = c.take<Real>(3 * B * d.n4());  // planar [atmosphere][channel][node]
  w.hrows = c.take<Real>(B * d.n0 * d.n2 * heading_rows_stride(d));
  for (int i = 0; i < 2; i++) {
    w.dS[i] = c.take<Vec4<Real>>(B * d.n4());
    w.Sacc[i] = c.take<Vec4<Real>>(B * d.n4());
  }
  if (outputs) {
    w.oT = c.take<float>(3 * B * d.nT());
    w.oE = c.take<float>(3 * B * d.nE());
    w.oS = c.take<float>(3 * B * d.n4());
    w.oM = c.take<float>(3 * B * d.n4());
  } else {
    w.oT = w.oE = w.oS = w.oM = nullptr;
  }
  w.sun = (sun_table && sizeof(Real) == sizeof(float) && sun_tables_pay(d)) ? c.take<unsigned char>(B * kSunTableBytes)
                                                                             : nullptr;
  return c.off + 256;
}

int current_device(int* dev) {
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) return fail(SFSIM_ATMO_ENODEV, "no CUDA device is visible");
  CUDA_TRY(cudaGetDevice(dev));
  if (*dev < 0 || *dev >= kMaxDevices) return fail(SFSIM_ATMO_ENODEV, "device ordinal out of range");
  return 0;
}

int ensure_arena(int dev, size_t bytes) {
  Arena& a = g_arena[dev];
  if (a.size >= bytes) return 0;
  if (a.base) {
    CUDA_TRY(cudaDeviceSynchronize());
    CUDA_TRY(cudaFree(a.base));
    a.base = nullptr;
    a.size = 0;
  }
  cudaError_t e = cudaMalloc(&a.base, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(SFSIM_ATMO_ENOMEM, std::string("cudaMalloc of workspace failed: ") + cudaGetErrorString(e));
  }
  a.size = bytes;
  return 0;
}

int ensure_stream(int dev) {
  if (!g_stream[dev]) {
    CUDA_TRY(cudaStreamCreateWithFlags(&g_copy_stream[dev], cudaStreamNonBlocking));
    CUDA_TRY(cudaEventCreateWithFlags(&g_early_done[dev], cudaEventDisableTiming));
    CUDA_TRY(cudaStreamCreateWithFlags(&g_stream[dev], cudaStreamNonBlocking));
    CUDA_TRY(cudaStreamCreateWithFlags(&g_side_stream[dev], cudaStreamNonBlocking));
    for (cudaEvent_t* e : {&g_side_fork[dev], &g_side_sr[dev], &g_side_rs[dev], &g_side_acc[dev], &g_side_setup[dev],
                           &g_side_sun[dev], &g_side_rows[dev]})
      CUDA_TRY(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
    for (int i = 0; i < 2 * 512; i++) CUDA_TRY(cudaEventCreate(&g_events[dev][i]));
  }
  return 0;
}

// Stage boundaries of a build: CUDA events on the build stream when timing
// is enabled, and always an NVTX range per stage ("sfsim first order",
// "sfsim iteration 3 ray scatter", ...), so that a profiler can select one
// stage of one iteration (ncu --nvtx --nvtx-include "sfsim iteration 3 ray scatter/").
struct Timer {
  int dev;
  cudaStream_t st;
  int n = 0;
  int stage_of[512];
  int iteration = 0;  // iteration of the stages that follow (1-based); 0 outside the loop
  int open = 0;   // NVTX ranges pushed and not yet popped
  bool side = true;  // stages may run on the device's side stream
  void mark_begin(int stage, cudaStream_t on = nullptr) {
    char name[64];
    if (iteration > 0)
      snprintf(name, sizeof name, "sfsim iteration %d %s", iteration, kStageNames[stage]);
    else
      snprintf(name, sizeof name, "sfsim %s", kStageNames[stage]);
    nvtxRangePushA(name);
    open++;
    if (!g_timing || n >= 511) return;
    stage_of[n / 2] = stage;
    cudaEventRecord(g_events[dev][n++], on ? on : st);
  }
  // `on`: the stream of the matching mark_begin, when not the build stream
  void mark_end(cudaStream_t on = nullptr) {
    if (open > 0) {
      nvtxRangePop();
      open--;
    }
    if (!g_timing || n % 2 == 0) return;
    cudaEventRecord(g_events[dev][n++], on ? on : st);
  }
  ~Timer() {
    for (; open > 0; open--) nvtxRangePop();  // a stage left by an error return
  }
};

// Per-iteration state of sfsim_atmo_build_resumable: where to resume, where
// to copy each iteration's state, and whom to tell.
struct IterationHooks {
  const sfsim_atmo_iteration_state* resume;
  sfsim_atmo_iteration_state* state;
  sfsim_atmo_iteration_fn on_iteration;
  void* user;
};

// The order loop of atmosphere_lut.clj:86-97 with every table resident in
// device memory; outputs are device pointers in the .scatter layout.
template <class Real>
int run_build(const Work<Real>& w, const BuildDims& d, float* oT, float* oE, float* oS, float* oM, cudaStream_t st,
              Timer& tm, const sfsim_atmo_intermediates* inter, Vec4<float>* jsum = nullptr,
              cudaEvent_t early_done = nullptr, const IterationHooks* hooks = nullptr) {
  int launches = 0;
  // The first order needs the sun tables, the rows (row info, point rows)
  // and the view-row samples; each of its blocks forms its cells' light
  // directions itself (as k_remap4 does).  So the build stream runs the rows
  // and the view-row samples, the side stream the sun tables and then the
  // node maps (remap4), the other set-up tables, the transmittance nodes and
  // E0 beside the first order; the outputs and the iterations wait for all
  // of them.  Builds with stage timing on, entry points without a side
  // stream, and rows whose cells' geometry does not fit beside their samples
  // in shared memory keep the node maps before the first order.
  cudaStream_t ss = tm.side ? g_side_stream[tm.dev] : nullptr;
  const bool setup_fork = ss != nullptr && !g_timing;
  const bool cells = setup_fork && first_order_smem<Real>(d, true) <= kMaxSmem;
  cudaStream_t sa = setup_fork ? ss : st;
  if (setup_fork) {
    CUDA_TRY(cudaEventRecord(g_side_fork[tm.dev], st));
    CUDA_TRY(cudaStreamWaitEvent(ss, g_side_fork[tm.dev], 0));
    if (w.sun) {
      tm.mark_begin(3, ss);
      launch_sun_table(w.params, d, w.sun, ss);
      launches++;
      tm.mark_end(ss);
    }
    CUDA_TRY(cudaEventRecord(g_side_sun[tm.dev], ss));
  }
  tm.mark_begin(0);
  launch_setup_rows<Real>(w.params, d, w.setup, st);
  if (cells) {
    CUDA_TRY(cudaEventRecord(g_side_rows[tm.dev], st));
    CUDA_TRY(cudaStreamWaitEvent(ss, g_side_rows[tm.dev], 0));
  }
  launch_node_maps<Real>(w.params, d, w.setup, cells ? ss : st);
  launch_view_rows<Real>(w.params, d, w.setup, st);
  launches += 4 + launch_setup_aux<Real>(w.params, d, w.dirs, w.hdirs, w.setup, sa);
  tm.mark_end();
  tm.mark_begin(1, sa);
  launch_transmittance<Real>(w.params, d, w.T, sa);
  launches++;
  tm.mark_end(sa);
  tm.mark_begin(2, sa);
  launch_surface_base<Real>(w.params, d, w.E0, sa);
  launches++;
  tm.mark_end(sa);
  if (setup_fork) {
    CUDA_TRY(cudaEventRecord(g_side_setup[tm.dev], ss));
    CUDA_TRY(cudaStreamWaitEvent(st, (cells ? g_side_sun : g_side_setup)[tm.dev], 0));
  }
  tm.mark_begin(3);
  if (w.sun && !setup_fork) {
    launch_sun_table(w.params, d, w.sun, st);
    launches++;
  }
  if (launch_first_order<Real>(w.params, d, w.setup.rowinfo, w.setup.rows, cells ? nullptr : w.setup.geom,
                               w.setup.prow, w.setup.hdvs, w.sun, w.S1R, w.M, st))
    return fail(SFSIM_ATMO_ECUDA, "first order launch configuration failed");
  launches++;
  tm.mark_end();
  if (cells) CUDA_TRY(cudaStreamWaitEvent(st, g_side_setup[tm.dev], 0));  // node maps, T, E0 and the rest
  // the transmittance and Mie-strength tables are final here: their outputs
  // (and, for host outputs, their copies) need not wait for the iterations
  tm.mark_begin(9);
  launch_output2<Real>(d.B, d.nT0, d.nT1, w.setup.remapT, w.T, oT, st);
  launch_output4<Real>(d, w.setup.remapS, w.M, oM, st);
  launches += 2;
  tm.mark_end();
  if (early_done) CUDA_TRY(cudaEventRecord(early_done, st));
  CUDA_TRY(cudaGetLastError());
  if (inter) {
    if (inter->transmittance_nodes) launch_export<Real>(d.B * d.nT(), w.T, inter->transmittance_nodes, st);
    if (inter->surface_base) launch_export<Real>(d.B * d.nE(), w.E0, inter->surface_base, st);
    if (inter->rayleigh_first) launch_export<Real>(d.B * d.n4(), w.S1R, inter->rayleigh_first, st);
    if (inter->mie_first) launch_export<Real>(d.B * d.n4(), w.M, inter->mie_first, st);
  }

  const Vec4<Real>* dS_prev = w.S1R;  // with M * phase in the first iteration
  const Vec4<Real>* M_first = w.M;
  const Vec4<Real>* dE_prev = w.E0;
  const Vec4<Real>* S_prev = w.S1R;
  const Vec4<Real>* E_prev = nullptr;  // E = constantly 0
  const size_t state4 = sizeof(Vec4<Real>) * d.B * d.n4(), state2 = sizeof(Vec4<Real>) * d.B * d.nE();
  int it0 = 0;
  if (hooks && hooks->resume) {
    // the state after iteration k into the buffers iteration k wrote
    const sfsim_atmo_iteration_state& r = *hooks->resume;
    const int k = r.iteration;
    Vec4<Real>* rdS = w.dS[(k - 1) & 1];
    Vec4<Real>* rdE = w.dE[(k - 1) & 1];
    Vec4<Real>* rS = w.Sacc[(k - 1) & 1];
    Vec4<Real>* rE = w.Eacc[(k - 1) & 1];
    CUDA_TRY(cudaMemcpyAsync(rdS, r.ray_scatter_delta, state4, cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(rdE, r.surface_delta, state2, cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(rS, r.ray_scatter_sum, state4, cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(rE, r.surface_sum, state2, cudaMemcpyHostToDevice, st));
    g_h2d_bytes += 2 * (state4 + state2);
    dS_prev = rdS;
    dE_prev = rdE;
    S_prev = rS;
    E_prev = rE;
    M_first = nullptr;
    it0 = k;
  }
  // Each iteration's surface radiance (which reads only the previous
  // iteration's dS and the first-order Mie strength) and accumulation (which
  // nothing reads before the next iteration's ray scatter) run on a side
  // stream beside point and ray scatter:
  //   side: surface radiance after everything on the build stream so far
  //         (so the dE buffer it overwrites is no longer read), then the
  //         accumulation after this iteration's ray scatter;
  //   build stream: the next point scatter after this surface radiance (its
  //         dE), the next ray scatter after this accumulation (it overwrites
  //         the dS buffer accumulation read), the outputs after the last one.
  // Entry points that create no streams (the allocation-free build) keep
  // every stage on the build stream, and so do builds with stage timing on
  // (each stage's time stays its own and the stages add up to the build) and
  // builds that export per-iteration tables or states.
  const bool fork = setup_fork && !inter && !(hooks && hooks->state);
  if (!fork) ss = st;
  for (int it = it0; it < d.iterations; it++) {
    tm.iteration = it + 1;
    Vec4<Real>* dE_new = w.dE[it & 1];
    Vec4<Real>* dS_new = w.dS[it & 1];
    Vec4<Real>* E_new = w.Eacc[it & 1];
    Vec4<Real>* S_new = w.Sacc[it & 1];
    if (fork) {
      if (it > it0) CUDA_TRY(cudaStreamWaitEvent(st, g_side_sr[tm.dev], 0));  // dE of the last iteration
      CUDA_TRY(cudaEventRecord(g_side_fork[tm.dev], st));
      CUDA_TRY(cudaStreamWaitEvent(ss, g_side_fork[tm.dev], 0));
    }
    tm.mark_begin(6, ss);
    launch_surface_radiance<Real>(w.params, d, w.setup.erow, w.setup.hdir, dS_prev, M_first, dE_new, ss);
    launches++;
    tm.mark_end(ss);
    if (fork) CUDA_TRY(cudaEventRecord(g_side_sr[tm.dev], ss));
    tm.mark_begin(5);
    if (launch_point_scatter<Real>(w.params, d, w.setup.rowinfo, w.setup.pdirs, w.setup.dimage, w.setup.pcount,
                                   w.setup.prow,
                                   w.setup.geom, dS_prev, M_first, dE_prev, w.hrows, w.J, st))
      return fail(SFSIM_ATMO_ECUDA, "point scatter launch configuration failed");
    launches += 2;
    tm.mark_end();
    if (jsum) {
      launch_add_to_sum<Real>(d.n4(), d.B, w.J, jsum, it == 0, st);
      launches++;
    }

    if (fork && it > it0) CUDA_TRY(cudaStreamWaitEvent(st, g_side_acc[tm.dev], 0));  // its dS buffer read
    tm.mark_begin(7);
    if (launch_ray_scatter<Real>(w.params, d, w.setup.rowinfo, w.setup.rows, w.setup.geom, w.setup.remapS, w.J,
                                 dS_new, st))
      return fail(SFSIM_ATMO_ECUDA, "ray scatter launch configuration failed");
    launches++;
    tm.mark_end();
    if (fork) {
      CUDA_TRY(cudaEventRecord(g_side_rs[tm.dev], st));
      CUDA_TRY(cudaStreamWaitEvent(ss, g_side_rs[tm.dev], 0));
    }
    tm.mark_begin(8, ss);
    launch_accumulate2<Real>(d.B, d.nE0, d.nE1, w.setup.remapE, E_prev, dE_new, E_new, ss);
    launch_accumulate4<Real>(d, w.setup.remapS, S_prev, dS_new, S_new, ss);
    launches += 2;
    tm.mark_end(ss);
    if (fork) CUDA_TRY(cudaEventRecord(g_side_acc[tm.dev], ss));
    CUDA_TRY(cudaGetLastError());
    if (inter) {
      if (inter->point_scatter)
        launch_export_planar<Real>(d.n4(), d.B, w.J, inter->point_scatter + (size_t)3 * d.B * d.n4() * it, st);
      if (inter->surface_delta)
        launch_export<Real>(d.B * d.nE(), dE_new, inter->surface_delta + (size_t)3 * d.B * d.nE() * it, st);
      if (inter->ray_scatter_delta)
        launch_export<Real>(d.B * d.n4(), dS_new, inter->ray_scatter_delta + (size_t)3 * d.B * d.n4() * it, st);
    }
    dS_prev = dS_new;
    M_first = nullptr;
    dE_prev = dE_new;
    S_prev = S_new;
    E_prev = E_new;
    if (hooks && hooks->state) {
      sfsim_atmo_iteration_state& o = *hooks->state;
      CUDA_TRY(cudaMemcpyAsync(o.ray_scatter_delta, dS_new, state4, cudaMemcpyDeviceToHost, st));
      CUDA_TRY(cudaMemcpyAsync(o.surface_delta, dE_new, state2, cudaMemcpyDeviceToHost, st));
      CUDA_TRY(cudaMemcpyAsync(o.ray_scatter_sum, S_new, state4, cudaMemcpyDeviceToHost, st));
      CUDA_TRY(cudaMemcpyAsync(o.surface_sum, E_new, state2, cudaMemcpyDeviceToHost, st));
      CUDA_TRY(cudaStreamSynchronize(st));
      g_d2h_bytes += 2 * (state4 + state2);
      o.iteration = it + 1;
      if (hooks->on_iteration && hooks->on_iteration(&o, hooks->user))
        return fail(SFSIM_ATMO_ESTOPPED, "the iteration callback stopped the build after iteration " + std::to_string(it + 1));
    }
  }
  tm.iteration = 0;
  if (fork && d.iterations > it0) CUDA_TRY(cudaStreamWaitEvent(st, g_side_acc[tm.dev], 0));  // the final S and E
  tm.mark_begin(9);
  launch_output2<Real>(d.B, d.nE0, d.nE1, w.setup.remapE, E_prev, oE, st);
  launch_output4<Real>(d, w.setup.remapS, S_prev, oS, st);
  launches += 2;
  tm.mark_end();
  CUDA_TRY(cudaGetLastError());
  g_launches = launches;
  return 0;
}

void collect_timings(Timer& tm) {
  for (int s = 0; s < kStages; s++) g_stage_ms[s] = 0;
  g_have_timings = 0;
  if (!g_timing) return;
  for (int p = 0; p + 1 < tm.n; p += 2) {
    float ms = 0;
    if (cudaEventSynchronize(g_events[tm.dev][p + 1]) == cudaSuccess &&
        cudaEventElapsedTime(&ms, g_events[tm.dev][p], g_events[tm.dev][p + 1]) == cudaSuccess)
      g_stage_ms[tm.stage_of[p / 2]] += ms;
  }
  g_have_timings = kStages;
}

// Shared driver of all build entry points.  `host_out`: the four output
// pointers are host memory (copied back and synchronised); otherwise device
// memory on `user_stream`.
template <class Real>
int build_impl(const sfsim_atmo_config* cfgs, int B, float* T, float* E, float* S, float* M, bool host_out,
               cudaStream_t user_stream, const sfsim_atmo_intermediates* inter, const IterationHooks* hooks = nullptr) {
  int dev = 0;
  int rc = current_device(&dev);
  if (rc) return rc;
  if ((rc = ensure_stream(dev))) return rc;
  BuildDims d = make_dims(cfgs[0], B);
  if ((rc = check_smem<Real>(d))) return rc;
  std::vector<AtmoParams> hp(B);
  for (int b = 0; b < B; b++)
    if ((rc = make_params(cfgs[b], hp[b]))) return rc;
  std::vector<DirLocal> dirs, hdirs;
  sphere_directions(cfgs[0].sphere_steps >> 1, cfgs[0].sphere_steps, M_PI, dirs);
  sphere_directions(cfgs[0].ray_steps >> 2, cfgs[0].ray_steps, M_PI / 2, hdirs);

  Work<Real> w;
  size_t bytes = carve<Real>(w, nullptr, d, host_out);
  if ((rc = ensure_arena(dev, bytes))) return rc;
  carve<Real>(w, (char*)g_arena[dev].base, d, host_out);

  cudaStream_t st = host_out ? g_stream[dev] : user_stream;
  g_h2d_bytes = sizeof(AtmoParams) * B + sizeof(DirLocal) * (dirs.size() + hdirs.size());
  g_d2h_bytes = host_out ? sizeof(float) * 3 * B * (d.nT() + d.nE() + 2 * d.n4()) : 0;
  CUDA_TRY(cudaMemcpyAsync(w.params, hp.data(), sizeof(AtmoParams) * B, cudaMemcpyHostToDevice, st));
  if (!dirs.empty()) {
    CUDA_TRY(cudaMemcpyAsync(w.dirs, dirs.data(), sizeof(DirLocal) * dirs.size(), cudaMemcpyHostToDevice, st));
  }
  if (!hdirs.empty())
    CUDA_TRY(cudaMemcpyAsync(w.hdirs, hdirs.data(), sizeof(DirLocal) * hdirs.size(), cudaMemcpyHostToDevice, st));

  // debug intermediates go through device staging buffers
  sfsim_atmo_intermediates dinter;
  std::vector<std::pair<float*, float*>> copies;  // (device, host)
  std::vector<size_t> copy_bytes;
  float* staging = nullptr;
  if (inter) {
    const size_t n4 = 3 * (size_t)B * d.n4(), nE = 3 * (size_t)B * d.nE(), nT = 3 * (size_t)B * d.nT();
    const size_t it = d.iterations;
    size_t total = nT + nE + 2 * n4 + it * (2 * n4 + nE);
    CUDA_TRY(cudaMalloc(&staging, total * sizeof(float)));
    float* p = staging;
    auto take = [&](float* host, size_t n) -> float* {
      if (!host) return nullptr;
      float* dptr = p;
      p += n;
      copies.push_back({dptr, host});
      copy_bytes.push_back(n * sizeof(float));
      return dptr;
    };
    dinter.transmittance_nodes = take(inter->transmittance_nodes, nT);
    dinter.surface_base = take(inter->surface_base, nE);
    dinter.rayleigh_first = take(inter->rayleigh_first, n4);
    dinter.mie_first = take(inter->mie_first, n4);
    dinter.point_scatter = take(inter->point_scatter, it * n4);
    dinter.surface_delta = take(inter->surface_delta, it * nE);
    dinter.ray_scatter_delta = take(inter->ray_scatter_delta, it * n4);
  }

  Timer tm;
  tm.dev = dev;
  tm.st = st;
  float *dT = host_out ? w.oT : T, *dE = host_out ? w.oE : E, *dS = host_out ? w.oS : S, *dM = host_out ? w.oM : M;
  rc = run_build<Real>(w, d, dT, dE, dS, dM, st, tm, inter ? &dinter : nullptr, nullptr,
                       host_out ? g_early_done[dev] : nullptr, hooks);
  if (rc) {
    if (staging) cudaFree(staging);
    return rc;
  }
  if (host_out) {
    // T and M copy on the second stream once their outputs are written (the
    // whole build is queued first, so a copy into pageable memory, which
    // blocks the host, cannot hold back the launches)
    cudaStream_t cs = g_copy_stream[dev];
    CUDA_TRY(cudaStreamWaitEvent(cs, g_early_done[dev], 0));
    CUDA_TRY(cudaMemcpyAsync(T, w.oT, sizeof(float) * 3 * B * d.nT(), cudaMemcpyDeviceToHost, cs));
    CUDA_TRY(cudaMemcpyAsync(M, w.oM, sizeof(float) * 3 * B * d.n4(), cudaMemcpyDeviceToHost, cs));
    CUDA_TRY(cudaMemcpyAsync(E, w.oE, sizeof(float) * 3 * B * d.nE(), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaMemcpyAsync(S, w.oS, sizeof(float) * 3 * B * d.n4(), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(cs));
  }
  for (size_t i = 0; i < copies.size(); i++) {
    CUDA_TRY(cudaMemcpyAsync(copies[i].second, copies[i].first, copy_bytes[i], cudaMemcpyDeviceToHost, st));
    g_d2h_bytes += copy_bytes[i];
  }
  if (host_out || inter) CUDA_TRY(cudaStreamSynchronize(st));
  if (staging) CUDA_TRY(cudaFree(staging));
  collect_timings(tm);
  return 0;
}

int dispatch(const sfsim_atmo_config* cfgs, int B, float* T, float* E, float* S, float* M, bool host_out,
             cudaStream_t st, const sfsim_atmo_intermediates* inter) {
  if (!cfgs) return fail(SFSIM_ATMO_ENULL, "config is NULL");
  if (B < 1) return fail(SFSIM_ATMO_EINVAL, "batch size must be at least 1");
  if (B > 65535) return fail(SFSIM_ATMO_ETOOBIG, "a batch holds at most 65535 atmospheres (one grid row each)");
  if (!T || !E || !S || !M) return fail(SFSIM_ATMO_ENULL, "an output pointer is NULL");
  for (int b = 0; b < B; b++) {
    int rc = validate(&cfgs[b]);
    if (rc) return rc;
    if (!same_layout(cfgs[0], cfgs[b]))
      return fail(SFSIM_ATMO_EINVAL, "batched configs must share shapes, steps, iterations, precision and flags");
  }
  std::lock_guard<std::mutex> lock(g_mutex);
  if (cfgs[0].precision == SFSIM_ATMO_FP64) return build_impl<double>(cfgs, B, T, E, S, M, host_out, st, inter);
  return build_impl<float>(cfgs, B, T, E, S, M, host_out, st, inter);
}

template <class Real>
int census_impl(const sfsim_atmo_config& cfg, unsigned long long* out, int n) {
  int dev = 0;
  int rc = current_device(&dev);
  if (rc) return rc;
  if ((rc = ensure_stream(dev))) return rc;
  BuildDims d = make_dims(cfg, 1);
  AtmoParams hp;
  if ((rc = make_params(cfg, hp))) return rc;
  std::vector<DirLocal> dirs;
  sphere_directions(cfg.sphere_steps >> 1, cfg.sphere_steps, M_PI, dirs);
  Work<Real> w;
  size_t bytes = carve<Real>(w, nullptr, d, false, false);
  if ((rc = ensure_arena(dev, bytes + 256))) return rc;
  carve<Real>(w, (char*)g_arena[dev].base, d, false, false);
  unsigned long long* dcount = reinterpret_cast<unsigned long long*>((char*)g_arena[dev].base + bytes);
  cudaStream_t st = g_stream[dev];
  CUDA_TRY(cudaMemcpyAsync(w.params, &hp, sizeof(AtmoParams), cudaMemcpyHostToDevice, st));
  if (!dirs.empty()) {
    CUDA_TRY(cudaMemcpyAsync(w.dirs, dirs.data(), sizeof(DirLocal) * dirs.size(), cudaMemcpyHostToDevice, st));
  }
  CUDA_TRY(cudaMemsetAsync(dcount, 0, 2 * sizeof(unsigned long long), st));
  launch_setup<Real>(w.params, d, w.dirs, w.hdirs, w.setup, st);
  launch_first_order_census<Real>(w.params, d, w.setup.rowinfo, w.setup.rows, w.setup.geom, dcount, st);
  CUDA_TRY(cudaGetLastError());
  unsigned long long cnt[2] = {0, 0};
  CUDA_TRY(cudaMemcpyAsync(cnt, dcount, sizeof(cnt), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  const unsigned long long lit = cnt[0], climb = cnt[1];
  // ground directions of the point-scatter sphere per height
  std::vector<SphereDir<Real>> sd((size_t)d.n0 * (d.P + 1));
  CUDA_TRY(cudaMemcpy(sd.data(), w.setup.sdirs, sizeof(SphereDir<Real>) * sd.size(), cudaMemcpyDeviceToHost));
  unsigned long long ground = 0, flat = 0;
  for (int i = 0; i < d.n0; i++)
    for (int k = 0; k < d.P; k++) {
      const SphereDir<Real>& e = sd[(size_t)i * d.P + k];
      ground += e.surface ? 1 : 0;
      flat += (e.surface && e.sE0 == Real(0)) ? 1 : 0;
    }
  const unsigned long long S = (unsigned long long)d.S, it = (unsigned long long)d.iterations;
  const unsigned long long per_height = (unsigned long long)d.n1 * d.n2 * d.n3;
  const unsigned long long vals[10] = {lit,
                                       lit * S,
                                       (unsigned long long)d.rows() * S * S,
                                       (unsigned long long)d.n4() * d.P * it,
                                       (unsigned long long)d.n4() * S * it,
                                       (unsigned long long)d.nE() * d.Ph * it,
                                       climb,
                                       ground * per_height * it,
                                       it > 0 ? (unsigned long long)d.n4() * d.P : 0ull,
                                       flat * per_height * it};
  int m = n < 10 ? n : 10;
  for (int i = 0; i < m; i++) out[i] = vals[i];
  return m;
}

}  // namespace

extern "C" {

int sfsim_atmo_census(const sfsim_atmo_config* cfg, unsigned long long* counts, int n) {
  int rc = validate(cfg);
  if (rc) return rc;
  if (!counts) return fail(SFSIM_ATMO_ENULL, "counts is NULL");
  std::lock_guard<std::mutex> lock(g_mutex);
  if (cfg->precision == SFSIM_ATMO_FP64) return census_impl<double>(*cfg, counts, n);
  return census_impl<float>(*cfg, counts, n);
}

int sfsim_atmo_sfu_peak(double* ex2_per_second) {
  if (!ex2_per_second) return fail(SFSIM_ATMO_ENULL, "ex2_per_second is NULL");
  std::lock_guard<std::mutex> lock(g_mutex);
  int dev = 0;
  int rc = current_device(&dev);
  if (rc) return rc;
  if ((rc = ensure_stream(dev))) return rc;
  int sms = 0;
  CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int blocks = sms * 8, threads = 256, iters = 4096;
  float* sink = nullptr;
  CUDA_TRY(cudaMalloc(&sink, sizeof(float) * blocks));
  cudaStream_t st = g_stream[dev];
  cudaEvent_t e0, e1;
  CUDA_TRY(cudaEventCreate(&e0));
  CUDA_TRY(cudaEventCreate(&e1));
  double best = 0;
  for (int rep = 0; rep < 5; rep++) {
    CUDA_TRY(cudaEventRecord(e0, st));
    launch_sfu_probe(blocks, threads, iters, sink, st);
    CUDA_TRY(cudaEventRecord(e1, st));
    CUDA_TRY(cudaEventSynchronize(e1));
    float ms = 0;
    CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
    const double ops = (double)blocks * threads * iters * 8;
    if (rep > 0 && ms > 0) best = std::fmax(best, ops / (ms * 1e-3));
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  CUDA_TRY(cudaFree(sink));
  *ex2_per_second = best;
  return 0;
}

int sfsim_atmo_smem_peak(double* bytes_per_second) {
  if (!bytes_per_second) return fail(SFSIM_ATMO_ENULL, "bytes_per_second is NULL");
  std::lock_guard<std::mutex> lock(g_mutex);
  int dev = 0;
  int rc = current_device(&dev);
  if (rc) return rc;
  if ((rc = ensure_stream(dev))) return rc;
  int sms = 0;
  CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int blocks = sms, iters = 4096;
  float* sink = nullptr;
  CUDA_TRY(cudaMalloc(&sink, sizeof(float) * blocks));
  cudaStream_t st = g_stream[dev];
  cudaEvent_t e0, e1;
  CUDA_TRY(cudaEventCreate(&e0));
  CUDA_TRY(cudaEventCreate(&e1));
  double best = 0;
  for (int rep = 0; rep < 5 && !rc; rep++) {
    CUDA_TRY(cudaEventRecord(e0, st));
    if (launch_smem_probe(blocks, iters, sink, st)) rc = fail(SFSIM_ATMO_ECUDA, "shared-memory probe launch failed");
    CUDA_TRY(cudaEventRecord(e1, st));
    CUDA_TRY(cudaEventSynchronize(e1));
    float ms = 0;
    CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
    const double bytes = (double)blocks * 1024 * iters * 8 * 16;
    if (rep > 0 && ms > 0) best = std::fmax(best, bytes / (ms * 1e-3));
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(sink);
  if (rc) return rc;
  *bytes_per_second = best;
  return 0;
}


void sfsim_atmo_default_config(sfsim_atmo_config* c) {
  if (!c) return;
  memset(c, 0, sizeof(*c));
  c->radius = 6378000.0;
  c->height = 35000.0;
  for (int i = 0; i < 3; i++) {
    c->brightness[i] = 0.3;
    c->intensity[i] = 1.0;
    c->mie.scatter_base[i] = 2e-5;
  }
  c->mie.scatter_scale = 1200.0;
  c->mie.scatter_quotient = 0.9;
  c->mie.scatter_g = 0.76;
  c->rayleigh.scatter_base[0] = 5.8e-6;
  c->rayleigh.scatter_base[1] = 13.5e-6;
  c->rayleigh.scatter_base[2] = 33.1e-6;
  c->rayleigh.scatter_scale = 8000.0;
  c->rayleigh.scatter_quotient = 1.0;
  c->rayleigh.scatter_g = 0.0;
  c->transmittance_shape[0] = 64;
  c->transmittance_shape[1] = 255;
  c->surface_radiance_shape[0] = 16;
  c->surface_radiance_shape[1] = 63;
  c->ray_scatter_shape[0] = 32;
  c->ray_scatter_shape[1] = 127;
  c->ray_scatter_shape[2] = 32;
  c->ray_scatter_shape[3] = 8;
  c->ray_steps = 100;
  c->sphere_steps = 15;
  c->iterations = 5;
  c->precision = SFSIM_ATMO_FP32;
  c->flags = 0;
}

int sfsim_atmo_validate(const sfsim_atmo_config* cfg) { return validate(cfg); }

int sfsim_atmo_table_sizes(const sfsim_atmo_config* c, size_t* nT, size_t* nE, size_t* nS, size_t* nM) {
  int rc = validate(c);
  if (rc) return rc;
  size_t n4 = 3;
  for (int i = 0; i < 4; i++) n4 *= (size_t)c->ray_scatter_shape[i];
  if (nT) *nT = 3 * (size_t)c->transmittance_shape[0] * c->transmittance_shape[1];
  if (nE) *nE = 3 * (size_t)c->surface_radiance_shape[0] * c->surface_radiance_shape[1];
  if (nS) *nS = n4;
  if (nM) *nM = n4;
  return 0;
}

int sfsim_atmo_build(const sfsim_atmo_config* cfg, float* T, float* E, float* S, float* M) {
  return dispatch(cfg, 1, T, E, S, M, true, nullptr, nullptr);
}

int sfsim_atmo_build_device(const sfsim_atmo_config* cfg, float* T, float* E, float* S, float* M, void* stream) {
  return dispatch(cfg, 1, T, E, S, M, false, (cudaStream_t)stream, nullptr);
}

int sfsim_atmo_build_batch(const sfsim_atmo_config* cfgs, int n, float* T, float* E, float* S, float* M) {
  return dispatch(cfgs, n, T, E, S, M, true, nullptr, nullptr);
}

int sfsim_atmo_build_debug(const sfsim_atmo_config* cfg, float* T, float* E, float* S, float* M,
                           const sfsim_atmo_intermediates* inter) {
  return dispatch(cfg, 1, T, E, S, M, true, nullptr, inter);
}

int sfsim_atmo_iteration_state_bytes(const sfsim_atmo_config* cfg, size_t* s_bytes, size_t* e_bytes) {
  if (!cfg) return fail(SFSIM_ATMO_ENULL, "config is NULL");
  int rc = validate(cfg);
  if (rc) return rc;
  const size_t rec = 4 * (cfg->precision == SFSIM_ATMO_FP64 ? sizeof(double) : sizeof(float));
  const int* s = cfg->ray_scatter_shape;
  if (s_bytes) *s_bytes = rec * (size_t)s[0] * s[1] * s[2] * s[3];
  if (e_bytes) *e_bytes = rec * (size_t)cfg->surface_radiance_shape[0] * cfg->surface_radiance_shape[1];
  return 0;
}

int sfsim_atmo_build_resumable(const sfsim_atmo_config* cfg, const sfsim_atmo_iteration_state* resume,
                            sfsim_atmo_iteration_state* state, sfsim_atmo_iteration_fn on_iteration, void* user, float* T,
                            float* E, float* S, float* M) {
  if (!cfg) return fail(SFSIM_ATMO_ENULL, "config is NULL");
  if (!T || !E || !S || !M) return fail(SFSIM_ATMO_ENULL, "an output pointer is NULL");
  int rc = validate(cfg);
  if (rc) return rc;
  auto complete = [](const sfsim_atmo_iteration_state* o) {
    return o->ray_scatter_delta && o->surface_delta && o->ray_scatter_sum && o->surface_sum;
  };
  if (resume) {
    if (!complete(resume)) return fail(SFSIM_ATMO_ENULL, "a table of the resume state is NULL");
    if (resume->iteration < 1 || resume->iteration > cfg->iterations)
      return fail(SFSIM_ATMO_EINVAL, "the resume iteration must be in [1, iterations]");
  }
  if (state && !complete(state)) return fail(SFSIM_ATMO_ENULL, "a table of the state buffers is NULL");
  const IterationHooks hooks{resume, state, on_iteration, user};
  std::lock_guard<std::mutex> lock(g_mutex);
  if (cfg->precision == SFSIM_ATMO_FP64) return build_impl<double>(cfg, 1, T, E, S, M, true, nullptr, nullptr, &hooks);
  return build_impl<float>(cfg, 1, T, E, S, M, true, nullptr, nullptr, &hooks);
}

int sfsim_atmo_set_timing(int enabled) {
  g_timing = enabled != 0;
  return 0;
}

int sfsim_atmo_last_timings(double* ms, int n) {
  if (!ms) return fail(SFSIM_ATMO_ENULL, "ms is NULL");
  int m = n < g_have_timings ? n : g_have_timings;
  for (int i = 0; i < m; i++) ms[i] = g_stage_ms[i];
  return m;
}

int sfsim_atmo_last_launch_count(void) { return g_launches; }

int sfsim_atmo_last_transfer_bytes(unsigned long long* h2d, unsigned long long* d2h) {
  if (h2d) *h2d = g_h2d_bytes;
  if (d2h) *d2h = g_d2h_bytes;
  return 0;
}

int sfsim_atmo_release(void) {
  std::lock_guard<std::mutex> lock(g_mutex);
  int dev = 0;
  int rc = current_device(&dev);
  if (rc) return rc;
  Arena& a = g_arena[dev];
  if (a.base) {
    CUDA_TRY(cudaDeviceSynchronize());
    CUDA_TRY(cudaFree(a.base));
  }
  a.base = nullptr;
  a.size = 0;
  return 0;
}

const char* sfsim_atmo_strerror(int code) {
  switch (code) {
    case SFSIM_ATMO_OK: return "success";
    case SFSIM_ATMO_EINVAL: return "invalid configuration value";
    case SFSIM_ATMO_ENOMEM: return "out of memory";
    case SFSIM_ATMO_ECUDA: return "CUDA runtime error";
    case SFSIM_ATMO_ENODEV: return "no CUDA device";
    case SFSIM_ATMO_ESHAPE: return "unsupported table shape";
    case SFSIM_ATMO_ENULL: return "NULL pointer argument";
    case SFSIM_ATMO_ETOOBIG: return "size exceeds a fixed capacity";
    case SFSIM_ATMO_ENUMERIC: return "result contains NaN or Inf";
    case SFSIM_ATMO_ESTOPPED: return "stopped by the iteration callback";
    default: return "unknown error";
  }
}

const char* sfsim_atmo_last_error(void) { return g_last_error.c_str(); }

const char* sfsim_atmo_version(void) { return "sfsim-atmo-gb300 0.1.0 (sm_103a)"; }

}  // extern "C"

// ---------------------------------------------------------------------------
// Contexts: a built atmosphere kept on the device for queries.
// ---------------------------------------------------------------------------

struct Surrogate;

struct sfsim_atmo_context {
  int dev;
  sfsim_atmo_config cfg;
  BuildDims dims;
  void* mem;
  AtmoParams* params;
  float *T, *E, *S, *M;
  Vec4<float>* jsum;  // point scatter summed over the iterations, NULL without iterations
  void* geom;         // per-node light directions (CellGeom<Real>)
  Surrogate* sur;     // trained surrogate or NULL
};

namespace {

template <class Real>
int context_build(sfsim_atmo_context* c) {
  int rc = 0;
  const sfsim_atmo_config& cfg = c->cfg;
  BuildDims d = make_dims(cfg, 1);
  if ((rc = check_smem<Real>(d))) return rc;
  AtmoParams hp;
  if ((rc = make_params(cfg, hp))) return rc;
  std::vector<DirLocal> dirs, hdirs;
  sphere_directions(cfg.sphere_steps >> 1, cfg.sphere_steps, M_PI, dirs);
  sphere_directions(cfg.ray_steps >> 2, cfg.ray_steps, M_PI / 2, hdirs);
  Work<Real> w;
  const size_t wbytes = carve<Real>(w, nullptr, d, true);
  const size_t total = wbytes + sizeof(Vec4<float>) * (size_t)d.n4() + 256;
  cudaError_t e = cudaMalloc(&c->mem, total);
  if (e != cudaSuccess) {
    cudaGetLastError();
    c->mem = nullptr;
    return fail(SFSIM_ATMO_ENOMEM, std::string("cudaMalloc of the context failed: ") + cudaGetErrorString(e));
  }
  carve<Real>(w, (char*)c->mem, d, true);
  c->jsum = cfg.iterations > 0 ? reinterpret_cast<Vec4<float>*>((char*)c->mem + ((wbytes + 255) & ~size_t(255)))
                               : nullptr;
  cudaStream_t st = g_stream[c->dev];
  CUDA_TRY(cudaMemcpyAsync(w.params, &hp, sizeof(AtmoParams), cudaMemcpyHostToDevice, st));
  if (!dirs.empty()) {
    CUDA_TRY(cudaMemcpyAsync(w.dirs, dirs.data(), sizeof(DirLocal) * dirs.size(), cudaMemcpyHostToDevice, st));
  }
  if (!hdirs.empty())
    CUDA_TRY(cudaMemcpyAsync(w.hdirs, hdirs.data(), sizeof(DirLocal) * hdirs.size(), cudaMemcpyHostToDevice, st));
  Timer tm;
  tm.dev = c->dev;
  tm.st = st;
  tm.n = 512;  // no stage timings for context builds
  if ((rc = run_build<Real>(w, d, w.oT, w.oE, w.oS, w.oM, st, tm, nullptr, c->jsum))) return rc;
  CUDA_TRY(cudaStreamSynchronize(st));
  c->dims = d;
  c->params = w.params;
  c->geom = w.setup.geom;
  c->T = w.oT;
  c->E = w.oE;
  c->S = w.oS;
  c->M = w.oM;
  return 0;
}

}  // namespace

// ---------------------------------------------------------------------------
// Surrogate of the rendered in-scatter: Fourier features of the four table
// coordinates -> 4 x 256 SiLU -> 3 log-space corrections to the table lookup
// and the log of their expected squared error, trained on the GPU against the
// direct quadrature.
// ---------------------------------------------------------------------------

constexpr float kLogEps = 1e-7f;     // corrections are log(value + kLogEps) - log(table + kLogEps)
constexpr float kVarWeight = 0.01f;  // weight of the variance output's gradient in the shared layers
constexpr long long kQueryChunk = 1 << 22;  // surrogate queries per lookup + inference pass

// parameter offsets (floats) in the concatenated FP32 vector; a conditioned
// network appends U [kMlpHidden][cond], the first layer's weights of the
// atmosphere inputs
struct MlpLayout {
  long long W[5], b[5], U, total;
  int in[5], out[5], cond;
  explicit MlpLayout(int cond_inputs = 0) {
    const int ins[5] = {kMlpIn, kMlpHidden, kMlpHidden, kMlpHidden, kMlpHidden};
    const int outs[5] = {kMlpHidden, kMlpHidden, kMlpHidden, kMlpHidden, kMlpOut};
    long long o = 0;
    for (int l = 0; l < 5; l++) {
      in[l] = ins[l];
      out[l] = outs[l];
      W[l] = o;
      o += (long long)outs[l] * ins[l];
      b[l] = o;
      o += outs[l];
    }
    cond = cond_inputs;
    U = o;
    total = o + (long long)kMlpHidden * cond;
  }
};

struct Surrogate {
  MlpLayout lay;
  explicit Surrogate(int cond) : lay(cond) {}
  long long batch = 0;             // rows of the activation buffers
  float *w = nullptr, *g = nullptr, *m = nullptr, *v = nullptr;  // master weights, grads, Adam moments
  __nv_bfloat16 *wb[4] = {}, *wbt[4] = {};  // BF16 W_l [out][in] and W_l^T [in][out]
  // activations of one batch
  float *coords = nullptr, *target = nullptr, *out = nullptr, *dout = nullptr, *loss = nullptr;
  __nv_bfloat16 *F = nullptr, *FT = nullptr, *H[4] = {}, *HT[4] = {}, *dZ[4] = {}, *dZT[4] = {};
  float* dsilu[4] = {};
  unsigned char* packed = nullptr;  // weight chunks of the fused inference kernel
  float* qbuf = nullptr;            // coordinates and table values of one chunk of queries
  long long qcap = 0;               // queries qbuf holds
  int* error = nullptr;
  int trained_steps = 0;
  // conditioned network: the groups' atmosphere inputs G [groups][kCondInputs],
  // their first-layer row biases U g [groups][kMlpHidden], each row's group,
  // and for queries the first-layer bias b1 + U g of the queried atmosphere
  int groups = 0;
  float *G = nullptr, *cbias = nullptr, *qbias = nullptr, *qG = nullptr;
  int* group = nullptr;
  std::vector<void*> allocs;
  float* alloc_f(size_t n) {
    void* p = nullptr;
    if (cudaMalloc(&p, n * sizeof(float)) != cudaSuccess) return nullptr;
    allocs.push_back(p);
    return (float*)p;
  }
  __nv_bfloat16* alloc_h(size_t n) {
    void* p = nullptr;
    if (cudaMalloc(&p, n * sizeof(__nv_bfloat16)) != cudaSuccess) return nullptr;
    allocs.push_back(p);
    return (__nv_bfloat16*)p;
  }
  void free_all() {
    for (void* p : allocs) cudaFree(p);
    allocs.clear();
    if (qbuf) cudaFree(qbuf);
    qbuf = nullptr;
    qcap = 0;
  }
};

void surrogate_free(sfsim_atmo_context* c) {
  if (c->sur) {
    c->sur->free_all();
    delete c->sur;
    c->sur = nullptr;
  }
}

// Xavier-uniform initial weights (seeded LCG on the host), zero biases.
void init_weights(const MlpLayout& lay, unsigned long long seed, std::vector<float>& h) {
  h.assign(lay.total, 0.0f);
  unsigned long long s = seed * 6364136223846793005ull + 1442695040888963407ull;
  for (int l = 0; l < 5; l++) {
    const double a = std::sqrt(6.0 / (lay.in[l] + lay.out[l]));
    for (long long t = 0; t < (long long)lay.in[l] * lay.out[l]; t++) {
      s = s * 6364136223846793005ull + 1442695040888963407ull;
      const double u = (double)(s >> 11) * (1.0 / 9007199254740992.0);
      h[lay.W[l] + t] = (float)((2.0 * u - 1.0) * a);
    }
  }
}

int surrogate_alloc(Surrogate*& sur, int cond, long long batch, unsigned long long seed) {
  if (!sur) {
    sur = new Surrogate(cond);
    Surrogate& S = *sur;
    const long long P = S.lay.total;
    S.w = S.alloc_f(P);
    S.g = S.alloc_f(P);
    S.m = S.alloc_f(P);
    S.v = S.alloc_f(P);
    S.loss = S.alloc_f(1);
    void* e = nullptr;
    if (cudaMalloc(&e, sizeof(int)) != cudaSuccess) return fail(SFSIM_ATMO_ENOMEM, "surrogate allocation failed");
    S.allocs.push_back(e);
    S.error = (int*)e;
    for (int l = 0; l < 4; l++) {
      S.wb[l] = S.alloc_h((size_t)S.lay.in[l] * S.lay.out[l]);
      S.wbt[l] = S.alloc_h((size_t)S.lay.in[l] * S.lay.out[l]);
    }
    S.packed = reinterpret_cast<unsigned char*>(S.alloc_h(infer_packed_bytes() / 2));
    if (!S.w || !S.g || !S.m || !S.v || !S.loss || !S.wb[3] || !S.wbt[3] || !S.packed)
      return fail(SFSIM_ATMO_ENOMEM, "surrogate allocation failed");
    if (cond) {
      S.G = S.alloc_f((size_t)kMaxCondGroups * kCondInputs);
      S.cbias = S.alloc_f((size_t)kMaxCondGroups * kMlpHidden);
      S.qbias = S.alloc_f(kMlpHidden);
      S.qG = S.alloc_f(kCondInputs);
      if (!S.G || !S.cbias || !S.qbias || !S.qG) return fail(SFSIM_ATMO_ENOMEM, "surrogate allocation failed");
    }
    std::vector<float> h;
    init_weights(S.lay, seed, h);
    CUDA_TRY(cudaMemcpy(S.w, h.data(), sizeof(float) * P, cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemset(S.m, 0, sizeof(float) * P));
    CUDA_TRY(cudaMemset(S.v, 0, sizeof(float) * P));
    CUDA_TRY(cudaMemset(S.error, 0, sizeof(int)));
    for (int l = 0; l < 4; l++)
      launch_to_bf16((long long)S.lay.in[l] * S.lay.out[l], S.w + S.lay.W[l], S.lay.out[l], S.lay.in[l], S.wb[l],
                     S.wbt[l], 0);
    CUDA_TRY(cudaGetLastError());
  }
  Surrogate& S = *sur;
  if (S.batch < batch) {
    // activation buffers for `batch` rows
    auto drop = [&](void* p) {
      if (!p) return;
      for (size_t i = 0; i < S.allocs.size(); i++)
        if (S.allocs[i] == p) {
          cudaFree(p);
          S.allocs.erase(S.allocs.begin() + i);
          return;
        }
    };
    drop(S.coords); drop(S.target); drop(S.out); drop(S.dout); drop(S.F); drop(S.FT); drop(S.group);
    for (int l = 0; l < 4; l++) {
      drop(S.H[l]); drop(S.HT[l]); drop(S.dZ[l]); drop(S.dZT[l]); drop(S.dsilu[l]);
    }
    S.coords = S.alloc_f(kMlpCoords * batch);
    S.target = S.alloc_f(3 * batch);
    S.out = S.alloc_f(kMlpOut * batch);
    S.dout = S.alloc_f(kMlpOut * batch);
    S.F = S.alloc_h(kMlpIn * batch);
    S.FT = S.alloc_h(kMlpIn * batch);
    S.group = nullptr;
    if (S.lay.cond) {
      void* p = nullptr;
      if (cudaMalloc(&p, sizeof(int) * (size_t)batch) == cudaSuccess) {
        S.allocs.push_back(p);
        S.group = (int*)p;
      }
    }
    bool okay = S.coords && S.target && S.out && S.dout && S.F && S.FT && (!S.lay.cond || S.group);
    for (int l = 0; l < 4 && okay; l++) {
      S.H[l] = S.alloc_h(kMlpHidden * batch);
      S.HT[l] = S.alloc_h(kMlpHidden * batch);
      S.dZ[l] = S.alloc_h(kMlpHidden * batch);
      S.dZT[l] = S.alloc_h(kMlpHidden * batch);
      S.dsilu[l] = S.alloc_f(kMlpHidden * batch);
      okay = S.H[l] && S.HT[l] && S.dZ[l] && S.dZT[l] && S.dsilu[l];
    }
    if (!okay) {
      S.batch = 0;
      return fail(SFSIM_ATMO_ENOMEM, "surrogate activation allocation failed");
    }
    S.batch = batch;
  }
  return 0;
}

// Forward pass over n rows of S.coords (n <= S.batch); `train` keeps what the
// backward pass needs.  Leaves the kMlpOut outputs per row in S.out.
int surrogate_forward(Surrogate& S, long long n, bool train, cudaStream_t st) {
  launch_features(n, S.coords, S.F, train ? S.FT : nullptr, st);
  if (S.lay.cond) launch_cond_bias(S.groups, S.w + S.lay.U, S.G, nullptr, S.cbias, st);
  const __nv_bfloat16* prev = S.F;
  for (int l = 0; l < 4; l++) {
    GemmArgs g = {};
    g.A = prev;
    g.lda = S.lay.in[l];
    g.B = S.wb[l];
    g.ldb = S.lay.in[l];
    g.M = (int)n;
    g.N = S.lay.out[l];
    g.K = S.lay.in[l];
    g.alpha = 1.0f;
    g.bias = S.w + S.lay.b[l];
    if (l == 0 && S.lay.cond) {
      g.row_bias = S.cbias;
      g.row_group = S.group;
    }
    g.Dsilu = train ? S.dsilu[l] : nullptr;
    g.silu = 1;
    g.Hbf16 = S.H[l];
    g.ldh = S.lay.out[l];
    g.HTbf16 = train ? S.HT[l] : nullptr;
    g.ldht = n;
    g.error = S.error;
    if (launch_gemm_tn(g, 1, st)) return fail(SFSIM_ATMO_ECUDA, "forward GEMM launch failed");
    prev = S.H[l];
  }
  launch_head_forward(n, S.H[3], S.w + S.lay.W[4], S.w + S.lay.b[4], S.out, st);
  CUDA_TRY(cudaGetLastError());
  return 0;
}

// Gradients of the loss (k_mlp.cu: k_loss_grad) over n rows into S.g (zeroed
// first); the loss lands in S.loss.
int surrogate_backward(Surrogate& S, long long n, float huber, cudaStream_t st) {
  CUDA_TRY(cudaMemsetAsync(S.g, 0, sizeof(float) * S.lay.total, st));
  CUDA_TRY(cudaMemsetAsync(S.loss, 0, sizeof(float), st));
  launch_loss_grad(n, S.out, S.target, huber, kVarWeight, S.dout, S.loss, st);
  launch_head_backward(n, S.dout, S.H[3], S.w + S.lay.W[4], S.dsilu[3], S.dZ[3], S.dZT[3], S.g + S.lay.W[4],
                       S.g + S.lay.b[4], st);
  int splits = 1;
  while (splits < 64 && n % (64LL * splits * 2) == 0) splits *= 2;
  for (int l = 3; l >= 0; l--) {
    // dW_l = dZ_l^T H_{l-1}: A = dZ_l^T [out][n], B = H_{l-1}^T [in][n], K = n
    GemmArgs g = {};
    g.A = S.dZT[l];
    g.lda = n;
    g.B = l > 0 ? S.HT[l - 1] : S.FT;
    g.ldb = n;
    g.M = S.lay.out[l];
    g.N = S.lay.in[l];
    g.K = n;
    g.alpha = 1.0f;
    g.Cacc = S.g + S.lay.W[l];
    g.ldc = S.lay.in[l];
    g.error = S.error;
    if (launch_gemm_tn(g, splits, st)) return fail(SFSIM_ATMO_ECUDA, "weight-gradient GEMM launch failed");
    launch_bias_grad(n, S.lay.out[l], S.dZT[l], S.g + S.lay.b[l], st);
    if (l == 0 && S.lay.cond) launch_cond_grad(n, S.dZT[0], S.group, S.groups, S.G, S.g + S.lay.U, st);
    if (l > 0) {
      // dZ_{l-1} = (dZ_l W_l) * SiLU'(z_{l-1}): A = dZ_l [n][out], B = W_l^T [in][out]
      GemmArgs h = {};
      h.A = S.dZ[l];
      h.lda = S.lay.out[l];
      h.B = S.wbt[l];
      h.ldb = S.lay.out[l];
      h.M = (int)n;
      h.N = S.lay.in[l];
      h.K = S.lay.out[l];
      h.alpha = 1.0f;
      h.dact = S.dsilu[l - 1];
      h.Hbf16 = S.dZ[l - 1];
      h.ldh = S.lay.in[l];
      h.HTbf16 = S.dZT[l - 1];
      h.ldht = n;
      h.error = S.error;
      if (launch_gemm_tn(h, 1, st)) return fail(SFSIM_ATMO_ECUDA, "activation-gradient GEMM launch failed");
    }
  }
  CUDA_TRY(cudaGetLastError());
  return 0;
}

void surrogate_adam(Surrogate& S, float lr, int step, cudaStream_t st) {
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  // one launch over every parameter (W_l, b_l, and U of a conditioned
  // network), refreshing the BF16 copies of the four hidden-layer matrices
  AdamMatrices mats;
  mats.n = 4;
  for (int l = 0; l < 4; l++) {
    mats.start[l] = S.lay.W[l];
    mats.rows[l] = S.lay.out[l];
    mats.cols[l] = S.lay.in[l];
    mats.wb[l] = S.wb[l];
    mats.wbt[l] = S.wbt[l];
  }
  launch_adam_all(S.lay.total, S.w, S.g, S.m, S.v, lr, b1, b2, eps, step, mats, st);
}

QueryTables context_tables(const sfsim_atmo_context* ctx) {
  QueryTables q;
  q.radius = (float)ctx->cfg.radius;
  q.max_height = (float)ctx->cfg.height;
  q.mie_g = (float)ctx->cfg.mie.scatter_g;
  q.t_height = ctx->dims.nT0;
  q.t_elevation = ctx->dims.nT1;
  q.height = ctx->dims.n0;
  q.elevation = ctx->dims.n1;
  q.light = ctx->dims.n2;
  q.heading = ctx->dims.n3;
  q.T = ctx->T;
  q.S = ctx->S;
  q.M = ctx->M;
  return q;
}

int check_error_flag(Surrogate& S, cudaStream_t st) {
  int h = 0;
  CUDA_TRY(cudaMemcpyAsync(&h, S.error, sizeof(int), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  if (h) return fail(SFSIM_ATMO_ECUDA, "a tensor-core GEMM wait timed out");
  return 0;
}

// ---------------------------------------------------------------------------
// Allocation-free build.  Some callers cannot call cudaMalloc: engines whose
// allocator reserves every device byte at start-up, or that run under a fixed
// device budget.  For them this entry point builds the tables with all
// scratch in one fixed device array that the library declares at file scope.
// The array (kStaticScratchBytes, 64 MiB) is held on every GPU that loads the
// library until the process exits.  Every call shares it and it keeps the
// last call's contents, so calls that overlap on the GPU race.
// ---------------------------------------------------------------------------

namespace {

constexpr size_t kStaticScratchBytes = 64ull << 20;

static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

// Device address of g_static_scratch per device.  In host code the array's
// name only stands in for the symbol, so the address must come from
// cudaGetSymbolAddress, called with the device current.
void* g_static_base[kMaxDevices];

int static_scratch_base(int dev, void** base) {
  if (!g_static_base[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
    if (e != cudaSuccess || !p)
      return fail(SFSIM_ATMO_ECUDA, std::string("cudaGetSymbolAddress of the static scratch failed: ") +
                                        cudaGetErrorString(e));
    g_static_base[dev] = p;
  }
  *base = g_static_base[dev];
  return 0;
}

template <class Real>
int build_static_impl(const sfsim_atmo_config& cfg, float* T, float* E, float* S, float* M, cudaStream_t st) {
  int dev = 0;
  int rc = current_device(&dev);
  if (rc) return rc;
  BuildDims d = make_dims(cfg, 1);
  if ((rc = check_smem<Real>(d))) return rc;
  Work<Real> w;
  const size_t bytes = carve<Real>(w, nullptr, d, false, false);
  if (bytes > kStaticScratchBytes)
    return fail(SFSIM_ATMO_ETOOBIG, "the build needs " + std::to_string(bytes) +
                                        " bytes of scratch, more than the 67108864-byte static array");
  AtmoParams hp;
  if ((rc = make_params(cfg, hp))) return rc;
  std::vector<DirLocal> dirs, hdirs;
  sphere_directions(cfg.sphere_steps >> 1, cfg.sphere_steps, M_PI, dirs);
  sphere_directions(cfg.ray_steps >> 2, cfg.ray_steps, M_PI / 2, hdirs);
  void* base = nullptr;
  if ((rc = static_scratch_base(dev, &base))) return rc;
  carve<Real>(w, (char*)base, d, false, false);
  // every scratch table is written before it is read, so nothing is cleared;
  // parameters and quadrature directions are copied in on the caller's stream
  g_h2d_bytes = sizeof(AtmoParams) + sizeof(DirLocal) * (dirs.size() + hdirs.size());
  g_d2h_bytes = 0;
  CUDA_TRY(cudaMemcpyAsync(w.params, &hp, sizeof(AtmoParams), cudaMemcpyHostToDevice, st));
  if (!dirs.empty()) {
    CUDA_TRY(cudaMemcpyAsync(w.dirs, dirs.data(), sizeof(DirLocal) * dirs.size(), cudaMemcpyHostToDevice, st));
  }
  if (!hdirs.empty())
    CUDA_TRY(cudaMemcpyAsync(w.hdirs, hdirs.data(), sizeof(DirLocal) * hdirs.size(), cudaMemcpyHostToDevice, st));
  Timer tm;
  tm.dev = dev;
  tm.st = st;
  tm.n = 512;  // a full event list: this entry point records no stage timings
  tm.side = false;  // and uses no stream but the caller's
  g_have_timings = 0;  // so sfsim_atmo_last_timings reports none for this build
  return run_build<Real>(w, d, T, E, S, M, st, tm, nullptr);
}

}  // namespace

// ---------------------------------------------------------------------------
// Plans: a build prepared once (scratch allocated, parameters and quadrature
// directions uploaded) so that the build itself only launches kernels and can
// be captured into a CUDA graph and replayed.
// ---------------------------------------------------------------------------

struct sfsim_atmo_plan {
  int dev;
  sfsim_atmo_config cfg;
  BuildDims dims;
  void* mem;
  Work<float> wf;
  Work<double> wd;
};

namespace {

template <class Real>
int plan_prepare(sfsim_atmo_plan* p, Work<Real>& w) {
  int rc = 0;
  const sfsim_atmo_config& cfg = p->cfg;
  BuildDims d = make_dims(cfg, 1);
  if ((rc = check_smem<Real>(d))) return rc;
  AtmoParams hp;
  if ((rc = make_params(cfg, hp))) return rc;
  std::vector<DirLocal> dirs, hdirs;
  sphere_directions(cfg.sphere_steps >> 1, cfg.sphere_steps, M_PI, dirs);
  sphere_directions(cfg.ray_steps >> 2, cfg.ray_steps, M_PI / 2, hdirs);
  const size_t bytes = carve<Real>(w, nullptr, d, false);
  cudaError_t e = cudaMalloc(&p->mem, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    p->mem = nullptr;
    return fail(SFSIM_ATMO_ENOMEM, std::string("cudaMalloc of the plan failed: ") + cudaGetErrorString(e));
  }
  carve<Real>(w, (char*)p->mem, d, false);
  CUDA_TRY(cudaMemcpy(w.params, &hp, sizeof(AtmoParams), cudaMemcpyHostToDevice));
  if (!dirs.empty()) CUDA_TRY(cudaMemcpy(w.dirs, dirs.data(), sizeof(DirLocal) * dirs.size(), cudaMemcpyHostToDevice));
  if (!hdirs.empty())
    CUDA_TRY(cudaMemcpy(w.hdirs, hdirs.data(), sizeof(DirLocal) * hdirs.size(), cudaMemcpyHostToDevice));
  p->dims = d;
  return 0;
}

}  // namespace

extern "C" int sfsim_atmo_plan_create(const sfsim_atmo_config* cfg, sfsim_atmo_plan** out) {
  if (!out) return fail(SFSIM_ATMO_ENULL, "out is NULL");
  *out = nullptr;
  int rc = validate(cfg);
  if (rc) return rc;
  std::lock_guard<std::mutex> lock(g_mutex);
  int dev = 0;
  if ((rc = current_device(&dev))) return rc;
  if ((rc = ensure_stream(dev))) return rc;
  sfsim_atmo_plan* p = new sfsim_atmo_plan();
  p->dev = dev;
  p->cfg = *cfg;
  p->mem = nullptr;
  rc = cfg->precision == SFSIM_ATMO_FP64 ? plan_prepare<double>(p, p->wd) : plan_prepare<float>(p, p->wf);
  if (rc) {
    if (p->mem) cudaFree(p->mem);
    delete p;
    return rc;
  }
  *out = p;
  return 0;
}

extern "C" int sfsim_atmo_plan_build(sfsim_atmo_plan* p, float* T, float* E, float* S, float* M, void* stream) {
  if (!p) return fail(SFSIM_ATMO_ENULL, "plan is NULL");
  if (!T || !E || !S || !M) return fail(SFSIM_ATMO_ENULL, "an output pointer is NULL");
  std::lock_guard<std::mutex> lock(g_mutex);
  int cur = 0;
  CUDA_TRY(cudaGetDevice(&cur));
  if (cur != p->dev) return fail(SFSIM_ATMO_EINVAL, "the plan belongs to another device");
  Timer tm;
  tm.dev = p->dev;
  tm.st = (cudaStream_t)stream;
  tm.n = 512;  // a full event list: no stage timings, nothing but kernel launches
  g_have_timings = 0;
  g_h2d_bytes = g_d2h_bytes = 0;
  if (p->cfg.precision == SFSIM_ATMO_FP64)
    return run_build<double>(p->wd, p->dims, T, E, S, M, (cudaStream_t)stream, tm, nullptr);
  return run_build<float>(p->wf, p->dims, T, E, S, M, (cudaStream_t)stream, tm, nullptr);
}

extern "C" int sfsim_atmo_plan_destroy(sfsim_atmo_plan* p) {
  if (!p) return 0;
  int cur = 0;
  cudaGetDevice(&cur);
  cudaSetDevice(p->dev);
  cudaError_t e = p->mem ? cudaFree(p->mem) : cudaSuccess;
  cudaSetDevice(cur);
  delete p;
  if (e != cudaSuccess) return fail(SFSIM_ATMO_ECUDA, std::string("cudaFree: ") + cudaGetErrorString(e));
  return 0;
}

extern "C" int sfsim_atmo_build_static(const sfsim_atmo_config* cfg, float* T, float* E, float* S, float* M,
                                       void* stream) {
  int rc = validate(cfg);
  if (rc) return rc;
  if (!T || !E || !S || !M) return fail(SFSIM_ATMO_ENULL, "an output pointer is NULL");
  std::lock_guard<std::mutex> lock(g_mutex);
  if (cfg->precision == SFSIM_ATMO_FP64) return build_static_impl<double>(*cfg, T, E, S, M, (cudaStream_t)stream);
  return build_static_impl<float>(*cfg, T, E, S, M, (cudaStream_t)stream);
}

extern "C" {

int sfsim_atmo_context_create(const sfsim_atmo_config* cfg, sfsim_atmo_context** out) {
  if (!out) return fail(SFSIM_ATMO_ENULL, "out is NULL");
  *out = nullptr;
  int rc = validate(cfg);
  if (rc) return rc;
  std::lock_guard<std::mutex> lock(g_mutex);
  int dev = 0;
  if ((rc = current_device(&dev))) return rc;
  if ((rc = ensure_stream(dev))) return rc;
  sfsim_atmo_context* c = new sfsim_atmo_context();
  c->dev = dev;
  c->cfg = *cfg;
  c->mem = nullptr;
  c->sur = nullptr;
  rc = cfg->precision == SFSIM_ATMO_FP64 ? context_build<double>(c) : context_build<float>(c);
  if (rc) {
    if (c->mem) cudaFree(c->mem);
    delete c;
    return rc;
  }
  *out = c;
  return 0;
}

int sfsim_atmo_context_destroy(sfsim_atmo_context* ctx) {
  if (!ctx) return 0;
  int cur = 0;
  cudaGetDevice(&cur);
  cudaSetDevice(ctx->dev);
  surrogate_free(ctx);
  cudaError_t e = ctx->mem ? cudaFree(ctx->mem) : cudaSuccess;
  cudaSetDevice(cur);
  delete ctx;
  if (e != cudaSuccess) return fail(SFSIM_ATMO_ECUDA, std::string("cudaFree: ") + cudaGetErrorString(e));
  return 0;
}

int sfsim_atmo_context_tables(const sfsim_atmo_context* ctx, float** T, float** E, float** S, float** M) {
  if (!ctx) return fail(SFSIM_ATMO_ENULL, "context is NULL");
  if (T) *T = ctx->T;
  if (E) *E = ctx->E;
  if (S) *S = ctx->S;
  if (M) *M = ctx->M;
  return 0;
}

int sfsim_atmo_context_point_scatter_sum(const sfsim_atmo_context* ctx, float** jsum) {
  if (!ctx || !jsum) return fail(SFSIM_ATMO_ENULL, "NULL argument");
  *jsum = reinterpret_cast<float*>(ctx->jsum);
  return 0;
}

int sfsim_atmo_query_table(const sfsim_atmo_context* ctx, int kind, long long n, const float* a, const float* b,
                           const float* light, float* out, int weight_bits, void* stream) {
  if (!ctx) return fail(SFSIM_ATMO_ENULL, "context is NULL");
  if (kind < 0 || kind > 4) return fail(SFSIM_ATMO_EINVAL, "query kind must be in [0, 4]");
  if (weight_bits < 0 || weight_bits > 16) return fail(SFSIM_ATMO_EINVAL, "weight_bits must be in [0, 16]");
  if (n < 0) return fail(SFSIM_ATMO_EINVAL, "n must be non-negative");
  if (n == 0) return 0;
  if (!a || !b || !out || (kind >= 2 && !light)) return fail(SFSIM_ATMO_ENULL, "a point array is NULL");
  QueryTables q;
  q.radius = (float)ctx->cfg.radius;
  q.max_height = (float)ctx->cfg.height;
  q.mie_g = (float)ctx->cfg.mie.scatter_g;
  q.t_height = ctx->dims.nT0;
  q.t_elevation = ctx->dims.nT1;
  q.height = ctx->dims.n0;
  q.elevation = ctx->dims.n1;
  q.light = ctx->dims.n2;
  q.heading = ctx->dims.n3;
  q.T = ctx->T;
  q.S = ctx->S;
  q.M = ctx->M;
  launch_query_table(q, kind, n, a, b, light, out, weight_bits, (cudaStream_t)stream);
  CUDA_TRY(cudaGetLastError());
  return 0;
}

int sfsim_atmo_query_attenuation(const sfsim_atmo_context* ctx, int kind, long long n, const float* light,
                                 const float* p, const float* d, const float* s, const float* incoming,
                                 float amplification, float* out, int weight_bits, void* stream) {
  if (!ctx) return fail(SFSIM_ATMO_ENULL, "context is NULL");
  if (kind < 0 || kind > 3) return fail(SFSIM_ATMO_EINVAL, "attenuation kind must be in [0, 3]");
  if (weight_bits < 0 || weight_bits > 16) return fail(SFSIM_ATMO_EINVAL, "weight_bits must be in [0, 16]");
  if (n < 0) return fail(SFSIM_ATMO_EINVAL, "n must be non-negative");
  if (n == 0) return 0;
  if (!light || !p || !out || (kind <= 2 && (!d || !incoming)) || (kind <= 1 && !s))
    return fail(SFSIM_ATMO_ENULL, "an input or output array of this kind is NULL");
  QueryTables q;
  q.radius = (float)ctx->cfg.radius;
  q.max_height = (float)ctx->cfg.height;
  q.mie_g = (float)ctx->cfg.mie.scatter_g;
  q.t_height = ctx->dims.nT0;
  q.t_elevation = ctx->dims.nT1;
  q.height = ctx->dims.n0;
  q.elevation = ctx->dims.n1;
  q.light = ctx->dims.n2;
  q.heading = ctx->dims.n3;
  q.T = ctx->T;
  q.S = ctx->S;
  q.M = ctx->M;
  launch_query_attenuation(q, kind, n, light, p, d, s, incoming, amplification, out, weight_bits,
                           (cudaStream_t)stream);
  CUDA_TRY(cudaGetLastError());
  return 0;
}

int sfsim_atmo_query_direct(const sfsim_atmo_context* ctx, long long n, const double* x, const double* v,
                            const double* l, float* out, void* stream) {
  if (!ctx) return fail(SFSIM_ATMO_ENULL, "context is NULL");
  if (n < 0) return fail(SFSIM_ATMO_EINVAL, "n must be non-negative");
  if (n == 0) return 0;
  if (!x || !v || !l || !out) return fail(SFSIM_ATMO_ENULL, "a point array is NULL");
  launch_query_direct(ctx->params, ctx->dims, ctx->jsum, n, x, v, l, out, (cudaStream_t)stream);
  CUDA_TRY(cudaGetLastError());
  return 0;
}

}  // extern "C"

extern "C" int sfsim_atmo_gemm_bf16(const void* A, const void* B, float* C, int M, int N, long long K, int splits,
                                    void* stream) {
  if (!A || !B || !C) return fail(SFSIM_ATMO_ENULL, "a matrix pointer is NULL");
  if (M < 1 || N < 1 || N > 256 || K < 64 || splits < 1 || K % (64LL * splits) != 0)
    return fail(SFSIM_ATMO_EINVAL, "need M >= 1, 1 <= N <= 256, K a multiple of 64 * splits");
  GemmArgs g = {};
  g.A = (const __nv_bfloat16*)A;
  g.lda = K;
  g.B = (const __nv_bfloat16*)B;
  g.ldb = K;
  g.M = M;
  g.N = N;
  g.K = K;
  g.alpha = 1.0f;
  g.ldc = N;
  if (splits > 1) g.Cacc = C;
  else g.Cf32 = C;
  if (splits > 1) CUDA_TRY(cudaMemsetAsync(C, 0, sizeof(float) * (size_t)M * N, (cudaStream_t)stream));
  if (launch_gemm_tn(g, splits, (cudaStream_t)stream)) return fail(SFSIM_ATMO_ECUDA, "GEMM launch configuration failed");
  CUDA_TRY(cudaGetLastError());
  return 0;
}

// ---------------------------------------------------------------------------
// Bounded waits of the tensor-core kernels
// ---------------------------------------------------------------------------

namespace {
std::atomic<int> g_wait_limit{kDefaultWaitLimit};
}

int sfsim::wait_limit() { return g_wait_limit.load(std::memory_order_relaxed); }

extern "C" long long sfsim_atmo_set_wait_limit(long long polls) {
  const int v = polls <= 0 ? kDefaultWaitLimit : (int)std::min<long long>(polls, 0x7fffffffLL);
  return g_wait_limit.exchange(v);
}

extern "C" int sfsim_atmo_wait_selftest(int polls) {
  if (polls < 1 || polls > 1000000) return fail(SFSIM_ATMO_EINVAL, "polls must be in 1 .. 1000000");
  std::lock_guard<std::mutex> lock(g_mutex);
  int dev = 0;
  int rc = current_device(&dev);
  if (rc) return rc;
  if ((rc = ensure_stream(dev))) return rc;
  const int M = 128, N = 256;
  const long long K = 4096;
  void *A = nullptr, *B = nullptr;
  float* C = nullptr;
  int* err = nullptr;
  auto release = [&] {
    cudaFree(A);
    cudaFree(B);
    cudaFree(C);
    cudaFree(err);
  };
  if (cudaMalloc(&A, sizeof(__nv_bfloat16) * M * K) != cudaSuccess ||
      cudaMalloc(&B, sizeof(__nv_bfloat16) * N * K) != cudaSuccess ||
      cudaMalloc(&C, sizeof(float) * M * N) != cudaSuccess || cudaMalloc(&err, sizeof(int)) != cudaSuccess) {
    cudaGetLastError();
    release();
    return fail(SFSIM_ATMO_ENOMEM, "self-test operands could not be allocated");
  }
  cudaStream_t st = g_stream[dev];
  int h = 0;
  cudaError_t e = cudaMemsetAsync(A, 0, sizeof(__nv_bfloat16) * M * K, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(B, 0, sizeof(__nv_bfloat16) * N * K, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(err, 0, sizeof(int), st);
  GemmArgs g = {};
  g.A = (const __nv_bfloat16*)A;
  g.lda = K;
  g.B = (const __nv_bfloat16*)B;
  g.ldb = K;
  g.M = M;
  g.N = N;
  g.K = K;
  g.alpha = 1.0f;
  g.Cf32 = C;
  g.ldc = N;
  g.error = err;
  g.stall_polls = polls;
  if (e == cudaSuccess && launch_gemm_tn(g, 1, st)) e = cudaErrorInvalidConfiguration;
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  release();
  if (e != cudaSuccess) return fail(SFSIM_ATMO_ECUDA, std::string("wait self-test: ") + cudaGetErrorString(e));
  if (h)
    return fail(SFSIM_ATMO_ECUDA, "a tensor-core wait timed out after " + std::to_string(polls) +
                                      " polls (self-test: the GEMM epilogue waited on a barrier that nothing "
                                      "arrives on)");
  return 0;
}

// ---------------------------------------------------------------------------
// Surrogate entry points
// ---------------------------------------------------------------------------

namespace {

int surrogate_pools(sfsim_atmo_context* c, long long n_direct, unsigned long long seed, float** node_pool,
                    float** direct_pool, std::vector<void*>& temps, cudaStream_t st) {
  const BuildDims& d = c->dims;
  void* p = nullptr;
  if (cudaMalloc(&p, sizeof(float) * kPoolRow * (size_t)d.n4()) != cudaSuccess)
    return fail(SFSIM_ATMO_ENOMEM, "node pool allocation failed");
  temps.push_back(p);
  *node_pool = (float*)p;
  launch_node_pool(d, *node_pool, st);
  *direct_pool = nullptr;
  if (n_direct > 0) {
    if (cudaMalloc(&p, sizeof(float) * kPoolRow * (size_t)n_direct) != cudaSuccess)
      return fail(SFSIM_ATMO_ENOMEM, "direct pool allocation failed");
    temps.push_back(p);
    *direct_pool = (float*)p;
    const long long chunk = 1 << 20;
    double* xvl = nullptr;
    float *vals = nullptr, *crd = nullptr, *tab = nullptr;
    auto get = [&](void** q, size_t bytes) {
      if (cudaMalloc(q, bytes) != cudaSuccess) return false;
      temps.push_back(*q);
      return true;
    };
    if (!get((void**)&xvl, sizeof(double) * 9 * chunk) || !get((void**)&vals, sizeof(float) * 3 * chunk) ||
        !get((void**)&crd, sizeof(float) * kMlpCoords * chunk) || !get((void**)&tab, sizeof(float) * 3 * chunk))
      return fail(SFSIM_ATMO_ENOMEM, "direct sample allocation failed");
    const QueryTables q = context_tables(c);
    for (long long o = 0; o < n_direct; o += chunk) {
      const long long m = std::min(chunk, n_direct - o);
      launch_random_queries(m, seed * 1000003ull + (unsigned long long)o, c->cfg.radius, c->cfg.height, xvl,
                            xvl + 3 * chunk, xvl + 6 * chunk, st);
      launch_query_direct(c->params, d, c->jsum, m, xvl, xvl + 3 * chunk, xvl + 6 * chunk, vals, st);
      launch_query_coords(q, m, xvl, xvl + 3 * chunk, xvl + 6 * chunk, crd, tab, st);
      launch_make_pool(m, crd, vals, tab, kLogEps, *direct_pool + kPoolRow * o, st);
    }
  }
  CUDA_TRY(cudaGetLastError());
  return 0;
}

int check_train_config(const sfsim_atmo_surrogate_config* sc) {
  if (sc->steps < 0 || sc->batch < 1024 || sc->batch % 1024 != 0 || sc->direct_samples < 0 ||
      !(sc->node_fraction >= 0 && sc->node_fraction <= 1) || !(sc->lr > 0) || !(sc->huber_delta >= 0))
    return fail(SFSIM_ATMO_EINVAL,
                "steps >= 0, batch a positive multiple of 1024, lr > 0, node_fraction in [0, 1], huber_delta >= 0");
  return 0;
}

// The Adam steps of one training call (cosine-decayed learning rate); `gather`
// fills S.coords and S.target (and S.group) for step t.  `rc` carries an
// error of the caller's set-up, in which case nothing runs.  Frees `temps`.
template <class Gather>
int run_training(Surrogate& S, const sfsim_atmo_surrogate_config* sc, int rc, Gather gather, float* loss_history,
                 std::vector<void*>& temps, cudaStream_t st) {
  float* hist = nullptr;
  if (!rc && cudaMalloc(&hist, sizeof(float) * std::max(1, sc->steps)) != cudaSuccess)
    rc = fail(SFSIM_ATMO_ENOMEM, "loss history allocation failed");
  if (hist) temps.push_back(hist);
  const long long n = sc->batch;
  for (int t = 0; t < sc->steps && !rc; t++) {
    const float lr = sc->lr * 0.5f * (1.0f + std::cos(3.14159265358979f * (float)t / (float)sc->steps));
    gather(t);
    if ((rc = surrogate_forward(S, n, true, st))) break;
    if ((rc = surrogate_backward(S, n, sc->huber_delta, st))) break;
    surrogate_adam(S, lr, S.trained_steps + t + 1, st);
    if (cudaMemcpyAsync(hist + t, S.loss, sizeof(float), cudaMemcpyDeviceToDevice, st) != cudaSuccess)
      rc = fail(SFSIM_ATMO_ECUDA, "loss copy failed");
  }
  if (!rc && loss_history && sc->steps > 0 &&
      cudaMemcpyAsync(loss_history, hist, sizeof(float) * sc->steps, cudaMemcpyDeviceToHost, st) != cudaSuccess)
    rc = fail(SFSIM_ATMO_ECUDA, "loss history copy failed");
  if (!rc) rc = check_error_flag(S, st);
  if (!rc && sc->steps > 0) {
    // a diverged run (learning rate too high) leaves non-finite losses
    float last = 0.0f;
    if (cudaMemcpyAsync(&last, hist + sc->steps - 1, sizeof(float), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
      rc = fail(SFSIM_ATMO_ECUDA, "loss readback failed");
    else if (!std::isfinite(last))
      rc = fail(SFSIM_ATMO_ENUMERIC, "surrogate training diverged (non-finite loss); lower the learning rate");
  }
  cudaStreamSynchronize(st);
  for (void* p : temps) cudaFree(p);
  temps.clear();
  if (!rc) S.trained_steps += sc->steps;
  return rc;
}

}  // namespace

extern "C" {

int sfsim_atmo_surrogate_train(sfsim_atmo_context* ctx, const sfsim_atmo_surrogate_config* sc, float* loss_history) {
  if (!ctx || !sc) return fail(SFSIM_ATMO_ENULL, "NULL argument");
  if (ctx->cfg.precision != SFSIM_ATMO_FP32) return fail(SFSIM_ATMO_EINVAL, "the surrogate needs an FP32 context");
  int rc = check_train_config(sc);
  if (rc) return rc;
  std::lock_guard<std::mutex> lock(g_mutex);
  int cur = 0;
  CUDA_TRY(cudaGetDevice(&cur));
  if (cur != ctx->dev) return fail(SFSIM_ATMO_EINVAL, "the context belongs to another device");
  rc = surrogate_alloc(ctx->sur, 0, sc->batch, sc->seed);
  if (rc) return rc;
  Surrogate& S = *ctx->sur;
  cudaStream_t st = g_stream[ctx->dev];
  std::vector<void*> temps;
  float *node_pool = nullptr, *direct_pool = nullptr;
  rc = surrogate_pools(ctx, sc->direct_samples, sc->seed, &node_pool, &direct_pool, temps, st);
  const long long na = ctx->dims.n4();
  auto gather = [&](int t) {
    launch_gather_batch(sc->batch, sc->seed * 0x9E3779B97F4A7C15ull + (unsigned long long)t, sc->node_fraction,
                        node_pool, na, direct_pool, sc->direct_samples, S.coords, S.target, st);
  };
  return run_training(S, sc, rc, gather, loss_history, temps, st);
}

int sfsim_atmo_surrogate_parameters(sfsim_atmo_context* ctx, float* get, const float* set, long long* count) {
  if (!ctx) return fail(SFSIM_ATMO_ENULL, "context is NULL");
  MlpLayout lay;
  if (count) *count = lay.total;
  if (!get && !set) return 0;
  std::lock_guard<std::mutex> lock(g_mutex);
  int rc = surrogate_alloc(ctx->sur, 0, 1024, 1);
  if (rc) return rc;
  Surrogate& S = *ctx->sur;
  if (set) {
    CUDA_TRY(cudaMemcpy(S.w, set, sizeof(float) * lay.total, cudaMemcpyHostToDevice));
    for (int l = 0; l < 4; l++)
      launch_to_bf16((long long)lay.in[l] * lay.out[l], S.w + lay.W[l], lay.out[l], lay.in[l], S.wb[l], S.wbt[l], 0);
    CUDA_TRY(cudaDeviceSynchronize());
  }
  if (get) CUDA_TRY(cudaMemcpy(get, S.w, sizeof(float) * lay.total, cudaMemcpyDeviceToHost));
  return 0;
}

int sfsim_atmo_surrogate_gradients(sfsim_atmo_context* ctx, long long n, const float* coords, const float* targets,
                                   float* loss, float* grads) {
  if (!ctx || !coords || !targets) return fail(SFSIM_ATMO_ENULL, "NULL argument");
  if (n < 1024 || n % 1024 != 0) return fail(SFSIM_ATMO_EINVAL, "n must be a positive multiple of 1024");
  std::lock_guard<std::mutex> lock(g_mutex);
  int rc = surrogate_alloc(ctx->sur, 0, n, 1);
  if (rc) return rc;
  Surrogate& S = *ctx->sur;
  cudaStream_t st = g_stream[ctx->dev];
  CUDA_TRY(cudaMemcpyAsync(S.coords, coords, sizeof(float) * kMlpCoords * n, cudaMemcpyHostToDevice, st));
  CUDA_TRY(cudaMemcpyAsync(S.target, targets, sizeof(float) * 3 * n, cudaMemcpyHostToDevice, st));
  if ((rc = surrogate_forward(S, n, true, st))) return rc;
  if ((rc = surrogate_backward(S, n, 0.0f, st))) return rc;
  if (loss) CUDA_TRY(cudaMemcpyAsync(loss, S.loss, sizeof(float), cudaMemcpyDeviceToHost, st));
  if (grads) CUDA_TRY(cudaMemcpyAsync(grads, S.g, sizeof(float) * S.lay.total, cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  return check_error_flag(S, st);
}

int sfsim_atmo_query_coords(const sfsim_atmo_context* ctx, long long n, const double* x, const double* v,
                            const double* l, float* coords, void* stream) {
  if (!ctx || !x || !v || !l || !coords) return fail(SFSIM_ATMO_ENULL, "NULL argument");
  if (n < 0) return fail(SFSIM_ATMO_EINVAL, "n must be non-negative");
  if (n == 0) return 0;
  launch_query_coords(context_tables(ctx), n, x, v, l, coords, nullptr, (cudaStream_t)stream);
  CUDA_TRY(cudaGetLastError());
  return 0;
}

}  // extern "C"

namespace {

// Surrogate queries of the atmosphere `ctx` (its tables, and its quadrature
// for the fallback) with the network S, whose first-layer bias is `bias0`.
// The caller holds g_mutex.
int surrogate_query(Surrogate& S, const float* bias0, const sfsim_atmo_context* ctx, long long n, const double* x,
                    const double* v, const double* l, float* out, float threshold, long long* n_fallback,
                    cudaStream_t st) {
  const QueryTables q = context_tables(ctx);
  const bool fallback = threshold > 0;
  long long* list = nullptr;  // indices of the flagged queries
  unsigned long long* count = nullptr;
  if (fallback) {
    if (cudaMalloc(&list, sizeof(long long) * (size_t)n) != cudaSuccess ||
        cudaMalloc(&count, sizeof(unsigned long long)) != cudaSuccess) {
      if (list) cudaFree(list);
      return fail(SFSIM_ATMO_ENOMEM, "fallback list allocation failed");
    }
    CUDA_TRY(cudaMemsetAsync(count, 0, sizeof(unsigned long long), st));
  }
  const float* biases[4];
  for (int i = 0; i < 4; i++) biases[i] = S.w + S.lay.b[i];
  biases[0] = bias0;
  int rc = 0, sms = 0;
  CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->dev));
  // queries go through in chunks: the lookup kernel forms coordinates and
  // table values into a cached scratch buffer, the fused kernel evaluates them
  const long long chunk = std::min(n, kQueryChunk);
  if (S.qcap < chunk) {
    if (S.qbuf) cudaFree(S.qbuf);
    S.qbuf = nullptr;
    S.qcap = 0;
    if (cudaMalloc(&S.qbuf, sizeof(float) * (kMlpCoords + 3) * (size_t)chunk) != cudaSuccess) {
      S.qbuf = nullptr;
      rc = fail(SFSIM_ATMO_ENOMEM, "query scratch allocation failed");
    } else {
      S.qcap = chunk;
    }
  }
  if (!rc) launch_pack_infer(S.wb, S.packed, st);
  for (long long o = 0; o < n && !rc; o += chunk) {
    const long long m = std::min(chunk, n - o);
    float* crd = S.qbuf;
    float* tab = S.qbuf + kMlpCoords * chunk;
    launch_query_coords(q, m, x + 3 * o, v + 3 * o, l + 3 * o, crd, tab, st);
    if (launch_surrogate_infer(m, crd, tab, S.packed, biases, S.w + S.lay.W[4], S.w + S.lay.b[4], kLogEps,
                               fallback ? threshold : 0.0f, out + 3 * o, list, o, count, S.error, sms, st))
      rc = fail(SFSIM_ATMO_ECUDA, "surrogate inference launch configuration failed");
  }
  if (!rc && cudaGetLastError() != cudaSuccess) rc = fail(SFSIM_ATMO_ECUDA, "surrogate query launch failed");
  if (fallback) {
    // the flagged queries, compacted into `list`, go to the direct quadrature
    unsigned long long h = 0;
    if (!rc && (cudaMemcpyAsync(&h, count, sizeof(h), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
                cudaStreamSynchronize(st) != cudaSuccess))
      rc = fail(SFSIM_ATMO_ECUDA, "fallback count readback failed");
    if (!rc && h > (unsigned long long)n) rc = fail(SFSIM_ATMO_ECUDA, "fallback count out of range");
    if (!rc) launch_query_direct(ctx->params, ctx->dims, ctx->jsum, (long long)h, x, v, l, out, st, list);
    if (!rc && cudaGetLastError() != cudaSuccess) rc = fail(SFSIM_ATMO_ECUDA, "fallback launch failed");
    if (!rc && n_fallback) *n_fallback = (long long)h;
    cudaStreamSynchronize(st);
    cudaFree(list);
    cudaFree(count);
    // the call synchronised: report a wait that timed out in the inference kernel
    if (!rc) rc = check_error_flag(S, st);
  }
  return rc;
}


}  // namespace

extern "C" {

int sfsim_atmo_query_surrogate(sfsim_atmo_context* ctx, long long n, const double* x, const double* v,
                               const double* l, float* out, float threshold, long long* n_fallback, void* stream) {
  if (!ctx || !x || !v || !l || !out) return fail(SFSIM_ATMO_ENULL, "NULL argument");
  if (!ctx->sur) return fail(SFSIM_ATMO_EINVAL, "the context has no trained surrogate");
  if (n < 0) return fail(SFSIM_ATMO_EINVAL, "n must be non-negative");
  if (n_fallback) *n_fallback = 0;
  if (n == 0) return 0;
  std::lock_guard<std::mutex> lock(g_mutex);
  Surrogate& S = *ctx->sur;
  return surrogate_query(S, S.w + S.lay.b[0], ctx, n, x, v, l, out, threshold, n_fallback, (cudaStream_t)stream);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Conditioned surrogate: one network for many atmospheres, whose first layer
// also takes kCondInputs inputs describing the atmosphere.  Trained on several
// contexts at once; queried on any context (also one it never saw), whose
// table it corrects.
// ---------------------------------------------------------------------------

struct sfsim_atmo_cond_surrogate {
  int dev;
  unsigned long long seed;
  Surrogate* sur;
};

namespace {

// The atmosphere inputs, each about [-1, 1] over the parameter sweep: log2 of
// the Rayleigh coefficients (RGB) and of the Mie coefficient (red) relative
// to Earth's, the two scale heights, the Mie asymmetry and the radius.
void condition_inputs(const sfsim_atmo_config& c, float* g) {
  auto lg = [](double a, double ref) { return std::log2(std::max(a, 1e-30) / ref); };
  const double v[kCondInputs] = {lg(c.rayleigh.scatter_base[0], 5.8e-6), lg(c.rayleigh.scatter_base[1], 13.5e-6),
                                 lg(c.rayleigh.scatter_base[2], 33.1e-6), lg(c.mie.scatter_base[0], 2e-5),
                                 (c.rayleigh.scatter_scale - 8000.0) / 2000.0, (c.mie.scatter_scale - 1400.0) / 600.0,
                                 (c.mie.scatter_g - 0.725) / 0.125,        (c.radius - 5.0e6) / 2.0e6};
  for (int p = 0; p < kCondInputs; p++) g[p] = (float)std::min(8.0, std::max(-8.0, v[p]));
}

int cond_prologue(sfsim_atmo_cond_surrogate* cs) {
  int cur = 0;
  CUDA_TRY(cudaGetDevice(&cur));
  if (cur != cs->dev) return fail(SFSIM_ATMO_EINVAL, "the surrogate belongs to another device");
  return ensure_stream(cs->dev);
}

}  // namespace

extern "C" {

int sfsim_atmo_condition_inputs(const sfsim_atmo_config* cfg, float* inputs) {
  if (!cfg || !inputs) return fail(SFSIM_ATMO_ENULL, "NULL argument");
  condition_inputs(*cfg, inputs);
  return 0;
}

int sfsim_atmo_cond_surrogate_create(unsigned long long seed, sfsim_atmo_cond_surrogate** out) {
  if (!out) return fail(SFSIM_ATMO_ENULL, "out is NULL");
  *out = nullptr;
  std::lock_guard<std::mutex> lock(g_mutex);
  int dev = 0, rc = current_device(&dev);
  if (rc) return rc;
  if ((rc = ensure_stream(dev))) return rc;
  sfsim_atmo_cond_surrogate* cs = new sfsim_atmo_cond_surrogate();
  cs->dev = dev;
  cs->seed = seed;
  cs->sur = nullptr;
  if ((rc = surrogate_alloc(cs->sur, kCondInputs, 1024, seed))) {
    if (cs->sur) {
      cs->sur->free_all();
      delete cs->sur;
    }
    delete cs;
    return rc;
  }
  *out = cs;
  return 0;
}

int sfsim_atmo_cond_surrogate_destroy(sfsim_atmo_cond_surrogate* cs) {
  if (!cs) return 0;
  int cur = 0;
  cudaGetDevice(&cur);
  cudaSetDevice(cs->dev);
  if (cs->sur) {
    cs->sur->free_all();
    delete cs->sur;
  }
  cudaSetDevice(cur);
  delete cs;
  return 0;
}

int sfsim_atmo_cond_surrogate_train(sfsim_atmo_cond_surrogate* cs, sfsim_atmo_context* const* ctxs, int n_ctx,
                                    const sfsim_atmo_surrogate_config* sc, float* loss_history) {
  if (!cs || !ctxs || !sc) return fail(SFSIM_ATMO_ENULL, "NULL argument");
  if (n_ctx < 1 || n_ctx > kMaxCondGroups)
    return fail(SFSIM_ATMO_EINVAL, "n_ctx must be in [1, " + std::to_string(kMaxCondGroups) + "]");
  int rc = check_train_config(sc);
  if (rc) return rc;
  for (int a = 0; a < n_ctx; a++) {
    const sfsim_atmo_context* c = ctxs[a];
    if (!c) return fail(SFSIM_ATMO_ENULL, "a context is NULL");
    if (c->cfg.precision != SFSIM_ATMO_FP32) return fail(SFSIM_ATMO_EINVAL, "the surrogate needs FP32 contexts");
    if (c->dev != cs->dev) return fail(SFSIM_ATMO_EINVAL, "a context belongs to another device");
    if (c->dims.n4() != ctxs[0]->dims.n4())
      return fail(SFSIM_ATMO_EINVAL, "the contexts must share their ray-scatter shape");
  }
  std::lock_guard<std::mutex> lock(g_mutex);
  if ((rc = cond_prologue(cs))) return rc;
  if ((rc = surrogate_alloc(cs->sur, kCondInputs, sc->batch, cs->seed))) return rc;
  Surrogate& S = *cs->sur;
  cudaStream_t st = g_stream[cs->dev];
  std::vector<void*> temps;
  // per atmosphere: its inputs and its two pools (table nodes, direct samples)
  std::vector<float> G((size_t)n_ctx * kCondInputs);
  std::vector<const float*> pa(n_ctx), pb(n_ctx);
  for (int a = 0; a < n_ctx && !rc; a++) {
    condition_inputs(ctxs[a]->cfg, G.data() + (size_t)a * kCondInputs);
    float *node_pool = nullptr, *direct_pool = nullptr;
    rc = surrogate_pools(ctxs[a], sc->direct_samples, sc->seed * 7919ull + (unsigned long long)a, &node_pool,
                         &direct_pool, temps, st);
    pa[a] = node_pool;
    pb[a] = direct_pool;
  }
  const float** dp = nullptr;
  if (!rc) {
    void* p = nullptr;
    if (cudaMalloc(&p, sizeof(float*) * 2 * (size_t)n_ctx) != cudaSuccess) {
      rc = fail(SFSIM_ATMO_ENOMEM, "pool table allocation failed");
    } else {
      temps.push_back(p);
      dp = (const float**)p;
      std::vector<const float*> both(pa);
      both.insert(both.end(), pb.begin(), pb.end());
      if (cudaMemcpyAsync(dp, both.data(), sizeof(float*) * 2 * (size_t)n_ctx, cudaMemcpyHostToDevice, st) !=
              cudaSuccess ||
          cudaMemcpyAsync(S.G, G.data(), sizeof(float) * G.size(), cudaMemcpyHostToDevice, st) != cudaSuccess ||
          cudaStreamSynchronize(st) != cudaSuccess)
        rc = fail(SFSIM_ATMO_ECUDA, "pool table copy failed");
    }
  }
  S.groups = n_ctx;
  const long long na = ctxs[0]->dims.n4();
  auto gather = [&](int t) {
    launch_gather_batch_groups(sc->batch, sc->seed * 0x9E3779B97F4A7C15ull + (unsigned long long)t,
                               sc->node_fraction, n_ctx, dp, na, dp + n_ctx, sc->direct_samples, S.coords, S.target,
                               S.group, st);
  };
  return run_training(S, sc, rc, gather, loss_history, temps, st);
}

int sfsim_atmo_cond_surrogate_parameters(sfsim_atmo_cond_surrogate* cs, float* get, const float* set,
                                         long long* count) {
  if (!cs) return fail(SFSIM_ATMO_ENULL, "surrogate is NULL");
  const MlpLayout lay(kCondInputs);
  if (count) *count = lay.total;
  if (!get && !set) return 0;
  std::lock_guard<std::mutex> lock(g_mutex);
  int rc = cond_prologue(cs);
  if (rc) return rc;
  Surrogate& S = *cs->sur;
  if (set) {
    CUDA_TRY(cudaMemcpy(S.w, set, sizeof(float) * lay.total, cudaMemcpyHostToDevice));
    for (int l = 0; l < 4; l++)
      launch_to_bf16((long long)lay.in[l] * lay.out[l], S.w + lay.W[l], lay.out[l], lay.in[l], S.wb[l], S.wbt[l], 0);
    CUDA_TRY(cudaDeviceSynchronize());
  }
  if (get) CUDA_TRY(cudaMemcpy(get, S.w, sizeof(float) * lay.total, cudaMemcpyDeviceToHost));
  return 0;
}

int sfsim_atmo_cond_surrogate_gradients(sfsim_atmo_cond_surrogate* cs, long long n, const float* coords,
                                        const int* groups, int n_groups, const float* inputs, const float* targets,
                                        float* loss, float* grads) {
  if (!cs || !coords || !groups || !inputs || !targets) return fail(SFSIM_ATMO_ENULL, "NULL argument");
  if (n < 1024 || n % 1024 != 0) return fail(SFSIM_ATMO_EINVAL, "n must be a positive multiple of 1024");
  if (n_groups < 1 || n_groups > kMaxCondGroups)
    return fail(SFSIM_ATMO_EINVAL, "n_groups must be in [1, " + std::to_string(kMaxCondGroups) + "]");
  for (long long i = 0; i < n; i++)
    if (groups[i] < 0 || groups[i] >= n_groups) return fail(SFSIM_ATMO_EINVAL, "a group index is out of range");
  std::lock_guard<std::mutex> lock(g_mutex);
  int rc = cond_prologue(cs);
  if (rc) return rc;
  if ((rc = surrogate_alloc(cs->sur, kCondInputs, n, cs->seed))) return rc;
  Surrogate& S = *cs->sur;
  cudaStream_t st = g_stream[cs->dev];
  S.groups = n_groups;
  CUDA_TRY(cudaMemcpyAsync(S.coords, coords, sizeof(float) * kMlpCoords * n, cudaMemcpyHostToDevice, st));
  CUDA_TRY(cudaMemcpyAsync(S.target, targets, sizeof(float) * 3 * n, cudaMemcpyHostToDevice, st));
  CUDA_TRY(cudaMemcpyAsync(S.group, groups, sizeof(int) * n, cudaMemcpyHostToDevice, st));
  CUDA_TRY(cudaMemcpyAsync(S.G, inputs, sizeof(float) * kCondInputs * n_groups, cudaMemcpyHostToDevice, st));
  if ((rc = surrogate_forward(S, n, true, st))) return rc;
  if ((rc = surrogate_backward(S, n, 0.0f, st))) return rc;
  if (loss) CUDA_TRY(cudaMemcpyAsync(loss, S.loss, sizeof(float), cudaMemcpyDeviceToHost, st));
  if (grads) CUDA_TRY(cudaMemcpyAsync(grads, S.g, sizeof(float) * S.lay.total, cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  return check_error_flag(S, st);
}

int sfsim_atmo_query_cond_surrogate(sfsim_atmo_cond_surrogate* cs, const sfsim_atmo_context* ctx, long long n,
                                    const double* x, const double* v, const double* l, float* out, float threshold,
                                    long long* n_fallback, void* stream) {
  if (!cs || !ctx || !x || !v || !l || !out) return fail(SFSIM_ATMO_ENULL, "NULL argument");
  if (ctx->cfg.precision != SFSIM_ATMO_FP32) return fail(SFSIM_ATMO_EINVAL, "the surrogate needs an FP32 context");
  if (ctx->dev != cs->dev) return fail(SFSIM_ATMO_EINVAL, "the context belongs to another device");
  if (n < 0) return fail(SFSIM_ATMO_EINVAL, "n must be non-negative");
  if (n_fallback) *n_fallback = 0;
  if (n == 0) return 0;
  std::lock_guard<std::mutex> lock(g_mutex);
  int rc = cond_prologue(cs);
  if (rc) return rc;
  Surrogate& S = *cs->sur;
  cudaStream_t st = (cudaStream_t)stream;
  // first-layer bias of this atmosphere: b1 + U g
  float g[kCondInputs];
  condition_inputs(ctx->cfg, g);
  CUDA_TRY(cudaMemcpyAsync(S.qG, g, sizeof(g), cudaMemcpyHostToDevice, st));
  launch_cond_bias(1, S.w + S.lay.U, S.qG, S.w + S.lay.b[0], S.qbias, st);
  CUDA_TRY(cudaGetLastError());
  return surrogate_query(S, S.qbias, ctx, n, x, v, l, out, threshold, n_fallback, st);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Cloud-noise builders (include/sfsim_noise.h)
// ---------------------------------------------------------------------------

namespace {

// Device allocations of one call, freed on every return path.
struct DeviceScratch {
  std::vector<void*> ptrs;
  template <class T>
  T* get(size_t count) {
    void* p = nullptr;
    if (cudaMalloc(&p, sizeof(T) * (count ? count : 1)) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    ptrs.push_back(p);
    return static_cast<T*>(p);
  }
  ~DeviceScratch() {
    for (void* p : ptrs) cudaFree(p);
  }
};

int noise_prologue(cudaStream_t* st) {
  int dev = 0, rc = 0;
  if ((rc = current_device(&dev))) return rc;
  if ((rc = ensure_stream(dev))) return rc;
  *st = g_stream[dev];
  return 0;
}

}  // namespace

extern "C" {

int sfsim_noise_worley(int divisions, int size, const double* grid, float* out) {
  if (!grid || !out) return fail(SFSIM_ATMO_ENULL, "NULL argument");
  if (divisions < 1 || size < 1 || size % divisions != 0 || size > 1024)
    return fail(SFSIM_ATMO_EINVAL, "need 1 <= divisions, size <= 1024 and size a multiple of divisions");
  const long long nc = (long long)divisions * divisions * divisions, n = (long long)size * size * size;
  for (long long c = 0; c < 3 * nc; c++)
    if (!std::isfinite(grid[c])) return fail(SFSIM_ATMO_EINVAL, "grid points must be finite");
  std::lock_guard<std::mutex> lock(g_mutex);
  cudaStream_t st;
  int rc = noise_prologue(&st);
  if (rc) return rc;
  DeviceScratch d;
  double* g = d.get<double>(3 * nc);
  float4* local = d.get<float4>(nc);
  float* o = d.get<float>(n);
  unsigned int* mx = d.get<unsigned int>(1);
  if (!g || !local || !o || !mx) return fail(SFSIM_ATMO_ENOMEM, "Worley noise allocation failed");
  CUDA_TRY(cudaMemcpyAsync(g, grid, sizeof(double) * 3 * nc, cudaMemcpyHostToDevice, st));
  CUDA_TRY(cudaMemsetAsync(mx, 0, sizeof(unsigned int), st));
  launch_worley(divisions, size, g, local, o, mx, st);
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaMemcpyAsync(out, o, sizeof(float) * n, cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  return 0;
}

int sfsim_noise_perlin(int divisions, int size, const int* gradients, float* out) {
  if (!gradients || !out) return fail(SFSIM_ATMO_ENULL, "NULL argument");
  if (divisions < 1 || size < 1 || size > 1024) return fail(SFSIM_ATMO_EINVAL, "need divisions >= 1, 1 <= size <= 1024");
  const long long nc = (long long)divisions * divisions * divisions, n = (long long)size * size * size;
  for (long long c = 0; c < nc; c++)
    if (gradients[c] < 0 || gradients[c] > 11) return fail(SFSIM_ATMO_EINVAL, "gradient indices must be in [0, 11]");
  std::lock_guard<std::mutex> lock(g_mutex);
  cudaStream_t st;
  int rc = noise_prologue(&st);
  if (rc) return rc;
  DeviceScratch d;
  int* gi = d.get<int>(nc);
  float* o = d.get<float>(n);
  unsigned int* range = d.get<unsigned int>(2);
  if (!gi || !o || !range) return fail(SFSIM_ATMO_ENOMEM, "Perlin noise allocation failed");
  const unsigned int init[2] = {0xFFFFFFFFu, 0u};
  CUDA_TRY(cudaMemcpyAsync(gi, gradients, sizeof(int) * nc, cudaMemcpyHostToDevice, st));
  CUDA_TRY(cudaMemcpyAsync(range, init, sizeof(init), cudaMemcpyHostToDevice, st));
  launch_perlin(divisions, size, gi, o, range, st);
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaMemcpyAsync(out, o, sizeof(float) * n, cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  return 0;
}

int sfsim_noise_blue(int m, int n, const int* seed, double sigma, int* dither) {
  if (!seed || !dither) return fail(SFSIM_ATMO_ENULL, "NULL argument");
  if (m < 2 || m > 256) return fail(SFSIM_ATMO_EINVAL, "m must be in [2, 256]");
  const int total = m * m;
  if (n < 1 || n > total / 2) return fail(SFSIM_ATMO_EINVAL, "n must be in [1, m*m/2]");
  if (!(sigma > 0) || !std::isfinite(sigma)) return fail(SFSIM_ATMO_EINVAL, "sigma must be positive");
  std::vector<unsigned char> seen(total, 0);
  for (int t = 0; t < n; t++) {
    if (seed[t] < 0 || seed[t] >= total || seen[seed[t]])
      return fail(SFSIM_ATMO_EINVAL, "seed pixels must be distinct indices in [0, m*m)");
    seen[seed[t]] = 1;
  }
  // Gauss weights by |dx|, |dy| with the host's exp, as density-function
  // (bluenoise.clj:50-53) evaluates them
  const int h = m / 2 + 1;
  std::vector<double> table((size_t)h * h);
  for (int y = 0; y < h; y++)
    for (int x = 0; x < h; x++) table[(size_t)y * h + x] = std::exp(-((double)(x * x + y * y) / (2.0 * sigma * sigma)));
  std::lock_guard<std::mutex> lock(g_mutex);
  cudaStream_t st;
  int rc = noise_prologue(&st);
  if (rc) return rc;
  DeviceScratch d;
  int* sd = d.get<int>(n);
  double* tb = d.get<double>(table.size());
  double* dens = d.get<double>(total);
  double* dens0 = d.get<double>(total);
  unsigned char* mask = d.get<unsigned char>(total);
  unsigned char* work = d.get<unsigned char>(total);
  int* dith = d.get<int>(total);
  int* err = d.get<int>(1);
  if (!sd || !tb || !dens || !dens0 || !mask || !work || !dith || !err)
    return fail(SFSIM_ATMO_ENOMEM, "blue noise allocation failed");
  CUDA_TRY(cudaMemcpyAsync(sd, seed, sizeof(int) * n, cudaMemcpyHostToDevice, st));
  CUDA_TRY(cudaMemcpyAsync(tb, table.data(), sizeof(double) * table.size(), cudaMemcpyHostToDevice, st));
  CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int), st));
  if (launch_blue_noise(m, n, sd, sigma, tb, dens, dens0, mask, work, dith, err, st))
    return fail(SFSIM_ATMO_ECUDA, "blue noise launch configuration failed");
  CUDA_TRY(cudaGetLastError());
  int herr = 0;
  CUDA_TRY(cudaMemcpyAsync(dither, dith, sizeof(int) * total, cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  if (herr) return fail(SFSIM_ATMO_ECUDA, "blue noise: a wait between the cluster's CTAs timed out");
  return 0;
}

}  // extern "C"
