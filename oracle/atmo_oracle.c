/*
 * atmo_oracle.c -- FP64 CPU oracle for sfsim's atmosphere lookup-table build.
 *
 * TEST INFRASTRUCTURE ONLY.  This file restates, function by function, the
 * reference's Clojure code for the LUT build so that the GPU library can be
 * checked against it.  Nothing in the product path (the sfsim_gb300 package
 * and libsfsim_atmo.so) links, loads or calls it; only tests/, the smoke check
 * and bench.py's CPU-baseline leg do.
 *
 * Citations are paths inside wedesoft/sfsim.  The reference runs on the JVM in
 * IEEE double without fused multiply-add; this file is compiled with
 * -ffp-contract=off for the same reason.  fastmath 2.4.0 (deps.edn:10)
 * supplies only Vec3 add/sub/mult/emult/dot/mag/normalize/div/exp, restated
 * below; clojure.math maps onto the C library's exp, log, pow, sqrt, sin, cos.
 *
 * Parity pin: tests/test_oracle_kat.py checks every numeric known-answer test
 * of test/clj/sfsim/t_atmosphere.clj, t_sphere.clj, t_ray.clj and
 * t_interpolate.clj that concerns this path, and the LUT end-to-end shader
 * values of t_atmosphere.clj:629-775 through the GLSL restatement at the end
 * of this file.
 *
 * One part is not the reference's: ray_scatter_scan, the library's
 * SFSIM_ATMO_SCAN_RAYS quadrature (used only when a config sets that flag),
 * restated here so that the GPU's scan mode has a checker of its own; it is
 * pinned against a numpy restatement in tests/test_oracle_scan.py.
 */
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#include "../include/sfsim_atmo.h"
#include "atmo_oracle.h"

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* ------------------------------------------------------------------------ */
/* fastmath Vec3 (deps.edn:10)                                              */
/* ------------------------------------------------------------------------ */

typedef struct { double x, y, z; } v3;

static inline v3 V(double x, double y, double z) { v3 r = {x, y, z}; return r; }
static inline v3 vload(const double* p) { return V(p[0], p[1], p[2]); }
static inline void vstore(double* p, v3 a) { p[0] = a.x; p[1] = a.y; p[2] = a.z; }
static inline v3 add(v3 a, v3 b) { return V(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 sub(v3 a, v3 b) { return V(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 mult(v3 a, double s) { return V(a.x * s, a.y * s, a.z * s); }
static inline v3 emult(v3 a, v3 b) { return V(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline v3 vdiv(v3 a, double s) { return V(a.x / s, a.y / s, a.z / s); }
static inline double dot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline double mag(v3 a) { return sqrt(dot(a, a)); }
static inline v3 normalize(v3 a) { return vdiv(a, mag(a)); }
static inline v3 vexp(v3 a) { return V(exp(a.x), exp(a.y), exp(a.z)); }
static inline v3 neg(v3 a) { return V(-a.x, -a.y, -a.z); }
static inline v3 cross(v3 a, v3 b) {
  return V(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static const v3 ZERO = {0.0, 0.0, 0.0};

static inline double sqr(double x) { return x * x; }
/* clojure.core max/min on doubles */
static inline double dmax(double a, double b) { return a >= b ? a : b; }
static inline double dmin(double a, double b) { return a <= b ? a : b; }

/* ------------------------------------------------------------------------ */
/* Internal planet / component records                                      */
/* ------------------------------------------------------------------------ */

typedef struct {
  v3 centre;
  double radius;
  double height;
  v3 brightness;
} planet_t;

typedef struct {
  v3 base;
  double scale;
  double quotient;
  double g;
} comp_t;

static planet_t planet_from(const oracle_planet* p) {
  planet_t r;
  r.centre = vload(p->centre);
  r.radius = p->radius;
  r.height = p->height;
  r.brightness = vload(p->brightness);
  return r;
}

static comp_t comp_from(const oracle_component* c) {
  comp_t r;
  r.base = vload(c->base);
  r.scale = c->scale;
  r.quotient = c->quotient;
  r.g = c->g;
  return r;
}

/* ------------------------------------------------------------------------ */
/* util.clj:403-420 limit-quot                                               */
/* ------------------------------------------------------------------------ */

static double limit_quot4(double a, double b, double lower, double upper) {
  if (a == 0.0) return a;
  if (b < 0) return limit_quot4(-a, -b, lower, upper);
  if (a < b * upper) {
    if (a > b * lower) return a / b;
    return lower;
  }
  return upper;
}

static double limit_quot3(double a, double b, double limit) { return limit_quot4(a, b, -limit, limit); }

double oracle_limit_quot(double a, double b, double lower, double upper) {
  return limit_quot4(a, b, lower, upper);
}

/* ------------------------------------------------------------------------ */
/* sphere.clj:28-59 height, ray-sphere-intersection                         */
/* ------------------------------------------------------------------------ */

static double height_of(const planet_t* p, v3 point) { return mag(sub(point, p->centre)) - p->radius; }

typedef struct { double distance, length; } isect_t;

static isect_t ray_sphere(v3 centre, double radius, v3 origin, v3 direction) {
  v3 offset = sub(origin, centre);
  double direction_sqr = dot(direction, direction);
  /* ray-sphere-determinant, sphere.clj:34-40 */
  double discriminant = sqr(dot(direction, offset)) - direction_sqr * (dot(offset, offset) - sqr(radius));
  double middle = -(dot(direction, offset) / direction_sqr);
  isect_t r;
  if (discriminant > 0) {
    double length2 = sqrt(discriminant) / direction_sqr;
    if (middle < length2) {
      r.distance = 0.0;
      r.length = dmax(0.0, middle + length2);
    } else {
      r.distance = middle - length2;
      r.length = 2 * length2;
    }
  } else {
    r.distance = dmax(0.0, middle);
    r.length = 0.0;
  }
  return r;
}

/* ------------------------------------------------------------------------ */
/* atmosphere.clj:42-61 scattering, extinction, phase                        */
/* ------------------------------------------------------------------------ */

static v3 scattering(const comp_t* c, double h) { return mult(c->base, exp(-(h / c->scale))); }
static v3 scattering_at(const planet_t* p, const comp_t* c, v3 x) { return scattering(c, height_of(p, x)); }
static v3 extinction(const comp_t* c, double h) { return vdiv(scattering(c, h), c->quotient); }

static double phase(double g, double mu) {
  double g2 = sqr(g);
  return (3.0 * (1.0 - g2) * (1.0 + sqr(mu))) /
         (8.0 * M_PI * (2.0 + g2) * pow((1.0 + g2) - 2.0 * g * mu, 1.5));
}

/* ------------------------------------------------------------------------ */
/* atmosphere.clj:70-111 intersections, horizon, extremity                   */
/* ------------------------------------------------------------------------ */

static v3 atmosphere_intersection(const planet_t* p, v3 origin, v3 direction) {
  isect_t i = ray_sphere(p->centre, p->radius + p->height, origin, direction);
  return add(origin, mult(direction, i.distance + i.length));
}

static v3 surface_intersection(const planet_t* p, v3 origin, v3 direction) {
  isect_t i = ray_sphere(p->centre, p->radius, origin, direction);
  return add(origin, mult(direction, i.distance));
}

static int surface_point(const planet_t* p, v3 point) { return 2.0 * height_of(p, point) < p->height; }

static int is_above_horizon(const planet_t* p, v3 point, v3 direction) {
  double norm_point = mag(point);
  double sin_elevation_radius = dot(direction, point);
  double horizon_distance_sqr = sqr(norm_point) - sqr(p->radius);
  return (sin_elevation_radius >= 0) || (sqr(sin_elevation_radius) <= horizon_distance_sqr);
}

static v3 ray_extremity(const planet_t* p, v3 origin, v3 direction) {
  if (is_above_horizon(p, origin, direction)) return atmosphere_intersection(p, origin, direction);
  return surface_intersection(p, origin, direction);
}

/* ------------------------------------------------------------------------ */
/* ray.clj:19-30 integral-ray                                                */
/* ------------------------------------------------------------------------ */

typedef v3 (*point_fn)(const void* ctx, v3 p);

static v3 integral_ray(v3 origin, v3 direction, int steps, double distance, point_fn fun, const void* ctx) {
  double stepsize = distance / steps;
  double direction_len = mag(direction);
  double a = stepsize * direction_len;
  v3 acc = ZERO;
  for (int n = 0; n < steps; n++) {
    double s = (0.5 + n) * stepsize;
    v3 point = add(origin, mult(direction, s));
    acc = add(acc, mult(fun(ctx, point), a));
  }
  return acc;
}

/* ------------------------------------------------------------------------ */
/* atmosphere.clj:114-128 transmittance (both arities)                       */
/* ------------------------------------------------------------------------ */

typedef struct {
  const planet_t* planet;
  const comp_t* comps;
  int ncomp;
} ext_ctx;

static v3 overall_extinction(const void* vctx, v3 point) {
  const ext_ctx* c = (const ext_ctx*)vctx;
  if (c->ncomp == 1) return extinction(&c->comps[0], height_of(c->planet, point));
  return add(extinction(&c->comps[0], height_of(c->planet, point)),
             extinction(&c->comps[1], height_of(c->planet, point)));
}

static v3 transmittance2(const planet_t* p, const comp_t* comps, int ncomp, int steps, v3 x, v3 x0) {
  ext_ctx c = {p, comps, ncomp};
  return vexp(neg(integral_ray(x, sub(x0, x), steps, 1.0, overall_extinction, &c)));
}

static v3 transmittance3(const planet_t* p, const comp_t* comps, int ncomp, int steps, v3 x, v3 v, int above) {
  v3 x0 = above ? atmosphere_intersection(p, x, v) : surface_intersection(p, x, v);
  return transmittance2(p, comps, ncomp, steps, x, x0);
}

/* ------------------------------------------------------------------------ */
/* atmosphere.clj:131-189 E0, in-scattering, filtered sun light, J0          */
/* ------------------------------------------------------------------------ */

static v3 surface_radiance_base(const planet_t* p, const comp_t* comps, int ncomp, int steps, v3 intensity,
                                v3 x, v3 light) {
  v3 normal = normalize(sub(x, p->centre));
  return mult(emult(transmittance3(p, comps, ncomp, steps, x, light, 1), intensity), dmax(0.0, dot(normal, light)));
}

static v3 in_scattering_component(const planet_t* p, const comp_t* c, v3 x, v3 view, v3 light) {
  return mult(scattering_at(p, c, x), phase(c->g, dot(view, light)));
}

static v3 overall_in_scattering(const planet_t* p, const comp_t* comps, int ncomp, v3 x, v3 view, v3 light) {
  v3 acc = in_scattering_component(p, &comps[0], x, view, light);
  for (int i = 1; i < ncomp; i++) acc = add(acc, in_scattering_component(p, &comps[i], x, view, light));
  return acc;
}

static v3 filtered_sun_light(const planet_t* p, const comp_t* comps, int ncomp, int steps, v3 x, v3 light,
                             v3 intensity) {
  if (is_above_horizon(p, x, light)) return emult(intensity, transmittance3(p, comps, ncomp, steps, x, light, 1));
  return ZERO;
}

/* ------------------------------------------------------------------------ */
/* Function objects standing in for the reference's closures                 */
/* ------------------------------------------------------------------------ */

typedef v3 (*fn4_t)(const void* ctx, v3 x, v3 view, v3 light, int above);
typedef v3 (*fn2_t)(const void* ctx, v3 x, v3 light);

/* point-scatter-component / strength-component / point-scatter-base as J */
typedef struct {
  const planet_t* planet;
  const comp_t* comps;
  int ncomp;
  const comp_t* component;  /* NULL: point-scatter-base over all comps */
  int steps;
  v3 intensity;
  int strength;             /* 1: strength-component (no phase) */
} j0_ctx;

static v3 j0_fn(const void* vctx, v3 x, v3 view, v3 light, int above) {
  (void)above;
  const j0_ctx* c = (const j0_ctx*)vctx;
  v3 sun = filtered_sun_light(c->planet, c->comps, c->ncomp, c->steps, x, light, c->intensity);
  if (c->strength) return emult(scattering_at(c->planet, c->component, x), sun);
  if (c->component) return emult(overall_in_scattering(c->planet, c->component, 1, x, view, light), sun);
  return emult(overall_in_scattering(c->planet, c->comps, c->ncomp, x, view, light), sun);
}

/* ------------------------------------------------------------------------ */
/* atmosphere.clj:192-200 ray-scatter                                        */
/* ------------------------------------------------------------------------ */

typedef struct {
  const planet_t* planet;
  const comp_t* comps;
  int ncomp;
  int steps;
  fn4_t J;
  const void* Jctx;
  v3 x, view, light;
  int above;
} rs_ctx;

static v3 ray_scatter_integrand(const void* vctx, v3 point) {
  const rs_ctx* c = (const rs_ctx*)vctx;
  return emult(transmittance2(c->planet, c->comps, c->ncomp, c->steps, c->x, point),
               c->J(c->Jctx, point, c->view, c->light, c->above));
}

static v3 ray_scatter(const planet_t* p, const comp_t* comps, int ncomp, int steps, fn4_t J, const void* Jctx,
                      v3 x, v3 view, v3 light, int above) {
  v3 point = above ? atmosphere_intersection(p, x, view) : surface_intersection(p, x, view);
  rs_ctx c = {p, comps, ncomp, steps, J, Jctx, x, view, light, above};
  return integral_ray(x, sub(point, x), steps, 1.0, ray_scatter_integrand, &c);
}

/* The build's SFSIM_ATMO_SCAN_RAYS variant (not the reference's algorithm;
 * the check of the GPU's scan mode): the same midpoint samples p_n of the
 * view ray, with T(x, p_n) from the optical depth of the whole cells before
 * p_n (one extinction sample at each cell midpoint, which is p_m) plus the
 * half cell up to p_n sampled at its own midpoint, accumulated along the
 * ray instead of integrated anew for every p_n. */
static v3 ray_scatter_scan(const planet_t* p, const comp_t* comps, int ncomp, int steps, fn4_t J, const void* Jctx,
                           v3 x, v3 view, v3 light, int above) {
  v3 point = above ? atmosphere_intersection(p, x, view) : surface_intersection(p, x, view);
  v3 D = sub(point, x);
  ext_ctx e = {p, comps, ncomp};
  double stepsize = 1.0 / steps;
  double a = stepsize * mag(D);
  v3 depth = ZERO, acc = ZERO;
  for (int n = 0; n < steps; n++) {
    v3 pn = add(x, mult(D, (0.5 + n) * stepsize));
    v3 ph = add(x, mult(D, (0.25 + n) * stepsize));
    v3 tau = add(depth, mult(overall_extinction(&e, ph), 0.5 * a));
    acc = add(acc, mult(emult(vexp(neg(tau)), J(Jctx, pn, view, light, above)), a));
    depth = add(depth, mult(overall_extinction(&e, pn), a));
  }
  return acc;
}

/* ------------------------------------------------------------------------ */
/* sphere.clj:62-105 integrate-circle, spherical-integral; matrix.clj:207,   */
/* quaternion.clj:166 oriented-matrix / orthogonal                           */
/* ------------------------------------------------------------------------ */

typedef v3 (*dir_fn)(const void* ctx, v3 omega);

static v3 orthogonal(v3 n) {
  v3 rows[3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  /* stable sort-by |n.e|: the first row with the smallest key */
  int best = 0;
  double key = fabs(dot(n, rows[0]));
  for (int i = 1; i < 3; i++) {
    double k = fabs(dot(n, rows[i]));
    if (k < key) { key = k; best = i; }
  }
  return normalize(cross(n, rows[best]));
}

typedef struct { dir_fn fun; const void* ctx; double cos_t, sin_t; v3 n, o1, o2; } ring_ctx;

static v3 integrate_circle_ring(int steps, const ring_ctx* r) {
  double weight = (2 * M_PI) / steps;
  v3 acc = ZERO;
  for (int i = 0; i < steps; i++) {
    double phi = 2 * M_PI * ((0.5 + i) / steps);
    double x = r->cos_t, y = r->sin_t * cos(phi), z = r->sin_t * sin(phi);
    /* mulv (transpose oriented-matrix) (vec3 x y z): columns n, o1, o2 */
    v3 omega = V(r->n.x * x + r->o1.x * y + r->o2.x * z,
                 r->n.y * x + r->o1.y * y + r->o2.y * z,
                 r->n.z * x + r->o1.z * y + r->o2.z * z);
    v3 f = r->fun(r->ctx, omega);
    acc = (i == 0) ? f : add(acc, f);
  }
  return mult(acc, weight);
}

static v3 spherical_integral(int theta_steps, int phi_steps, double theta_range, v3 normal, dir_fn fun,
                             const void* ctx) {
  double delta2 = theta_range / theta_steps / 2;
  v3 o1 = orthogonal(normal);
  v3 o2 = cross(normal, o1);
  v3 acc = ZERO;
  for (int k = 0; k < theta_steps; k++) {
    double theta = theta_range * ((0.5 + k) / theta_steps);
    double factor = cos(theta - delta2) - cos(theta + delta2);
    int ringsteps = (int)ceil(sin(theta) * phi_steps);
    ring_ctx r = {fun, ctx, cos(theta), sin(theta), normal, o1, o2};
    v3 ring = mult(integrate_circle_ring(ringsteps, &r), factor);
    acc = (k == 0) ? ring : add(acc, ring);
  }
  return acc;
}

static v3 integral_half_sphere(int steps, v3 normal, dir_fn fun, const void* ctx) {
  return spherical_integral(steps >> 2, steps, M_PI / 2, normal, fun, ctx);
}

static v3 integral_sphere(int steps, v3 normal, dir_fn fun, const void* ctx) {
  return spherical_integral(steps >> 1, steps, M_PI, normal, fun, ctx);
}

/* ------------------------------------------------------------------------ */
/* atmosphere.clj:203-230 point-scatter (J), surface-radiance (E)            */
/* ------------------------------------------------------------------------ */

typedef struct {
  const planet_t* planet;
  const comp_t* comps;
  int ncomp;
  fn4_t dS;
  const void* dSctx;
  fn2_t dE;
  const void* dEctx;
  int ray_steps;
  v3 x, view, light;
} ps_ctx;

static v3 in_scatter_from_direction(const void* vctx, v3 omega) {
  const ps_ctx* c = (const ps_ctx*)vctx;
  const planet_t* p = c->planet;
  v3 point = ray_extremity(p, c->x, omega);
  int surface = surface_point(p, point);
  v3 overall = overall_in_scattering(p, c->comps, c->ncomp, c->x, c->view, omega);
  v3 ground = ZERO;
  if (surface) {
    v3 surface_brightness = emult(vdiv(p->brightness, M_PI), c->dE(c->dEctx, point, c->light));
    ground = emult(transmittance2(p, c->comps, c->ncomp, c->ray_steps, c->x, point), surface_brightness);
  }
  return emult(overall, add(c->dS(c->dSctx, c->x, omega, c->light, !surface), ground));
}

static v3 point_scatter(const planet_t* p, const comp_t* comps, int ncomp, fn4_t dS, const void* dSctx, fn2_t dE,
                        const void* dEctx, int sphere_steps, int ray_steps, v3 x, v3 view, v3 light) {
  v3 normal = normalize(sub(x, p->centre));
  ps_ctx c = {p, comps, ncomp, dS, dSctx, dE, dEctx, ray_steps, x, view, light};
  return integral_sphere(sphere_steps, normal, in_scatter_from_direction, &c);
}

typedef struct { fn4_t dS; const void* dSctx; v3 x, light, normal; } sr_ctx;

static v3 surface_radiance_integrand(const void* vctx, v3 omega) {
  const sr_ctx* c = (const sr_ctx*)vctx;
  return mult(c->dS(c->dSctx, c->x, omega, c->light, 1), dot(omega, c->normal));
}

static v3 surface_radiance(const planet_t* p, fn4_t dS, const void* dSctx, int steps, v3 x, v3 light) {
  v3 normal = normalize(sub(x, p->centre));
  sr_ctx c = {dS, dSctx, x, light, normal};
  return integral_half_sphere(steps, normal, surface_radiance_integrand, &c);
}

/* ------------------------------------------------------------------------ */
/* atmosphere.clj:233-384 table parameterisations                            */
/* ------------------------------------------------------------------------ */

static double horizon_distance(const planet_t* p, double radius) {
  return sqrt(dmax(0.0, sqr(radius) - sqr(p->radius)));
}

static double elevation_to_index(const planet_t* p, int size, v3 point, v3 direction, int above) {
  double radius = mag(point);
  double ground_radius = p->radius;
  double top_radius = ground_radius + p->height;
  double sin_elevation = dot(point, direction) / radius;
  double rho = horizon_distance(p, radius);
  double Delta = sqr(radius * sin_elevation) - sqr(rho);
  double H = sqrt(sqr(top_radius) - sqr(ground_radius));
  double idx;
  if (above)
    idx = 0.5 - limit_quot4(radius * sin_elevation - sqrt(dmax(0.0, Delta + sqr(H))), rho + rho + 2 * H, -0.5, 0.0);
  else
    idx = 0.5 + limit_quot4(radius * sin_elevation + sqrt(dmax(0.0, Delta)), rho + rho, -0.5, 0.0);
  return (size - 1) * idx;
}

static v3 index_to_elevation(const planet_t* p, int size, double radius, double index, int* above) {
  double ground_radius = p->radius;
  double top_radius = ground_radius + p->height;
  double horizon_dist = horizon_distance(p, radius);
  double H = sqrt(sqr(top_radius) - sqr(ground_radius));
  double scaled_index = index / (size - 1);
  double sin_elevation;
  if (scaled_index < 0.5 || (scaled_index == 0.5 && (2.0 * radius) < (ground_radius + top_radius))) {
    double ground_dist = horizon_dist * (1 - 2 * scaled_index);
    sin_elevation = limit_quot3(sqr(ground_radius) - sqr(radius) - sqr(ground_dist), 2 * radius * ground_dist, 1.0);
    *above = 0;
  } else {
    double sky_dist = (horizon_dist + H) * (2 * scaled_index - 1);
    sin_elevation = limit_quot4(sqr(top_radius) - sqr(radius) - sqr(sky_dist), 2 * radius * sky_dist, -1.0, 1.0);
    *above = 1;
  }
  return V(sin_elevation, sqrt(1 - sqr(sin_elevation)), 0);
}

static double height_to_index(const planet_t* p, int size, v3 point) {
  return (size - 1) * (horizon_distance(p, mag(point)) / horizon_distance(p, p->radius + p->height));
}

static v3 index_to_height(const planet_t* p, int size, double index) {
  double radius = p->radius;
  double max_horizon = sqrt(sqr(radius + p->height) - sqr(radius));
  double horizon_dist = (index / (size - 1)) * max_horizon;
  return V(sqrt(sqr(radius) + sqr(horizon_dist)), 0, 0);
}

static double sun_elevation_to_index(int size, v3 point, v3 light) {
  double sin_elevation = dot(point, light) / mag(point);
  return (size - 1) * dmax(0.0, (1 - exp(0 - (3 * sin_elevation) - 0.6)) / (1 - exp(-3.6)));
}

static double index_to_sin_sun_elevation(int size, double index) {
  return (log(1 - (index / (size - 1)) * (1 - exp(-3.6))) + 0.6) / -3;
}

static double sun_angle_to_index(int size, v3 direction, v3 light) {
  return (size - 1) * ((1 + dot(direction, light)) / 2);
}

static v3 index_to_sun_direction(int size, v3 direction, double sin_sun_elevation, double index) {
  double dot_view_sun = 2.0 * (index / (size - 1)) - 1.0;
  double max_sun_1 = sqrt(dmax(0.0, 1.0 - sqr(sin_sun_elevation)));
  double sun_1 = limit_quot3(dot_view_sun - direction.x * sin_sun_elevation, direction.y, max_sun_1);
  double sun_2 = sqrt(dmax(0.0, 1.0 - sqr(sun_1) - sqr(sin_sun_elevation)));
  return V(sin_sun_elevation, sun_1, sun_2);
}

/* ------------------------------------------------------------------------ */
/* Spaces: transmittance (:291-319), surface radiance (:335-365),           */
/* ray scatter = point scatter (:387-422)                                    */
/* ------------------------------------------------------------------------ */

static void transmittance_forward(const planet_t* p, const int* shape, v3 point, v3 direction, int above, double* c) {
  c[0] = height_to_index(p, shape[0], point);
  c[1] = elevation_to_index(p, shape[1], point, direction, above);
}

static void transmittance_backward(const planet_t* p, const int* shape, const double* idx, v3* point, v3* direction,
                                   int* above) {
  *point = index_to_height(p, shape[0], idx[0]);
  *direction = index_to_elevation(p, shape[1], point->x, idx[1], above);
}

static void surface_radiance_forward(const planet_t* p, const int* shape, v3 point, v3 light, double* c) {
  c[0] = height_to_index(p, shape[0], point);
  c[1] = sun_elevation_to_index(shape[1], point, light);
}

static void surface_radiance_backward(const planet_t* p, const int* shape, const double* idx, v3* point, v3* light) {
  *point = index_to_height(p, shape[0], idx[0]);
  double sin_sun = index_to_sin_sun_elevation(shape[1], idx[1]);
  double cos_sun = sqrt(dmax(0.0, 1 - sqr(sin_sun)));
  *light = V(sin_sun, cos_sun, 0);
}

static void ray_scatter_forward(const planet_t* p, const int* shape, v3 point, v3 direction, v3 light, int above,
                                double* c) {
  c[0] = height_to_index(p, shape[0], point);
  c[1] = elevation_to_index(p, shape[1], point, direction, above);
  c[2] = sun_elevation_to_index(shape[2], point, light);
  c[3] = sun_angle_to_index(shape[3], direction, light);
}

static void ray_scatter_backward(const planet_t* p, const int* shape, const double* idx, v3* point, v3* direction,
                                 v3* light, int* above) {
  *point = index_to_height(p, shape[0], idx[0]);
  *direction = index_to_elevation(p, shape[1], point->x, idx[1], above);
  double sin_sun = index_to_sin_sun_elevation(shape[2], idx[2]);
  *light = index_to_sun_direction(shape[3], *direction, sin_sun, idx[3]);
}

/* ------------------------------------------------------------------------ */
/* interpolate.clj:75-104 clip, mix, interpolate-value                       */
/* ------------------------------------------------------------------------ */

typedef struct {
  int ndim;
  int shape[4];
  long stride[4];  /* in vec3 units */
  double* data;    /* [...][3] */
} table_t;

static void table_init(table_t* t, int ndim, const int* shape, double* data) {
  t->ndim = ndim;
  for (int i = 0; i < ndim; i++) t->shape[i] = shape[i];
  long s = 1;
  for (int i = ndim - 1; i >= 0; i--) { t->stride[i] = s; s *= shape[i]; }
  t->data = data;
}

static long table_cells(const table_t* t) {
  long n = 1;
  for (int i = 0; i < t->ndim; i++) n *= t->shape[i];
  return n;
}

static inline double clip(double value, int size) { return dmin(dmax(value, 0.0), (double)(size - 1)); }

static v3 mix(v3 a, v3 b, double s) { return add(mult(a, 1 - s), mult(b, s)); }

static v3 interpolate_rec(const table_t* t, int dim, long offset, const double* c) {
  if (dim == t->ndim) return vload(t->data + 3 * offset);
  int size = t->shape[dim];
  double i = clip(c[dim], size);
  double u = floor(i);
  double v = clip(u + 1, size);
  double s = i - u;
  v3 a = interpolate_rec(t, dim + 1, offset + (long)u * t->stride[dim], c);
  v3 b = interpolate_rec(t, dim + 1, offset + (long)v * t->stride[dim], c);
  return mix(a, b, s);
}

static v3 interpolate_value(const table_t* t, const double* c) { return interpolate_rec(t, 0, 0, c); }

/* ------------------------------------------------------------------------ */
/* Interpolated functions over the spaces (interpolate-function)            */
/* ------------------------------------------------------------------------ */

typedef struct {
  const planet_t* planet;
  const int* shape;
  const table_t* a;      /* required */
  const table_t* b;      /* optional second table */
  double b_g;            /* b is multiplied by phase(b_g, view.light) when b_phase */
  int b_phase;
} interp4_ctx;

/* dS of the first iteration (atmosphere_lut.clj:79-84) when b is the Mie
 * strength table with its phase; a plain interpolated table otherwise. */
static v3 interp4_fn(const void* vctx, v3 x, v3 view, v3 light, int above) {
  const interp4_ctx* c = (const interp4_ctx*)vctx;
  double co[4];
  ray_scatter_forward(c->planet, c->shape, x, view, light, above, co);
  v3 r = interpolate_value(c->a, co);
  if (c->b) {
    v3 rb = interpolate_value(c->b, co);
    if (c->b_phase) rb = mult(rb, phase(c->b_g, dot(view, light)));
    r = add(r, rb);
  }
  return r;
}

typedef struct {
  const planet_t* planet;
  const int* shape;
  const table_t* a;  /* NULL: constantly zero */
  const table_t* b;  /* optional */
} interp2_ctx;

static v3 interp2_fn(const void* vctx, v3 x, v3 light) {
  const interp2_ctx* c = (const interp2_ctx*)vctx;
  double co[2];
  surface_radiance_forward(c->planet, c->shape, x, light, co);
  v3 r = c->a ? interpolate_value(c->a, co) : ZERO;
  if (c->b) r = add(r, interpolate_value(c->b, co));
  return r;
}

/* ------------------------------------------------------------------------ */
/* interpolate.clj:54-72 make-lookup-table (pmap over dimension 0)           */
/* ------------------------------------------------------------------------ */

typedef void (*node_fn)(const void* ctx, const int* idx, double* out);

typedef struct {
  const table_t* t;
  node_fn fun;
  const void* ctx;
  int next;
  pthread_mutex_t lock;
} mlt_job;

static void fill_slice(const table_t* t, node_fn fun, const void* ctx, int i0) {
  int idx[4] = {i0, 0, 0, 0};
  long inner = t->stride[0];
  for (long n = 0; n < inner; n++) {
    long r = n;
    for (int d = t->ndim - 1; d >= 1; d--) { idx[d] = (int)(r % t->shape[d]); r /= t->shape[d]; }
    fun(ctx, idx, t->data + 3 * ((long)i0 * inner + n));
  }
}

static void* mlt_worker(void* arg) {
  mlt_job* j = (mlt_job*)arg;
  for (;;) {
    pthread_mutex_lock(&j->lock);
    int i0 = j->next++;
    pthread_mutex_unlock(&j->lock);
    if (i0 >= j->t->shape[0]) break;
    fill_slice(j->t, j->fun, j->ctx, i0);
  }
  return NULL;
}

static int g_threads = 1;

static void make_lookup_table(const table_t* t, node_fn fun, const void* ctx) {
  int nthreads = g_threads < t->shape[0] ? g_threads : t->shape[0];
  if (nthreads <= 1) {
    for (int i = 0; i < t->shape[0]; i++) fill_slice(t, fun, ctx, i);
    return;
  }
  mlt_job job;
  job.t = t; job.fun = fun; job.ctx = ctx; job.next = 0;
  pthread_mutex_init(&job.lock, NULL);
  pthread_t th[256];
  if (nthreads > 256) nthreads = 256;
  for (int i = 0; i < nthreads; i++) pthread_create(&th[i], NULL, mlt_worker, &job);
  for (int i = 0; i < nthreads; i++) pthread_join(th[i], NULL);
  pthread_mutex_destroy(&job.lock);
}

/* ------------------------------------------------------------------------ */
/* The LUT driver, atmosphere_lut.clj:43-105                                 */
/* ------------------------------------------------------------------------ */

typedef struct {
  planet_t planet;
  comp_t comps[2];   /* scatter = [mie rayleigh], atmosphere_lut.clj:63 */
  v3 intensity;
  int tshape[2], eshape[2], sshape[4];
  int ray_steps, sphere_steps, iterations;
  int scan_rays;     /* SFSIM_ATMO_SCAN_RAYS */
} build_t;

static void build_from_config(const sfsim_atmo_config* cfg, build_t* b) {
  b->planet.centre = ZERO;
  b->planet.radius = cfg->radius;
  b->planet.height = cfg->height;
  b->planet.brightness = vload(cfg->brightness);
  b->comps[0].base = vload(cfg->mie.scatter_base);
  b->comps[0].scale = cfg->mie.scatter_scale;
  b->comps[0].quotient = cfg->mie.scatter_quotient;
  b->comps[0].g = cfg->mie.scatter_g;
  b->comps[1].base = vload(cfg->rayleigh.scatter_base);
  b->comps[1].scale = cfg->rayleigh.scatter_scale;
  b->comps[1].quotient = cfg->rayleigh.scatter_quotient;
  b->comps[1].g = cfg->rayleigh.scatter_g;
  b->intensity = vload(cfg->intensity);
  for (int i = 0; i < 2; i++) b->tshape[i] = cfg->transmittance_shape[i];
  for (int i = 0; i < 2; i++) b->eshape[i] = cfg->surface_radiance_shape[i];
  for (int i = 0; i < 4; i++) b->sshape[i] = cfg->ray_scatter_shape[i];
  b->ray_steps = cfg->ray_steps;
  b->sphere_steps = cfg->sphere_steps;
  b->iterations = cfg->iterations;
  b->scan_rays = (cfg->flags & SFSIM_ATMO_SCAN_RAYS) != 0;
}

/* Node functions for make-lookup-table */

static void node_transmittance(const void* vctx, const int* idx, double* out) {
  const build_t* b = (const build_t*)vctx;
  double di[2] = {idx[0], idx[1]};
  v3 point, dir;
  int above;
  transmittance_backward(&b->planet, b->tshape, di, &point, &dir, &above);
  vstore(out, transmittance3(&b->planet, b->comps, 2, b->ray_steps, point, dir, above));
}

static void node_surface_base(const void* vctx, const int* idx, double* out) {
  const build_t* b = (const build_t*)vctx;
  double di[2] = {idx[0], idx[1]};
  v3 point, light;
  surface_radiance_backward(&b->planet, b->eshape, di, &point, &light);
  vstore(out, surface_radiance_base(&b->planet, b->comps, 2, b->ray_steps, b->intensity, point, light));
}

typedef struct { const build_t* b; fn4_t J; const void* Jctx; } rs_node_ctx;

static void node_ray_scatter(const void* vctx, const int* idx, double* out) {
  const rs_node_ctx* c = (const rs_node_ctx*)vctx;
  const build_t* b = c->b;
  double di[4] = {idx[0], idx[1], idx[2], idx[3]};
  v3 point, dir, light;
  int above;
  ray_scatter_backward(&b->planet, b->sshape, di, &point, &dir, &light, &above);
  vstore(out, (b->scan_rays ? ray_scatter_scan : ray_scatter)(&b->planet, b->comps, 2, b->ray_steps, c->J, c->Jctx,
                                                               point, dir, light, above));
}

typedef struct { const build_t* b; fn4_t dS; const void* dSctx; fn2_t dE; const void* dEctx; } ps_node_ctx;

static void node_point_scatter(const void* vctx, const int* idx, double* out) {
  const ps_node_ctx* c = (const ps_node_ctx*)vctx;
  const build_t* b = c->b;
  double di[4] = {idx[0], idx[1], idx[2], idx[3]};
  v3 point, dir, light;
  int above;
  ray_scatter_backward(&b->planet, b->sshape, di, &point, &dir, &light, &above);
  vstore(out, point_scatter(&b->planet, b->comps, 2, c->dS, c->dSctx, c->dE, c->dEctx, b->sphere_steps,
                            b->ray_steps, point, dir, light));
}

typedef struct { const build_t* b; fn4_t dS; const void* dSctx; } sr_node_ctx;

static void node_surface_radiance(const void* vctx, const int* idx, double* out) {
  const sr_node_ctx* c = (const sr_node_ctx*)vctx;
  const build_t* b = c->b;
  double di[2] = {idx[0], idx[1]};
  v3 point, light;
  surface_radiance_backward(&b->planet, b->eshape, di, &point, &light);
  /* (partial surface-radiance earth @dS ray-steps): the sphere steps are the ray steps */
  vstore(out, surface_radiance(&b->planet, c->dS, c->dSctx, b->ray_steps, point, light));
}

/* Re-tabulation of an interpolated function at its own nodes */

typedef struct { const build_t* b; const interp4_ctx* f; } remap4_ctx;

static void node_remap4(const void* vctx, const int* idx, double* out) {
  const remap4_ctx* c = (const remap4_ctx*)vctx;
  double di[4] = {idx[0], idx[1], idx[2], idx[3]};
  v3 point, dir, light;
  int above;
  ray_scatter_backward(&c->b->planet, c->b->sshape, di, &point, &dir, &light, &above);
  vstore(out, interp4_fn(c->f, point, dir, light, above));
}

typedef struct { const build_t* b; const interp2_ctx* f; } remap2_ctx;

static void node_remap2(const void* vctx, const int* idx, double* out) {
  const remap2_ctx* c = (const remap2_ctx*)vctx;
  double di[2] = {idx[0], idx[1]};
  v3 point, light;
  surface_radiance_backward(&c->b->planet, c->b->eshape, di, &point, &light);
  vstore(out, interp2_fn(c->f, point, light));
}

typedef struct { const build_t* b; const table_t* t; } remapT_ctx;

static void node_remapT(const void* vctx, const int* idx, double* out) {
  const remapT_ctx* c = (const remapT_ctx*)vctx;
  double di[2] = {idx[0], idx[1]};
  v3 point, dir;
  int above;
  transmittance_backward(&c->b->planet, c->b->tshape, di, &point, &dir, &above);
  double co[2];
  transmittance_forward(&c->b->planet, c->b->tshape, point, dir, above, co);
  vstore(out, interpolate_value(c->t, co));
}

/* image.clj:299-312 convert-4d-to-2d + matrix.clj:130 pack-matrices */
static void pack_4d(const table_t* t, double* out) {
  int n0 = t->shape[0], n1 = t->shape[1], n2 = t->shape[2], n3 = t->shape[3];
  for (int i = 0; i < n0; i++)
    for (int j = 0; j < n1; j++)
      for (int k = 0; k < n2; k++)
        for (int a = 0; a < n3; a++) {
          long src = (((long)i * n1 + j) * n2 + k) * n3 + a;
          long row = (long)i * n2 + k, col = (long)j * n3 + a;
          long dst = row * ((long)n1 * n3) + col;
          for (int ch = 0; ch < 3; ch++) out[3 * dst + ch] = t->data[3 * src + ch];
        }
}

static double* alloc_table(table_t* t, int ndim, const int* shape) {
  long n = 1;
  for (int i = 0; i < ndim; i++) n *= shape[i];
  double* d = (double*)calloc((size_t)n * 3, sizeof(double));
  table_init(t, ndim, shape, d);
  return d;
}

int oracle_build(const sfsim_atmo_config* cfg, int nthreads, double* T_out, double* E_out, double* S_out,
                 double* M_out, const oracle_intermediates* inter) {
  build_t b;
  build_from_config(cfg, &b);
  g_threads = nthreads > 0 ? nthreads : 1;
  const planet_t* P = &b.planet;

  table_t T, dE, S1R, M, J, dS, dEn, E, S, Etmp, Stmp;
  alloc_table(&T, 2, b.tshape);
  alloc_table(&dE, 2, b.eshape);
  alloc_table(&S1R, 4, b.sshape);
  alloc_table(&M, 4, b.sshape);
  alloc_table(&J, 4, b.sshape);
  alloc_table(&dS, 4, b.sshape);
  alloc_table(&dEn, 2, b.eshape);
  alloc_table(&E, 2, b.eshape);
  alloc_table(&S, 4, b.sshape);
  alloc_table(&Etmp, 2, b.eshape);
  alloc_table(&Stmp, 4, b.sshape);
  long n4 = table_cells(&S1R), n2e = table_cells(&dE), n2t = table_cells(&T);

  /* T, dE0 (atmosphere_lut.clj:74-75) */
  make_lookup_table(&T, node_transmittance, &b);
  make_lookup_table(&dE, node_surface_base, &b);
  /* first-order Rayleigh and Mie strength (atmosphere_lut.clj:68-78) */
  j0_ctx jr = {P, b.comps, 2, &b.comps[1], b.ray_steps, b.intensity, 0};
  j0_ctx jm = {P, b.comps, 2, &b.comps[0], b.ray_steps, b.intensity, 1};
  rs_node_ctx rr = {&b, j0_fn, &jr};
  rs_node_ctx rm = {&b, j0_fn, &jm};
  make_lookup_table(&S1R, node_ray_scatter, &rr);
  make_lookup_table(&M, node_ray_scatter, &rm);
  if (inter) {
    if (inter->transmittance_nodes) memcpy(inter->transmittance_nodes, T.data, sizeof(double) * 3 * n2t);
    if (inter->surface_base) memcpy(inter->surface_base, dE.data, sizeof(double) * 3 * n2e);
    if (inter->rayleigh_first) memcpy(inter->rayleigh_first, S1R.data, sizeof(double) * 3 * n4);
    if (inter->mie_first) memcpy(inter->mie_first, M.data, sizeof(double) * 3 * n4);
  }

  /* dS = S1R + M * phase(mie, v.l)  (atmosphere_lut.clj:79-84); S = S1R; E = 0 */
  interp4_ctx dS_fn = {P, b.sshape, &S1R, &M, b.comps[0].g, 1};
  interp2_ctx dE_fn = {P, b.eshape, &dE, NULL};
  interp4_ctx S_fn = {P, b.sshape, &S1R, NULL, 0.0, 0};
  table_t* S_cur = &S1R;  /* table behind S_fn */
  table_t* E_cur = NULL;  /* NULL: E = constantly 0 */
  table_t* dS_cur = NULL; /* NULL: first iteration's dS_fn */
  table_t* dE_cur = &dE;

  for (int it = 0; it < b.iterations; it++) {
    /* J from the current dS and dE (:88, :90) */
    ps_node_ctx pc = {&b, interp4_fn, &dS_fn, interp2_fn, &dE_fn};
    make_lookup_table(&J, node_point_scatter, &pc);
    /* new dE from the old dS (:89, :92) */
    sr_node_ctx sc = {&b, interp4_fn, &dS_fn};
    make_lookup_table(&dEn, node_surface_radiance, &sc);
    /* new dS from J (:91, :93) */
    interp4_ctx J_fn = {P, b.sshape, &J, NULL, 0.0, 0};
    rs_node_ctx rj = {&b, interp4_fn, &J_fn};
    make_lookup_table(&dS, node_ray_scatter, &rj);
    if (inter) {
      if (inter->point_scatter) memcpy(inter->point_scatter + 3 * n4 * it, J.data, sizeof(double) * 3 * n4);
      if (inter->surface_delta) memcpy(inter->surface_delta + 3 * n2e * it, dEn.data, sizeof(double) * 3 * n2e);
      if (inter->ray_scatter_delta) memcpy(inter->ray_scatter_delta + 3 * n4 * it, dS.data, sizeof(double) * 3 * n4);
    }
    /* swap in the new dE, dS */
    memcpy(dE.data, dEn.data, sizeof(double) * 3 * n2e);
    dE_cur = &dE;
    dE_fn.a = dE_cur;
    dS_cur = &dS;
    dS_fn.a = dS_cur; dS_fn.b = NULL; dS_fn.b_phase = 0;
    /* E = table(E + dE) (:94-95) */
    interp2_ctx Esum = {P, b.eshape, E_cur, dE_cur};
    remap2_ctx re = {&b, &Esum};
    make_lookup_table(&Etmp, node_remap2, &re);
    memcpy(E.data, Etmp.data, sizeof(double) * 3 * n2e);
    E_cur = &E;
    /* S = table(S + dS) (:96-97) */
    interp4_ctx Ssum = {P, b.sshape, S_cur, dS_cur, 0.0, 0};
    remap4_ctx rs = {&b, &Ssum};
    make_lookup_table(&Stmp, node_remap4, &rs);
    memcpy(S.data, Stmp.data, sizeof(double) * 3 * n4);
    S_cur = &S;
    S_fn.a = S_cur;
  }
  (void)S_fn;

  /* final make-lookup-table of T, E, S and the Mie strength (:98-101) */
  table_t Tout, Eout, Sout, Mout;
  alloc_table(&Tout, 2, b.tshape);
  alloc_table(&Eout, 2, b.eshape);
  alloc_table(&Sout, 4, b.sshape);
  alloc_table(&Mout, 4, b.sshape);
  remapT_ctx rt = {&b, &T};
  make_lookup_table(&Tout, node_remapT, &rt);
  interp2_ctx Efin = {P, b.eshape, E_cur, NULL};
  remap2_ctx ref = {&b, &Efin};
  make_lookup_table(&Eout, node_remap2, &ref);
  interp4_ctx Sfin = {P, b.sshape, S_cur, NULL, 0.0, 0};
  remap4_ctx rsf = {&b, &Sfin};
  make_lookup_table(&Sout, node_remap4, &rsf);
  interp4_ctx Mfin = {P, b.sshape, &M, NULL, 0.0, 0};
  remap4_ctx rmf = {&b, &Mfin};
  make_lookup_table(&Mout, node_remap4, &rmf);

  /* pack-matrices / convert-4d-to-2d layout (:102-105) */
  if (T_out) memcpy(T_out, Tout.data, sizeof(double) * 3 * n2t);
  if (E_out) memcpy(E_out, Eout.data, sizeof(double) * 3 * n2e);
  if (S_out) pack_4d(&Sout, S_out);
  if (M_out) pack_4d(&Mout, M_out);

  table_t* all[] = {&T, &dE, &S1R, &M, &J, &dS, &dEn, &E, &S, &Etmp, &Stmp, &Tout, &Eout, &Sout, &Mout};
  for (size_t i = 0; i < sizeof(all) / sizeof(all[0]); i++) free(all[i]->data);
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Per-node evaluation against supplied tables (size-independent checks)    */
/* ------------------------------------------------------------------------ */

static void tab4(table_t* t, const build_t* b, const double* data) { table_init(t, 4, b->sshape, (double*)data); }
static void tab2e(table_t* t, const build_t* b, const double* data) { table_init(t, 2, b->eshape, (double*)data); }

void oracle_transmittance_node(const sfsim_atmo_config* cfg, int i, int j, double* out) {
  build_t b; build_from_config(cfg, &b);
  int idx[2] = {i, j};
  node_transmittance(&b, idx, out);
}

void oracle_surface_base_node(const sfsim_atmo_config* cfg, int i, int k, double* out) {
  build_t b; build_from_config(cfg, &b);
  int idx[2] = {i, k};
  node_surface_base(&b, idx, out);
}

void oracle_first_order_node(const sfsim_atmo_config* cfg, int i, int j, int k, int a, double* rayleigh,
                             double* mie) {
  build_t b; build_from_config(cfg, &b);
  int idx[4] = {i, j, k, a};
  j0_ctx jr = {&b.planet, b.comps, 2, &b.comps[1], b.ray_steps, b.intensity, 0};
  j0_ctx jm = {&b.planet, b.comps, 2, &b.comps[0], b.ray_steps, b.intensity, 1};
  rs_node_ctx rr = {&b, j0_fn, &jr};
  rs_node_ctx rm = {&b, j0_fn, &jm};
  if (rayleigh) node_ray_scatter(&rr, idx, rayleigh);
  if (mie) node_ray_scatter(&rm, idx, mie);
}

void oracle_point_scatter_node(const sfsim_atmo_config* cfg, const double* dS, const double* mie_first,
                               const double* dE, int i, int j, int k, int a, double* out) {
  build_t b; build_from_config(cfg, &b);
  table_t tS, tM, tE;
  tab4(&tS, &b, dS);
  tab2e(&tE, &b, dE);
  interp4_ctx dS_fn = {&b.planet, b.sshape, &tS, NULL, 0.0, 0};
  if (mie_first) {
    tab4(&tM, &b, mie_first);
    dS_fn.b = &tM; dS_fn.b_g = b.comps[0].g; dS_fn.b_phase = 1;
  }
  interp2_ctx dE_fn = {&b.planet, b.eshape, &tE, NULL};
  ps_node_ctx pc = {&b, interp4_fn, &dS_fn, interp2_fn, &dE_fn};
  int idx[4] = {i, j, k, a};
  node_point_scatter(&pc, idx, out);
}

void oracle_ray_scatter_node(const sfsim_atmo_config* cfg, const double* J, int i, int j, int k, int a,
                             double* out) {
  build_t b; build_from_config(cfg, &b);
  table_t tJ;
  tab4(&tJ, &b, J);
  interp4_ctx J_fn = {&b.planet, b.sshape, &tJ, NULL, 0.0, 0};
  rs_node_ctx rj = {&b, interp4_fn, &J_fn};
  int idx[4] = {i, j, k, a};
  node_ray_scatter(&rj, idx, out);
}

void oracle_surface_radiance_node(const sfsim_atmo_config* cfg, const double* dS, const double* mie_first, int i,
                                  int k, double* out) {
  build_t b; build_from_config(cfg, &b);
  table_t tS, tM;
  tab4(&tS, &b, dS);
  interp4_ctx dS_fn = {&b.planet, b.sshape, &tS, NULL, 0.0, 0};
  if (mie_first) {
    tab4(&tM, &b, mie_first);
    dS_fn.b = &tM; dS_fn.b_g = b.comps[0].g; dS_fn.b_phase = 1;
  }
  sr_node_ctx sc = {&b, interp4_fn, &dS_fn};
  int idx[2] = {i, k};
  node_surface_radiance(&sc, idx, out);
}

void oracle_remap4_node(const sfsim_atmo_config* cfg, const double* table, int i, int j, int k, int a,
                        double* out) {
  build_t b; build_from_config(cfg, &b);
  table_t t;
  tab4(&t, &b, table);
  interp4_ctx f = {&b.planet, b.sshape, &t, NULL, 0.0, 0};
  remap4_ctx rc = {&b, &f};
  int idx[4] = {i, j, k, a};
  node_remap4(&rc, idx, out);
}

/* Rendered in-scatter S + M phase(mie, v.l) at an arbitrary (x, v, l), the
 * quantity the 4-D tables sample (ray-scatter-outer.glsl:18-20): the first
 * order by ray-scatter with point-scatter-component / strength-component
 * (atmosphere_lut.clj:68-78) and the higher orders by ray-scatter of the
 * point-scatter table summed over the iterations (NULL: first order only).
 * The table half is chosen by is-above-horizon?. */
void oracle_rendered_inscatter(const sfsim_atmo_config* cfg, const double* Jsum, const double* x, const double* v,
                               const double* l, double* out) {
  build_t b; build_from_config(cfg, &b);
  v3 X = vload(x), Vd = vload(v), L = vload(l);
  int above = is_above_horizon(&b.planet, X, Vd);
  j0_ctx jr = {&b.planet, b.comps, 2, &b.comps[1], b.ray_steps, b.intensity, 0};
  j0_ctx jm = {&b.planet, b.comps, 2, &b.comps[0], b.ray_steps, b.intensity, 1};
  v3 s1 = ray_scatter(&b.planet, b.comps, 2, b.ray_steps, j0_fn, &jr, X, Vd, L, above);
  v3 m = ray_scatter(&b.planet, b.comps, 2, b.ray_steps, j0_fn, &jm, X, Vd, L, above);
  v3 r = add(s1, mult(m, phase(b.comps[0].g, dot(Vd, L))));
  if (Jsum) {
    table_t t;
    tab4(&t, &b, Jsum);
    interp4_ctx f = {&b.planet, b.sshape, &t, NULL, 0.0, 0};
    r = add(r, ray_scatter(&b.planet, b.comps, 2, b.ray_steps, interp4_fn, &f, X, Vd, L, above));
  }
  vstore(out, r);
}

/* ------------------------------------------------------------------------ */
/* Exported unit functions for the known-answer tests                        */
/* ------------------------------------------------------------------------ */

double oracle_phase(double g, double mu) { return phase(g, mu); }

void oracle_scattering(const oracle_component* c, double h, double* out) {
  comp_t cc = comp_from(c);
  vstore(out, scattering(&cc, h));
}

void oracle_extinction(const oracle_component* c, double h, double* out) {
  comp_t cc = comp_from(c);
  vstore(out, extinction(&cc, h));
}

double oracle_height(const oracle_planet* p, const double* point) {
  planet_t pp = planet_from(p);
  return height_of(&pp, vload(point));
}

void oracle_ray_sphere_intersection(const double* centre, double radius, const double* origin,
                                    const double* direction, double* out) {
  isect_t i = ray_sphere(vload(centre), radius, vload(origin), vload(direction));
  out[0] = i.distance;
  out[1] = i.length;
}

void oracle_atmosphere_intersection(const oracle_planet* p, const double* origin, const double* direction,
                                    double* out) {
  planet_t pp = planet_from(p);
  vstore(out, atmosphere_intersection(&pp, vload(origin), vload(direction)));
}

void oracle_surface_intersection(const oracle_planet* p, const double* origin, const double* direction,
                                 double* out) {
  planet_t pp = planet_from(p);
  vstore(out, surface_intersection(&pp, vload(origin), vload(direction)));
}

int oracle_surface_point(const oracle_planet* p, const double* point) {
  planet_t pp = planet_from(p);
  return surface_point(&pp, vload(point));
}

int oracle_is_above_horizon(const oracle_planet* p, const double* point, const double* direction) {
  planet_t pp = planet_from(p);
  return is_above_horizon(&pp, vload(point), vload(direction));
}

void oracle_ray_extremity(const oracle_planet* p, const double* origin, const double* direction, double* out) {
  planet_t pp = planet_from(p);
  vstore(out, ray_extremity(&pp, vload(origin), vload(direction)));
}

void oracle_transmittance(const oracle_planet* p, const oracle_component* comps, int ncomp, int steps,
                          const double* x, const double* x0, double* out) {
  planet_t pp = planet_from(p);
  comp_t cc[2];
  for (int i = 0; i < ncomp && i < 2; i++) cc[i] = comp_from(&comps[i]);
  vstore(out, transmittance2(&pp, cc, ncomp, steps, vload(x), vload(x0)));
}

void oracle_transmittance_dir(const oracle_planet* p, const oracle_component* comps, int ncomp, int steps,
                              const double* x, const double* v, int above, double* out) {
  planet_t pp = planet_from(p);
  comp_t cc[2];
  for (int i = 0; i < ncomp && i < 2; i++) cc[i] = comp_from(&comps[i]);
  vstore(out, transmittance3(&pp, cc, ncomp, steps, vload(x), vload(v), above));
}

void oracle_surface_radiance_base(const oracle_planet* p, const oracle_component* comps, int ncomp, int steps,
                                  const double* intensity, const double* x, const double* light, double* out) {
  planet_t pp = planet_from(p);
  comp_t cc[2];
  for (int i = 0; i < ncomp && i < 2; i++) cc[i] = comp_from(&comps[i]);
  vstore(out, surface_radiance_base(&pp, cc, ncomp, steps, vload(intensity), vload(x), vload(light)));
}

/* kind 0: point-scatter-component, 1: strength-component, 2: point-scatter-base */
void oracle_single_scatter(const oracle_planet* p, const oracle_component* comps, int ncomp, int component, int kind,
                           int steps, const double* intensity, const double* x, const double* v, const double* l,
                           double* out) {
  planet_t pp = planet_from(p);
  comp_t cc[2];
  for (int i = 0; i < ncomp && i < 2; i++) cc[i] = comp_from(&comps[i]);
  j0_ctx j = {&pp, cc, ncomp, kind == 2 ? NULL : &cc[component], steps, vload(intensity), kind == 1};
  vstore(out, j0_fn(&j, vload(x), vload(v), vload(l), 1));
}

/* ray-scatter with J = point-scatter-component of `component` (t_atmosphere.clj:585) */
void oracle_ray_scatter_single(const oracle_planet* p, const oracle_component* comps, int ncomp, int component,
                               int kind, int steps, const double* intensity, const double* x, const double* v,
                               const double* l, int above, double* out) {
  planet_t pp = planet_from(p);
  comp_t cc[2];
  for (int i = 0; i < ncomp && i < 2; i++) cc[i] = comp_from(&comps[i]);
  j0_ctx j = {&pp, cc, ncomp, kind == 2 ? NULL : &cc[component], steps, vload(intensity), kind == 1};
  vstore(out, ray_scatter(&pp, cc, ncomp, steps, j0_fn, &j, vload(x), vload(v), vload(l), above));
}

/* constant J (t_atmosphere.clj:249-282) */
typedef struct { v3 value; } const_ctx;
static v3 const4(const void* vctx, v3 x, v3 v, v3 l, int above) {
  (void)x; (void)v; (void)l; (void)above;
  return ((const const_ctx*)vctx)->value;
}
static v3 const2(const void* vctx, v3 x, v3 l) {
  (void)x; (void)l;
  return ((const const_ctx*)vctx)->value;
}

void oracle_ray_scatter_const(const oracle_planet* p, const oracle_component* comps, int ncomp, int steps,
                              const double* J, const double* x, const double* v, const double* l, int above,
                              double* out) {
  planet_t pp = planet_from(p);
  comp_t cc[2];
  for (int i = 0; i < ncomp && i < 2; i++) cc[i] = comp_from(&comps[i]);
  const_ctx c = {vload(J)};
  vstore(out, ray_scatter(&pp, cc, ncomp, steps, const4, &c, vload(x), vload(v), vload(l), above));
}

void oracle_ray_scatter_scan_const(const oracle_planet* p, const oracle_component* comps, int ncomp, int steps,
                                   const double* J, const double* x, const double* v, const double* l, int above,
                                   double* out) {
  planet_t pp = planet_from(p);
  comp_t cc[2];
  for (int i = 0; i < ncomp && i < 2; i++) cc[i] = comp_from(&comps[i]);
  const_ctx c = {vload(J)};
  vstore(out, ray_scatter_scan(&pp, cc, ncomp, steps, const4, &c, vload(x), vload(v), vload(l), above));
}

void oracle_point_scatter_const(const oracle_planet* p, const oracle_component* comps, int ncomp,
                                const double* dS, const double* dE, int sphere_steps, int ray_steps,
                                const double* x, const double* v, const double* l, double* out) {
  planet_t pp = planet_from(p);
  comp_t cc[2];
  for (int i = 0; i < ncomp && i < 2; i++) cc[i] = comp_from(&comps[i]);
  const_ctx cs = {vload(dS)}, ce = {vload(dE)};
  vstore(out, point_scatter(&pp, cc, ncomp, const4, &cs, const2, &ce, sphere_steps, ray_steps, vload(x), vload(v),
                            vload(l)));
}

void oracle_surface_radiance_const(const oracle_planet* p, const double* dS, int steps, const double* x,
                                   const double* l, double* out) {
  planet_t pp = planet_from(p);
  const_ctx cs = {vload(dS)};
  vstore(out, surface_radiance(&pp, const4, &cs, steps, vload(x), vload(l)));
}

/* integral-ray / integral-sphere of simple test integrands (t_ray.clj, t_sphere.clj).
 * kind 0: constant c; kind 1: (x0, x0, 0) for rays, (1, v1, v2) style for spheres
 * selected by `select`: result[i] = c[i] when select[i] < 0 else omega[select[i]]. */
typedef struct { v3 c; int sel[3]; } sel_ctx;
static v3 sel_fn(const void* vctx, v3 p) {
  const sel_ctx* s = (const sel_ctx*)vctx;
  double q[3] = {p.x, p.y, p.z}, c[3] = {s->c.x, s->c.y, s->c.z}, r[3];
  for (int i = 0; i < 3; i++) r[i] = s->sel[i] < 0 ? c[i] : q[s->sel[i]];
  return V(r[0], r[1], r[2]);
}

void oracle_integral_ray(const double* origin, const double* direction, int steps, double distance,
                         const double* c, const int* select, double* out) {
  sel_ctx s = {vload(c), {select[0], select[1], select[2]}};
  vstore(out, integral_ray(vload(origin), vload(direction), steps, distance, sel_fn, &s));
}

void oracle_integral_sphere(int half, int steps, const double* normal, const double* c, const int* select,
                            double* out) {
  sel_ctx s = {vload(c), {select[0], select[1], select[2]}};
  v3 r = half ? integral_half_sphere(steps, vload(normal), sel_fn, &s)
              : integral_sphere(steps, vload(normal), sel_fn, &s);
  vstore(out, r);
}

void oracle_integrate_circle(int steps, const double* c, double* out) {
  sel_ctx s = {vload(c), {-1, -1, -1}};
  /* integrate-circle applies fun to the angle; a constant integrand ignores it */
  ring_ctx r = {sel_fn, &s, 1.0, 0.0, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  vstore(out, integrate_circle_ring(steps, &r));
}

/* number of directions of integral-sphere / integral-half-sphere */
int oracle_sphere_directions(int half, int steps) {
  int theta_steps = half ? steps >> 2 : steps >> 1;
  double range = half ? M_PI / 2 : M_PI;
  int n = 0;
  for (int k = 0; k < theta_steps; k++) {
    double theta = range * ((0.5 + k) / theta_steps);
    n += (int)ceil(sin(theta) * steps);
  }
  return n;
}

void oracle_orthogonal(const double* n, double* out) { vstore(out, orthogonal(vload(n))); }

double oracle_horizon_distance(const oracle_planet* p, double radius) {
  planet_t pp = planet_from(p);
  return horizon_distance(&pp, radius);
}

double oracle_elevation_to_index(const oracle_planet* p, int size, const double* point, const double* direction,
                                 int above) {
  planet_t pp = planet_from(p);
  return elevation_to_index(&pp, size, vload(point), vload(direction), above);
}

int oracle_index_to_elevation(const oracle_planet* p, int size, double radius, double index, double* direction) {
  planet_t pp = planet_from(p);
  int above;
  vstore(direction, index_to_elevation(&pp, size, radius, index, &above));
  return above;
}

double oracle_height_to_index(const oracle_planet* p, int size, const double* point) {
  planet_t pp = planet_from(p);
  return height_to_index(&pp, size, vload(point));
}

void oracle_index_to_height(const oracle_planet* p, int size, double index, double* point) {
  planet_t pp = planet_from(p);
  vstore(point, index_to_height(&pp, size, index));
}

double oracle_sun_elevation_to_index(int size, const double* point, const double* light) {
  return sun_elevation_to_index(size, vload(point), vload(light));
}

double oracle_index_to_sin_sun_elevation(int size, double index) { return index_to_sin_sun_elevation(size, index); }

double oracle_sun_angle_to_index(int size, const double* direction, const double* light) {
  return sun_angle_to_index(size, vload(direction), vload(light));
}

void oracle_index_to_sun_direction(int size, const double* direction, double sin_sun, double index, double* out) {
  vstore(out, index_to_sun_direction(size, vload(direction), sin_sun, index));
}

/* space: 0 transmittance (2-D), 1 surface radiance (2-D), 2 ray scatter (4-D) */
void oracle_space_forward(const oracle_planet* p, int space, const int* shape, const double* point,
                          const double* direction, const double* light, int above, double* out) {
  planet_t pp = planet_from(p);
  if (space == 0) transmittance_forward(&pp, shape, vload(point), vload(direction), above, out);
  else if (space == 1) surface_radiance_forward(&pp, shape, vload(point), vload(light), out);
  else ray_scatter_forward(&pp, shape, vload(point), vload(direction), vload(light), above, out);
}

int oracle_space_backward(const oracle_planet* p, int space, const int* shape, const double* idx, double* point,
                          double* direction, double* light) {
  planet_t pp = planet_from(p);
  v3 pt = ZERO, d = ZERO, l = ZERO;
  int above = 0;
  if (space == 0) transmittance_backward(&pp, shape, idx, &pt, &d, &above);
  else if (space == 1) surface_radiance_backward(&pp, shape, idx, &pt, &l);
  else ray_scatter_backward(&pp, shape, idx, &pt, &d, &l, &above);
  vstore(point, pt);
  vstore(direction, d);
  vstore(light, l);
  return above;
}

/* interpolation-table over a table of vec3 with explicit coordinates */
void oracle_interpolate(int ndim, const int* shape, const double* data, const double* coords, double* out) {
  table_t t;
  table_init(&t, ndim, shape, (double*)data);
  vstore(out, interpolate_value(&t, coords));
}

/* ------------------------------------------------------------------------ */
/* GLSL consumers restated on the CPU in FP32 (resources/shaders/...)        */
/* ------------------------------------------------------------------------ */

typedef struct { float x, y, z; } f3;
static inline f3 F(float x, float y, float z) { f3 r = {x, y, z}; return r; }
static inline float fdot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline float flen(f3 a) { return sqrtf(fdot(a, a)); }
static inline f3 fsub(f3 a, f3 b) { return F(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline f3 fadd(f3 a, f3 b) { return F(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline f3 fmulf(f3 a, float s) { return F(a.x * s, a.y * s, a.z * s); }
static inline f3 femul(f3 a, f3 b) { return F(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline f3 fediv(f3 a, f3 b) { return F(a.x / b.x, a.y / b.y, a.z / b.z); }

typedef struct {
  float radius, max_height;
  int t_height_size, t_elevation_size;
  int height_size, elevation_size, light_elevation_size, heading_size;
  const float* transmittance;  /* width t_elevation_size, height t_height_size, RGB */
  const float* ray_scatter;    /* width elevation*heading, height height*light-elevation */
  const float* mie_strength;
  int weight_bits;             /* 0: exact float weights; else fixed-point bilinear weights */
} glsl_env;

/* core/limit-quot.glsl */
static float limit_quot_f(float a, float b, float lower, float upper) {
  if (a == 0.0f) return 0.0f;
  if (b < 0) { a = -a; b = -b; }
  if (a < b * upper) {
    if (a > b * lower) return a / b;
    return lower;
  }
  return upper;
}

/* core/horizon-distance.glsl */
static float horizon_distance_f(float ground_radius, float radius_sqr) {
  float d = radius_sqr - ground_radius * ground_radius;
  return sqrtf(d > 0.0f ? d : 0.0f);
}

/* core/height-to-index.glsl (normalised to [0, 1]) */
static float height_to_index_f(const glsl_env* e, f3 point) {
  float current = horizon_distance_f(e->radius, fdot(point, point));
  float top = e->radius + e->max_height;
  float maxd = horizon_distance_f(e->radius, top * top);
  return current / maxd;
}

/* core/elevation-to-index.glsl */
static float elevation_to_index_f(const glsl_env* e, f3 point, f3 direction, int above) {
  float point_radius = flen(point);
  float sin_elevation = fdot(point, direction) / point_radius;
  float rho = horizon_distance_f(e->radius, point_radius * point_radius);
  float delta = point_radius * point_radius * sin_elevation * sin_elevation - rho * rho;
  if (above) {
    float top_radius = e->radius + e->max_height;
    float h = sqrtf(top_radius * top_radius - e->radius * e->radius);
    float d = delta + h * h;
    return 0.5f - limit_quot_f(point_radius * sin_elevation - sqrtf(d > 0 ? d : 0), 2 * rho + 2 * h, -0.5f, 0.0f);
  }
  return 0.5f + limit_quot_f(point_radius * sin_elevation + sqrtf(delta > 0 ? delta : 0), 2 * rho, -0.5f, 0.0f);
}

/* GLSL's exp() is implementation-defined; the CUDA lookups use their own
 * exponential, restated here with the same single-precision operations in the
 * same order so that both sides return the same bits: Cody and Waite's
 * reduction y = k ln2 + r (ln 2 split into the 16-bit head 45426/65536 and its
 * remainder), the degree-7 Taylor polynomial of exp(r) by Horner's rule, and
 * the exact scaling by 2^k. */
static float exp_cw(float y) {
  float k = rintf(y * 1.44269504088896341f);
  float r = (y - k * 0.693145751953125f) - k * 1.42860682030941723e-6f;
  float p = 1.0f / 5040.0f;
  p = p * r + 1.0f / 720.0f;
  p = p * r + 1.0f / 120.0f;
  p = p * r + 1.0f / 24.0f;
  p = p * r + 1.0f / 6.0f;
  p = p * r + 0.5f;
  p = p * r + 1.0f;
  p = p * r + 1.0f;
  return ldexpf(p, (int)k);
}

/* core/sun-elevation-to-index.glsl, core/sun-angle-to-index.glsl */
static float sun_elevation_to_index_f(f3 point, f3 light) {
  float sin_elevation = fdot(point, light) / flen(point);
  float r = (1 - exp_cw(-3 * sin_elevation - 0.6f)) / (1 - exp_cw(-3.6f));
  return r > 0 ? r : 0;
}
static float sun_angle_to_index_f(f3 direction, f3 light) { return 0.5f * (1 + fdot(direction, light)); }

/* core/is-above-horizon.glsl */
static int is_above_horizon_f(const glsl_env* e, f3 point, f3 direction) {
  float dist = flen(point);
  float sin_elevation_radius = fdot(direction, point);
  float horizon_distance_sqr = dist * dist - e->radius * e->radius;
  return sin_elevation_radius >= 0 || sin_elevation_radius * sin_elevation_radius <= horizon_distance_sqr;
}

/* GL_LINEAR + CLAMP_TO_EDGE texture() on an RGB32F texture at texel-space
 * coordinates (x, y) = uv * size - 0.5 */
static float quantize_weight(float f, int bits) {
  if (!bits) return f;
  float s = (float)(1 << bits);
  return floorf(f * s + 0.5f) / s;
}

static f3 texel(const float* tex, int w, int h, int x, int y) {
  if (x < 0) x = 0;
  if (x > w - 1) x = w - 1;
  if (y < 0) y = 0;
  if (y > h - 1) y = h - 1;
  const float* p = tex + 3 * ((long)y * w + x);
  return F(p[0], p[1], p[2]);
}

static f3 texture_bilinear(const float* tex, int w, int h, float u, float v, int bits) {
  float x = u * w - 0.5f, y = v * h - 0.5f;
  float x0 = floorf(x), y0 = floorf(y);
  float fx = quantize_weight(x - x0, bits), fy = quantize_weight(y - y0, bits);
  int ix = (int)x0, iy = (int)y0;
  f3 a = texel(tex, w, h, ix, iy), b = texel(tex, w, h, ix + 1, iy);
  f3 c = texel(tex, w, h, ix, iy + 1), d = texel(tex, w, h, ix + 1, iy + 1);
  f3 top = fadd(fmulf(a, 1 - fx), fmulf(b, fx));
  f3 bot = fadd(fmulf(c, 1 - fx), fmulf(d, fx));
  return fadd(fmulf(top, 1 - fy), fmulf(bot, fy));
}

/* core/interpolate-2d.glsl with core/convert-2d-index.glsl; idx = (x, y) */
static f3 interpolate_2d_f(const float* tex, int size_y, int size_x, float ix, float iy, int bits) {
  float u = (ix * (size_x - 1) + 0.5f) / size_x;
  float v = (iy * (size_y - 1) + 0.5f) / size_y;
  return texture_bilinear(tex, size_x, size_y, u, v, bits);
}

/* core/interpolate-4d.glsl with core/make-2d-index-from-4d.glsl; idx = (x, y, z, w) */
static f3 interpolate_4d_f(const float* tex, int size_w, int size_z, int size_y, int size_x, const float* idx,
                           int bits) {
  float px = idx[0] * (size_x - 1), py = idx[1] * (size_y - 1), pz = idx[2] * (size_z - 1), pw = idx[3] * (size_w - 1);
  float fz = pz - floorf(pz), fw = pw - floorf(pw);
  float z_floor = floorf(pz), w_floor = floorf(pw);
  float dx = (float)(size_x * size_z), dy = (float)(size_y * size_w);
  float z1 = z_floor + 1 < size_z - 1 ? z_floor + 1 : (float)(size_z - 1);
  float w1 = w_floor + 1 < size_w - 1 ? w_floor + 1 : (float)(size_w - 1);
  float s = (0.5f + px + z_floor * size_x) / dx, t = (0.5f + px + z1 * size_x) / dx;
  float p = (0.5f + py + w_floor * size_y) / dy, q = (0.5f + py + w1 * size_y) / dy;
  int W = size_x * size_z, H = size_y * size_w;
  f3 sp = texture_bilinear(tex, W, H, s, p, bits), tp = texture_bilinear(tex, W, H, t, p, bits);
  f3 sq = texture_bilinear(tex, W, H, s, q, bits), tq = texture_bilinear(tex, W, H, t, q, bits);
  return fadd(fadd(fmulf(sp, (1 - fz) * (1 - fw)), fmulf(tp, fz * (1 - fw))),
              fadd(fmulf(sq, (1 - fz) * fw), fmulf(tq, fz * fw)));
}

/* atmosphere/phase-function.glsl; pow(t, 1.5) as t * sqrt(t) */
static float phase_f(float g, float mu) {
  float t = 1 + g * g - 2 * g * mu;
  return 3 * (1 - g * g) * (1 + mu * mu) / (8 * (float)M_PI * (2 + g * g) * (t * sqrtf(t)));
}

/* core/transmittance-forward.glsl: (elevation, height) */
static void transmittance_forward_f(const glsl_env* e, f3 point, f3 direction, int above, float* out) {
  out[0] = elevation_to_index_f(e, point, direction, above);
  out[1] = height_to_index_f(e, point);
}

/* atmosphere/transmittance-track.glsl */
static f3 transmittance_track_f(const glsl_env* e, f3 p, f3 q) {
  float dist = flen(fsub(q, p));
  if (dist > 0) {
    f3 direction = fmulf(fsub(q, p), 1.0f / dist);
    int above = is_above_horizon_f(e, p, direction);
    float uvp[2], uvq[2];
    transmittance_forward_f(e, p, direction, above, uvp);
    transmittance_forward_f(e, q, direction, above, uvq);
    f3 t1 = interpolate_2d_f(e->transmittance, e->t_height_size, e->t_elevation_size, uvp[0], uvp[1], e->weight_bits);
    f3 t2 = interpolate_2d_f(e->transmittance, e->t_height_size, e->t_elevation_size, uvq[0], uvq[1], e->weight_bits);
    return fediv(t1, t2);
  }
  return F(1, 1, 1);
}

/* atmosphere/transmittance-outer.glsl */
static f3 transmittance_outer_f(const glsl_env* e, f3 point, f3 direction) {
  float uv[2];
  transmittance_forward_f(e, point, direction, 1, uv);
  return interpolate_2d_f(e->transmittance, e->t_height_size, e->t_elevation_size, uv[0], uv[1], e->weight_bits);
}

/* core/ray-scatter-forward.glsl: (sun angle, sun elevation, elevation, height) */
static void ray_scatter_forward_f(const glsl_env* e, f3 point, f3 direction, f3 light, int above, float* out) {
  out[0] = sun_angle_to_index_f(direction, light);
  out[1] = sun_elevation_to_index_f(point, light);
  out[2] = elevation_to_index_f(e, point, direction, above);
  out[3] = height_to_index_f(e, point);
}

static f3 in_scatter_at_f(const glsl_env* e, const float* idx, float mu) {
  f3 s = interpolate_4d_f(e->ray_scatter, e->height_size, e->elevation_size, e->light_elevation_size,
                          e->heading_size, idx, e->weight_bits);
  f3 m = interpolate_4d_f(e->mie_strength, e->height_size, e->elevation_size, e->light_elevation_size,
                          e->heading_size, idx, e->weight_bits);
  return fadd(s, fmulf(m, phase_f(0.76f, mu)));
}

/* atmosphere/ray-scatter-track.glsl */
static f3 ray_scatter_track_f(const glsl_env* e, f3 light, f3 p, f3 q) {
  float dist = flen(fsub(q, p));
  if (dist > 0) {
    f3 direction = fmulf(fsub(q, p), 1.0f / dist);
    int above = is_above_horizon_f(e, p, direction);
    float mu = fdot(direction, light);
    float ip[4], iq[4];
    ray_scatter_forward_f(e, p, direction, light, above, ip);
    f3 sp = in_scatter_at_f(e, ip, mu);
    ray_scatter_forward_f(e, q, direction, light, above, iq);
    f3 sq = in_scatter_at_f(e, iq, mu);
    f3 t = transmittance_track_f(e, p, q);
    return fsub(sp, femul(t, sq));
  }
  return F(0, 0, 0);
}

/* atmosphere/ray-scatter-outer.glsl */
static f3 ray_scatter_outer_f(const glsl_env* e, f3 light, f3 point, f3 direction) {
  float idx[4];
  ray_scatter_forward_f(e, point, direction, light, 1, idx);
  return in_scatter_at_f(e, idx, fdot(direction, light));
}

/* in-scatter at (point, direction) with the horizon test choosing the half */
static f3 in_scatter_query_f(const glsl_env* e, f3 light, f3 point, f3 direction) {
  float idx[4];
  ray_scatter_forward_f(e, point, direction, light, is_above_horizon_f(e, point, direction), idx);
  return in_scatter_at_f(e, idx, fdot(direction, light));
}

/* core/ray-hypersphere.glsl instantiated as ray_sphere (shaders.clj:18-20):
 * out = (distance to the entry, clipped at 0, and length inside) */
static void ray_sphere_f(f3 centre, float radius, f3 origin, f3 direction, float* out) {
  f3 pos = fsub(origin, centre);
  float direction_sqr = fdot(direction, direction);
  float direction_pos = fdot(direction, pos);
  float discriminant = direction_pos * direction_pos - direction_sqr * (fdot(pos, pos) - radius * radius);
  if (discriminant > 0) {
    float half_length = sqrtf(discriminant) / direction_sqr;
    float middle = -fdot(direction, pos) / direction_sqr;
    out[0] = middle - half_length;
    out[1] = 2 * half_length;
    if (out[0] < 0) {
      out[1] = fmaxf(0.0f, out[1] + out[0]);
      out[0] = 0;
    }
  } else {
    out[0] = 0;
    out[1] = 0;
  }
}

/* core/limit-interval.glsl */
static void limit_interval_f(float* interval, float limit) {
  float end = fminf(interval[0] + interval[1], limit);
  interval[1] = end - interval[0];
}

/* atmosphere/attenuate.glsl: incoming RGBA through the track from start to point */
static void attenuate_f(const glsl_env* e, f3 light, f3 start, f3 point, const float* incoming, float amplification,
                        float* out) {
  f3 transmittance = transmittance_track_f(e, start, point);
  f3 in_scatter = fmulf(ray_scatter_track_f(e, light, start, point), amplification);
  out[0] = incoming[0] * transmittance.x + in_scatter.x * incoming[3];
  out[1] = incoming[1] * transmittance.y + in_scatter.y * incoming[3];
  out[2] = incoming[2] * transmittance.z + in_scatter.z * incoming[3];
  out[3] = incoming[3];
}

/* atmosphere/attenuation-outer.glsl: RGB light from origin + a direction,
 * looking along direction out of the atmosphere */
static void attenuation_outer_f(const glsl_env* e, f3 light, f3 origin, f3 direction, float a, const float* incoming,
                                float amplification, float* out) {
  f3 point = fadd(origin, fmulf(direction, a));
  f3 transmittance = transmittance_outer_f(e, point, direction);
  f3 ray_scatter = fmulf(ray_scatter_outer_f(e, light, point, direction), amplification);
  out[0] = incoming[0] * transmittance.x + ray_scatter.x;
  out[1] = incoming[1] * transmittance.y + ray_scatter.y;
  out[2] = incoming[2] * transmittance.z + ray_scatter.z;
}

/* atmosphere/attenuation-track.glsl: segment = (start, length) along the ray */
static void attenuation_track_f(const glsl_env* e, f3 light, f3 origin, f3 direction, const float* segment,
                                const float* incoming, float amplification, float* out) {
  if (segment[1] > 0) {
    f3 p = fadd(origin, fmulf(direction, segment[0]));
    f3 q = fadd(origin, fmulf(direction, segment[0] + segment[1]));
    attenuate_f(e, light, p, q, incoming, amplification, out);
  } else {
    for (int c = 0; c < 4; c++) out[c] = incoming[c];
  }
}

/* atmosphere/attenuation-point.glsl with its uniforms origin (the eye) and
 * light_direction; normalize(v) taken as v times 1 / length(v), as the
 * track lookups above divide a vector by a distance */
static void attenuation_point_f(const glsl_env* e, f3 light, f3 origin, f3 point, const float* incoming,
                                float amplification, float* out) {
  f3 v = fsub(point, origin);
  f3 direction = fmulf(v, 1.0f / flen(v));
  float atmosphere[2];
  ray_sphere_f(F(0, 0, 0), e->radius + e->max_height, origin, direction, atmosphere);
  limit_interval_f(atmosphere, flen(fsub(origin, point)));
  attenuation_track_f(e, light, origin, direction, atmosphere, incoming, amplification, out);
}

/* atmosphere/transmittance-point.glsl with its uniform light_direction */
static f3 transmittance_point_f(const glsl_env* e, f3 light, f3 point) {
  float atmosphere[2];
  ray_sphere_f(F(0, 0, 0), e->radius + e->max_height, point, light, atmosphere);
  if (atmosphere[1] > 0) return transmittance_outer_f(e, fadd(point, fmulf(light, atmosphere[0])), light);
  return F(1, 1, 1);
}

/* n attenuation queries (out [n][4]):
 *   kind 0 attenuation_outer(light, p, d, s[0], incoming.rgb), alpha passed through
 *   kind 1 attenuation_track(light, p, d, (s[0], s[1]), incoming)
 *   kind 2 attenuation_point(point p, incoming) with the uniform origin d
 *   kind 3 transmittance_point(p), alpha 1
 * light, p, d [n][3]; s [n][2]; incoming [n][4]; unused arrays may be NULL. */
void oracle_glsl_attenuation_batch(const oracle_glsl_tables* t, int kind, long n, const float* light, const float* p,
                                   const float* d, const float* s, const float* incoming, float amplification,
                                   float* out) {
  glsl_env e = {t->radius, t->max_height, t->t_height_size, t->t_elevation_size, t->height_size, t->elevation_size,
                t->light_elevation_size, t->heading_size, t->transmittance, t->ray_scatter, t->mie_strength,
                t->weight_bits};
  for (long i = 0; i < n; i++) {
    f3 L = F(light[3 * i], light[3 * i + 1], light[3 * i + 2]), P = F(p[3 * i], p[3 * i + 1], p[3 * i + 2]);
    float* o = out + 4 * i;
    if (kind == 3) {
      f3 r = transmittance_point_f(&e, L, P);
      o[0] = r.x; o[1] = r.y; o[2] = r.z; o[3] = 1;
      continue;
    }
    f3 D = F(d[3 * i], d[3 * i + 1], d[3 * i + 2]);
    const float* in = incoming + 4 * i;
    if (kind == 0) {
      attenuation_outer_f(&e, L, P, D, s[2 * i], in, amplification, o);
      o[3] = in[3];
    } else if (kind == 1) {
      attenuation_track_f(&e, L, P, D, s + 2 * i, in, amplification, o);
    } else {
      attenuation_point_f(&e, L, D, P, in, amplification, o);
    }
  }
}

/* kind 0: transmittance_track(p, q); 1: transmittance_outer(p, d);
 * 2: ray_scatter_track(light, p, q); 3: ray_scatter_outer(light, p, d) */
void oracle_glsl_query(const oracle_glsl_tables* t, int kind, const float* light, const float* p, const float* q,
                       float* out) {
  glsl_env e = {t->radius, t->max_height, t->t_height_size, t->t_elevation_size, t->height_size, t->elevation_size,
                t->light_elevation_size, t->heading_size, t->transmittance, t->ray_scatter, t->mie_strength,
                t->weight_bits};
  f3 P = F(p[0], p[1], p[2]), Q = F(q[0], q[1], q[2]), L = F(light[0], light[1], light[2]);
  f3 r;
  switch (kind) {
    case 0: r = transmittance_track_f(&e, P, Q); break;
    case 1: r = transmittance_outer_f(&e, P, Q); break;
    case 2: r = ray_scatter_track_f(&e, L, P, Q); break;
    case 3: r = ray_scatter_outer_f(&e, L, P, Q); break;
    default: r = in_scatter_query_f(&e, L, P, Q); break;
  }
  out[0] = r.x; out[1] = r.y; out[2] = r.z;
}

/* n queries at once (light, p, q and out [n][3]); above (may be NULL)
 * receives is-above-horizon(p, q) of each query, the test that chooses the
 * table half in kinds 0, 2 and 4. */
void oracle_glsl_query_batch(const oracle_glsl_tables* t, int kind, long n, const float* light, const float* p,
                             const float* q, float* out, int* above) {
  glsl_env e = {t->radius, t->max_height, t->t_height_size, t->t_elevation_size, t->height_size, t->elevation_size,
                t->light_elevation_size, t->heading_size, t->transmittance, t->ray_scatter, t->mie_strength,
                t->weight_bits};
  for (long i = 0; i < n; i++) {
    oracle_glsl_query(t, kind, light + 3 * i, p + 3 * i, q + 3 * i, out + 3 * i);
    if (above) {
      f3 P = F(p[3 * i], p[3 * i + 1], p[3 * i + 2]), Q = F(q[3 * i], q[3 * i + 1], q[3 * i + 2]);
      f3 d = Q;
      if (kind == 0 || kind == 2) {
        float dist = flen(fsub(Q, P));
        d = dist > 0 ? fmulf(fsub(Q, P), 1.0f / dist) : Q;
      }
      above[i] = is_above_horizon_f(&e, P, d);
    }
  }
}
