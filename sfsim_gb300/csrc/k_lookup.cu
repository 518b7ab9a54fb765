// k_lookup.cu -- the table lookups sfsim's shaders perform, restated in FP32
// as the GLSL computes them (resources/shaders/atmosphere/
// transmittance-track.glsl, transmittance-outer.glsl, ray-scatter-track.glsl,
// ray-scatter-outer.glsl with core/interpolate-2d.glsl, interpolate-4d.glsl,
// core/*-to-index.glsl and limit-quot.glsl), on the .scatter tables; and the
// surrogate's coordinates, which are formed by the same lookup.
//
// This file is compiled with -fmad=false: every +, -, *, / and sqrt is a
// separately rounded IEEE operation, as in the oracle's C restatement
// (compiled with -ffp-contract=off), and the one transcendental is exp_cw
// below, restated there too.  Both sides therefore compute the same bits from
// the same FP32 inputs.
#include "atmo_device.cuh"
#include "kernels.h"

namespace sfsim {


struct f3 {
  float x, y, z;
};
__device__ __forceinline__ f3 F3(float x, float y, float z) { return f3{x, y, z}; }
__device__ __forceinline__ float fdot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ f3 fsub(f3 a, f3 b) { return F3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ f3 fadd(f3 a, f3 b) { return F3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ f3 fmul(f3 a, float s) { return F3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ f3 femul(f3 a, f3 b) { return F3(a.x * b.x, a.y * b.y, a.z * b.z); }

// core/horizon-distance.glsl
__device__ __forceinline__ float horizon_distance_f(float ground_radius, float radius_sqr) {
  return sqrtf(fmaxf(0.0f, radius_sqr - ground_radius * ground_radius));
}

struct GlslEnv {
  float radius, max_height;
  int t_height, t_elevation;           // transmittance table
  int height, elevation, light, heading;  // 4-D tables
  const float* T;                      // width t_elevation, height t_height
  const float* S;                      // width elevation*heading, height height*light
  const float* M;
  int weight_bits;                     // 0: exact weights; 8: GL 8-bit fixed-point filtering
  float mie_g;
};

// core/height-to-index.glsl (normalised)
__device__ __forceinline__ float height_to_index_g(const GlslEnv& e, f3 p) {
  const float top = e.radius + e.max_height;
  return horizon_distance_f(e.radius, fdot(p, p)) / horizon_distance_f(e.radius, top * top);
}

// core/elevation-to-index.glsl
__device__ __forceinline__ float elevation_to_index_g(const GlslEnv& e, f3 p, f3 d, bool above) {
  const float pr = sqrtf(fdot(p, p));
  const float sin_el = fdot(p, d) / pr;
  const float rho = horizon_distance_f(e.radius, pr * pr);
  const float delta = pr * pr * sin_el * sin_el - rho * rho;
  if (above) {
    const float top = e.radius + e.max_height;
    const float h = sqrtf(top * top - e.radius * e.radius);
    return 0.5f - limit_quot_f(pr * sin_el - sqrtf(fmaxf(0.0f, delta + h * h)), 2 * rho + 2 * h, -0.5f, 0.0f);
  }
  return 0.5f + limit_quot_f(pr * sin_el + sqrtf(fmaxf(0.0f, delta)), 2 * rho, -0.5f, 0.0f);
}

// GLSL's exp() is implementation-defined.  The lookups use this one, so that
// the oracle's C restatement (the same operations in the same order, no
// contraction) returns identical bits: Cody and Waite's reduction
// y = k ln2 + r with |r| <= ln2 / 2 and ln 2 split into a 16-bit head
// (45426 / 65536, so k * head is exact for |k| < 256) and its remainder, then
// the Taylor polynomial of exp(r) to degree 7 by Horner's rule (truncation
// below 1e-8 relative), scaled by 2^k.  Within about 2 ulp of exp(y) for
// |y| < 80.
__device__ __forceinline__ float exp_cw(float y) {
  const float k = rintf(y * 1.44269504088896341f);
  const float r = (y - k * 0.693145751953125f) - k * 1.42860682030941723e-6f;
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

// core/sun-elevation-to-index.glsl, core/sun-angle-to-index.glsl
__device__ __forceinline__ float sun_elevation_to_index_g(f3 p, f3 l) {
  const float s = fdot(p, l) / sqrtf(fdot(p, p));
  return fmaxf(0.0f, (1 - exp_cw(-3 * s - 0.6f)) / (1 - exp_cw(-3.6f)));
}
__device__ __forceinline__ float sun_angle_to_index_g(f3 d, f3 l) { return 0.5f * (1 + fdot(d, l)); }

// core/is-above-horizon.glsl
__device__ __forceinline__ bool is_above_horizon_g(const GlslEnv& e, f3 p, f3 d) {
  const float dist = sqrtf(fdot(p, p));
  const float s = fdot(d, p);
  return s >= 0 || s * s <= dist * dist - e.radius * e.radius;
}

// texture() with GL_LINEAR and CLAMP_TO_EDGE on an RGB float texture at
// texel coordinates (x, y) = uv * size - 0.5
__device__ __forceinline__ float q_weight(float f, int bits) {
  if (!bits) return f;
  const float s = (float)(1 << bits);
  return floorf(f * s + 0.5f) / s;
}

__device__ __forceinline__ f3 texel(const float* t, int w, int h, int x, int y) {
  x = min(max(x, 0), w - 1);
  y = min(max(y, 0), h - 1);
  const float* p = t + 3 * ((long long)y * w + x);
  return F3(p[0], p[1], p[2]);
}

__device__ __forceinline__ f3 texture_g(const float* t, int w, int h, float u, float v, int bits) {
  const float x = u * w - 0.5f, y = v * h - 0.5f;
  const float x0 = floorf(x), y0 = floorf(y);
  const float fx = q_weight(x - x0, bits), fy = q_weight(y - y0, bits);
  const int ix = (int)x0, iy = (int)y0;
  const f3 a = texel(t, w, h, ix, iy), b = texel(t, w, h, ix + 1, iy);
  const f3 c = texel(t, w, h, ix, iy + 1), d = texel(t, w, h, ix + 1, iy + 1);
  const f3 top = fadd(fmul(a, 1 - fx), fmul(b, fx));
  const f3 bot = fadd(fmul(c, 1 - fx), fmul(d, fx));
  return fadd(fmul(top, 1 - fy), fmul(bot, fy));
}

// core/interpolate-2d.glsl + convert-2d-index.glsl; idx = (x, y)
__device__ __forceinline__ f3 interpolate_2d_g(const float* t, int size_y, int size_x, float ix, float iy, int bits) {
  const float u = (ix * (size_x - 1) + 0.5f) / size_x;
  const float v = (iy * (size_y - 1) + 0.5f) / size_y;
  return texture_g(t, size_x, size_y, u, v, bits);
}

// core/interpolate-4d.glsl + make-2d-index-from-4d.glsl; idx = (x, y, z, w)
__device__ __forceinline__ f3 interpolate_4d_g(const float* t, int size_w, int size_z, int size_y, int size_x,
                                               const float* idx, int bits) {
  const float px = idx[0] * (size_x - 1), py = idx[1] * (size_y - 1);
  const float pz = idx[2] * (size_z - 1), pw = idx[3] * (size_w - 1);
  const float fz = pz - floorf(pz), fw = pw - floorf(pw);
  const float zf = floorf(pz), wf = floorf(pw);
  const float dx = (float)(size_x * size_z), dy = (float)(size_y * size_w);
  const float z1 = fminf(zf + 1, (float)(size_z - 1)), w1 = fminf(wf + 1, (float)(size_w - 1));
  const float s = (0.5f + px + zf * size_x) / dx, tt = (0.5f + px + z1 * size_x) / dx;
  const float p = (0.5f + py + wf * size_y) / dy, q = (0.5f + py + w1 * size_y) / dy;
  const int W = size_x * size_z, H = size_y * size_w;
  const f3 sp = texture_g(t, W, H, s, p, bits), tp = texture_g(t, W, H, tt, p, bits);
  const f3 sq = texture_g(t, W, H, s, q, bits), tq = texture_g(t, W, H, tt, q, bits);
  return fadd(fadd(fmul(sp, (1 - fz) * (1 - fw)), fmul(tp, fz * (1 - fw))),
              fadd(fmul(sq, (1 - fz) * fw), fmul(tq, fz * fw)));
}

// atmosphere/phase-function.glsl; pow(t, 1.5) as t * sqrt(t), two correctly
// rounded operations
__device__ __forceinline__ float phase_g(float g, float mu) {
  const float t = 1 + g * g - 2 * g * mu;
  return 3 * (1 - g * g) * (1 + mu * mu) / (8 * 3.14159265358979323846f * (2 + g * g) * (t * sqrtf(t)));
}

__device__ __forceinline__ void transmittance_forward_g(const GlslEnv& e, f3 p, f3 d, bool above, float* out) {
  out[0] = elevation_to_index_g(e, p, d, above);
  out[1] = height_to_index_g(e, p);
}

// atmosphere/transmittance-track.glsl
__device__ f3 transmittance_track_g(const GlslEnv& e, f3 p, f3 q) {
  const float dist = sqrtf(fdot(fsub(q, p), fsub(q, p)));
  if (dist > 0) {
    const f3 d = fmul(fsub(q, p), 1.0f / dist);
    const bool above = is_above_horizon_g(e, p, d);
    float a[2], b[2];
    transmittance_forward_g(e, p, d, above, a);
    transmittance_forward_g(e, q, d, above, b);
    const f3 t1 = interpolate_2d_g(e.T, e.t_height, e.t_elevation, a[0], a[1], e.weight_bits);
    const f3 t2 = interpolate_2d_g(e.T, e.t_height, e.t_elevation, b[0], b[1], e.weight_bits);
    return F3(t1.x / t2.x, t1.y / t2.y, t1.z / t2.z);
  }
  return F3(1, 1, 1);
}

// atmosphere/transmittance-outer.glsl
__device__ f3 transmittance_outer_g(const GlslEnv& e, f3 p, f3 d) {
  float a[2];
  transmittance_forward_g(e, p, d, true, a);
  return interpolate_2d_g(e.T, e.t_height, e.t_elevation, a[0], a[1], e.weight_bits);
}

// core/ray-scatter-forward.glsl: (sun angle, sun elevation, elevation, height)
__device__ __forceinline__ void ray_scatter_forward_g(const GlslEnv& e, f3 p, f3 d, f3 l, bool above, float* out) {
  out[0] = sun_angle_to_index_g(d, l);
  out[1] = sun_elevation_to_index_g(p, l);
  out[2] = elevation_to_index_g(e, p, d, above);
  out[3] = height_to_index_g(e, p);
}

__device__ __forceinline__ f3 in_scatter_g(const GlslEnv& e, const float* idx, float mu) {
  const f3 s = interpolate_4d_g(e.S, e.height, e.elevation, e.light, e.heading, idx, e.weight_bits);
  const f3 m = interpolate_4d_g(e.M, e.height, e.elevation, e.light, e.heading, idx, e.weight_bits);
  return fadd(s, fmul(m, phase_g(e.mie_g, mu)));
}

// atmosphere/ray-scatter-track.glsl
__device__ f3 ray_scatter_track_g(const GlslEnv& e, f3 l, f3 p, f3 q) {
  const float dist = sqrtf(fdot(fsub(q, p), fsub(q, p)));
  if (dist > 0) {
    const f3 d = fmul(fsub(q, p), 1.0f / dist);
    const bool above = is_above_horizon_g(e, p, d);
    const float mu = fdot(d, l);
    float ip[4], iq[4];
    ray_scatter_forward_g(e, p, d, l, above, ip);
    const f3 sp = in_scatter_g(e, ip, mu);
    ray_scatter_forward_g(e, q, d, l, above, iq);
    const f3 sq = in_scatter_g(e, iq, mu);
    const f3 t = transmittance_track_g(e, p, q);
    return fsub(sp, femul(t, sq));
  }
  return F3(0, 0, 0);
}

// atmosphere/ray-scatter-outer.glsl
__device__ f3 ray_scatter_outer_g(const GlslEnv& e, f3 l, f3 p, f3 d) {
  float idx[4];
  ray_scatter_forward_g(e, p, d, l, true, idx);
  return in_scatter_g(e, idx, fdot(d, l));
}

// In-scatter of the tables at (p, d, l) with the horizon test choosing the
// table half, the lookup the rendered in-scatter comparison uses.
__device__ f3 in_scatter_at_g(const GlslEnv& e, f3 l, f3 p, f3 d) {
  float idx[4];
  ray_scatter_forward_g(e, p, d, l, is_above_horizon_g(e, p, d), idx);
  return in_scatter_g(e, idx, fdot(d, l));
}

__global__ void k_query_table(GlslEnv e, int kind, long long n, const float* A, const float* Bv, const float* L,
                              float* out) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= n) return;
  const f3 a = F3(A[3 * t], A[3 * t + 1], A[3 * t + 2]);
  const f3 b = F3(Bv[3 * t], Bv[3 * t + 1], Bv[3 * t + 2]);
  const f3 l = L ? F3(L[3 * t], L[3 * t + 1], L[3 * t + 2]) : F3(0, 0, 1);
  f3 r;
  switch (kind) {
    case 0: r = transmittance_track_g(e, a, b); break;
    case 1: r = transmittance_outer_g(e, a, b); break;
    case 2: r = ray_scatter_track_g(e, l, a, b); break;
    case 3: r = ray_scatter_outer_g(e, l, a, b); break;
    default: r = in_scatter_at_g(e, l, a, b); break;
  }
  out[3 * t] = r.x;
  out[3 * t + 1] = r.y;
  out[3 * t + 2] = r.z;
}

// core/ray-hypersphere.glsl instantiated as ray_sphere (shaders.clj:18-20):
// (distance to the entry, clipped at 0, and length inside)
__device__ float2 ray_sphere_g(f3 centre, float radius, f3 origin, f3 direction) {
  const f3 pos = fsub(origin, centre);
  const float direction_sqr = fdot(direction, direction);
  const float direction_pos = fdot(direction, pos);
  const float discriminant = direction_pos * direction_pos - direction_sqr * (fdot(pos, pos) - radius * radius);
  if (discriminant > 0) {
    const float half_length = sqrtf(discriminant) / direction_sqr;
    const float middle = -fdot(direction, pos) / direction_sqr;
    float2 r = make_float2(middle - half_length, 2 * half_length);
    if (r.x < 0) {
      r.y = fmaxf(0.0f, r.y + r.x);
      r.x = 0;
    }
    return r;
  }
  return make_float2(0, 0);
}

// core/limit-interval.glsl
__device__ __forceinline__ float2 limit_interval_g(float2 interval, float limit) {
  const float end = fminf(interval.x + interval.y, limit);
  return make_float2(interval.x, end - interval.x);
}

// atmosphere/attenuate.glsl: incoming RGBA through the track from start to point
__device__ float4 attenuate_g(const GlslEnv& e, f3 l, f3 start, f3 point, float4 in, float amplification) {
  const f3 t = transmittance_track_g(e, start, point);
  const f3 s = fmul(ray_scatter_track_g(e, l, start, point), amplification);
  return make_float4(in.x * t.x + s.x * in.w, in.y * t.y + s.y * in.w, in.z * t.z + s.z * in.w, in.w);
}

// atmosphere/attenuation-track.glsl: segment = (start, length) along the ray
__device__ float4 attenuation_track_g(const GlslEnv& e, f3 l, f3 origin, f3 direction, float2 segment, float4 in,
                                      float amplification) {
  if (segment.y > 0) {
    const f3 p = fadd(origin, fmul(direction, segment.x));
    const f3 q = fadd(origin, fmul(direction, segment.x + segment.y));
    return attenuate_g(e, l, p, q, in, amplification);
  }
  return in;
}

// Attenuation queries of atmosphere/attenuation-outer.glsl (kind 0, alpha
// passed through), attenuation-track.glsl (1), attenuation-point.glsl (2,
// with the uniform origin, the eye, in D) and transmittance-point.glsl (3,
// alpha 1); normalize(v) is v times 1 / length(v), as the track lookups
// divide a vector by a distance.
__global__ void k_query_attenuation(GlslEnv e, int kind, long long n, const float* L, const float* P,
                                    const float* D, const float* Sg, const float* In, float amplification,
                                    float* out) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= n) return;
  const f3 l = F3(L[3 * t], L[3 * t + 1], L[3 * t + 2]);
  const f3 p = F3(P[3 * t], P[3 * t + 1], P[3 * t + 2]);
  float4 r;
  if (kind == 3) {
    const float2 atm = ray_sphere_g(F3(0, 0, 0), e.radius + e.max_height, p, l);
    const f3 tr = atm.y > 0 ? transmittance_outer_g(e, fadd(p, fmul(l, atm.x)), l) : F3(1, 1, 1);
    r = make_float4(tr.x, tr.y, tr.z, 1.0f);
  } else {
    const f3 d = F3(D[3 * t], D[3 * t + 1], D[3 * t + 2]);
    const float4 in = make_float4(In[4 * t], In[4 * t + 1], In[4 * t + 2], In[4 * t + 3]);
    if (kind == 0) {
      const f3 point = fadd(p, fmul(d, Sg[2 * t]));
      const f3 tr = transmittance_outer_g(e, point, d);
      const f3 rs = fmul(ray_scatter_outer_g(e, l, point, d), amplification);
      r = make_float4(in.x * tr.x + rs.x, in.y * tr.y + rs.y, in.z * tr.z + rs.z, in.w);
    } else if (kind == 1) {
      r = attenuation_track_g(e, l, p, d, make_float2(Sg[2 * t], Sg[2 * t + 1]), in, amplification);
    } else {
      // attenuation_point(point p, incoming) with origin = d
      const f3 v = fsub(p, d);
      const f3 direction = fmul(v, 1.0f / sqrtf(fdot(v, v)));
      float2 atm = ray_sphere_g(F3(0, 0, 0), e.radius + e.max_height, d, direction);
      const f3 w = fsub(d, p);
      atm = limit_interval_g(atm, sqrtf(fdot(w, w)));
      r = attenuation_track_g(e, l, d, direction, atm, in, amplification);
    }
  }
  out[4 * t] = r.x;
  out[4 * t + 1] = r.y;
  out[4 * t + 2] = r.z;
  out[4 * t + 3] = r.w;
}

static GlslEnv make_env(const QueryTables& q, int weight_bits) {
  GlslEnv e;
  e.radius = q.radius;
  e.max_height = q.max_height;
  e.t_height = q.t_height;
  e.t_elevation = q.t_elevation;
  e.height = q.height;
  e.elevation = q.elevation;
  e.light = q.light;
  e.heading = q.heading;
  e.T = q.T;
  e.S = q.S;
  e.M = q.M;
  e.weight_bits = weight_bits;
  e.mie_g = q.mie_g;
  return e;
}

void launch_query_table(const QueryTables& q, int kind, long long n, const float* a, const float* b, const float* l,
                        float* out, int weight_bits, cudaStream_t st) {
  const GlslEnv e = make_env(q, weight_bits);
  const int blk = 128;
  k_query_table<<<(unsigned)((n + blk - 1) / blk), blk, 0, st>>>(e, kind, n, a, b, l, out);
}

void launch_query_attenuation(const QueryTables& q, int kind, long long n, const float* light, const float* p,
                              const float* d, const float* s, const float* incoming, float amplification, float* out,
                              int weight_bits, cudaStream_t st) {
  const GlslEnv e = make_env(q, weight_bits);
  const int blk = 128;
  k_query_attenuation<<<(unsigned)((n + blk - 1) / blk), blk, 0, st>>>(e, kind, n, light, p, d, s, incoming,
                                                                       amplification, out);
}

// The surrogate's coordinates of (p, d, l): the table coordinates as the
// in-scatter lookup forms them (core/ray-scatter-forward.glsl order reversed
// to height, elevation, sun elevation, sun heading) with the table half chosen
// by the horizon test, then (1 + sin of the sun elevation) / 2, the half
// (0 upper, 1 lower) and the four cell phases of the lookup
// (interpolate-4d.glsl scales each coordinate by size - 1).  idx receives the
// lookup's indices.
__device__ __forceinline__ void network_coords(const GlslEnv& e, f3 p, f3 d, f3 l, float* u, float* idx) {
  const bool above = is_above_horizon_g(e, p, d);
  ray_scatter_forward_g(e, p, d, l, above, idx);
  u[0] = idx[3];
  u[1] = idx[2];
  u[2] = idx[1];
  u[3] = idx[0];
  u[4] = fminf(fmaxf(0.5f * (1.0f + fdot(p, l) / sqrtf(fdot(p, p))), 0.0f), 1.0f);
  u[5] = above ? 0.0f : 1.0f;
  const float size[4] = {(float)(e.height - 1), (float)(e.elevation - 1), (float)(e.light - 1),
                         (float)(e.heading - 1)};
#pragma unroll
  for (int c = 0; c < 4; c++) {
    const float x = u[c] * size[c];
    u[kMlpSmooth + c] = x - floorf(x);
  }
}

// The surrogate's coordinates of (x, v, l); the table value there (S + M
// phase) as a by-product when `table` is set.
__global__ void k_query_coords(GlslEnv e, long long n, const double* X, const double* V, const double* L,
                               float* coords, float* table) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= n) return;
  const f3 p = F3((float)X[3 * t], (float)X[3 * t + 1], (float)X[3 * t + 2]);
  const f3 d = F3((float)V[3 * t], (float)V[3 * t + 1], (float)V[3 * t + 2]);
  const f3 l = F3((float)L[3 * t], (float)L[3 * t + 1], (float)L[3 * t + 2]);
  float idx[4], u[kMlpCoords];
  network_coords(e, p, d, l, u, idx);
#pragma unroll
  for (int c = 0; c < kMlpCoords; c++) coords[kMlpCoords * t + c] = u[c];
  if (table) {
    const f3 r = in_scatter_g(e, idx, fdot(d, l));
    table[3 * t] = r.x;
    table[3 * t + 1] = r.y;
    table[3 * t + 2] = r.z;
  }
}

void launch_query_coords(const QueryTables& q, long long n, const double* x, const double* v, const double* l,
                         float* coords, float* table, cudaStream_t st) {
  const GlslEnv e = make_env(q, 0);
  const int blk = 128;
  k_query_coords<<<(unsigned)((n + blk - 1) / blk), blk, 0, st>>>(e, n, x, v, l, coords, table);
}

}  // namespace sfsim
