/*
 * sfsim_atmo.h -- C ABI of the GB300 atmosphere lookup-table builder.
 *
 * The library builds sfsim's four atmosphere lookup tables (transmittance,
 * surface radiance, ray scatter and Mie strength) on one GPU and returns them
 * in the exact `.scatter` file layout that sfsim's runtime loads:
 * little-endian float32, RGB interleaved, no header.
 *
 *   transmittance    [height][elevation][3]
 *   surface radiance [height][sun elevation][3]
 *   ray scatter, mie strength: 4-D tables [height][elevation][sun elevation][sun heading]
 *     stored as 2-D tiles, row = height*n_sun_elevation + sun_elevation,
 *     column = elevation*n_sun_heading + sun_heading, then [3].
 *
 * Reference interfaces replaced (paths inside wedesoft/sfsim):
 *   src/clj/sfsim/atmosphere_lut.clj:43-105  generate-atmosphere-luts (the whole build)
 *   src/clj/sfsim/atmosphere.clj:114-422     the integrands and table spaces
 *   src/clj/sfsim/interpolate.clj:54-109     make-lookup-table / interpolation-table
 *   src/clj/sfsim/matrix.clj:130, image.clj:299, util.clj:227-240  the file layout
 * The calling convention follows the reference's own native precedent,
 * src/c/sfsim/jolt.hh:1-25 (flat extern "C" functions, plain structs of
 * doubles), bound from Clojure with coffi `defcfn` as in src/clj/sfsim/jolt.clj:18-23.
 *
 * Errors: every entry point returns 0 on success or a negative SFSIM_ATMO_E*
 * code; sfsim_atmo_strerror() maps a code to text.  No entry point throws or
 * aborts.  Calls are synchronous unless stated; one host thread at a time per
 * device.
 */
#ifndef SFSIM_ATMO_H
#define SFSIM_ATMO_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Error codes. */
#define SFSIM_ATMO_OK            0
#define SFSIM_ATMO_EINVAL       -1  /* a configuration value is out of range */
#define SFSIM_ATMO_ENOMEM       -2  /* device or host allocation failed */
#define SFSIM_ATMO_ECUDA        -3  /* a CUDA runtime call failed */
#define SFSIM_ATMO_ENODEV       -4  /* no CUDA device is visible */
#define SFSIM_ATMO_ESHAPE       -5  /* a table shape is unsupported */
#define SFSIM_ATMO_ENULL        -6  /* a required pointer is NULL */
#define SFSIM_ATMO_ETOOBIG      -7  /* a size exceeds a fixed capacity */
#define SFSIM_ATMO_ENUMERIC     -8  /* a result contains NaN or Inf */
#define SFSIM_ATMO_ESTOPPED     -9  /* an iteration callback stopped the build */

/* Arithmetic of the bulk integrands.  Ray-sphere intersections and the table
 * parameterisations always run in FP64. */
#define SFSIM_ATMO_FP32 0
#define SFSIM_ATMO_FP64 1

/* Bits of sfsim_atmo_config.flags (0: the reference's algorithm).
 *
 * SFSIM_ATMO_SCAN_RAYS: the transmittance from a table node x to each
 *   midpoint sample p_s of its view ray comes from one prefix scan over the
 *   ray's S cells (O(S) per ray) instead of the reference's nested quadrature
 *   (S midpoint samples between x and every p_s, O(S^2) per ray;
 *   atmosphere.clj:192-200 with ray.clj:19-30).  The optical depth to p_s is
 *   the midpoint rule on the whole cells before p_s plus the half cell up to
 *   it, sampled at its own midpoint.  A different discretisation: the ray
 *   scatter, Mie strength and surface radiance tables deviate from the
 *   reference's by up to about 1e-2 (relative) at 128 ray steps.  The
 *   transmittance table does not change. */
#define SFSIM_ATMO_SCAN_RAYS 1

/* One scattering component; mirrors the malli schema `scatter` at
 * src/clj/sfsim/atmosphere.clj:35-39.  A component without
 * ::scatter-quotient uses 1.0, one without ::scatter-g uses 0.0. */
typedef struct sfsim_atmo_component {
  double scatter_base[3];   /* scattering coefficient at height 0, 1/m, RGB */
  double scatter_scale;     /* scale height, m */
  double scatter_quotient;  /* extinction = scattering / quotient */
  double scatter_g;         /* Cornette-Shanks asymmetry */
} sfsim_atmo_component;

/* Everything that the reference hard-codes in atmosphere_lut.clj:20-63. */
typedef struct sfsim_atmo_config {
  double radius;            /* planet radius, m (atmosphere_lut.clj:20) */
  double height;            /* atmosphere height, m (atmosphere_lut.clj:21) */
  double brightness[3];     /* ground albedo (atmosphere_lut.clj:28) */
  double intensity[3];      /* sun radiance (atmosphere_lut.clj:62) */
  sfsim_atmo_component mie;       /* first entry of `scatter` */
  sfsim_atmo_component rayleigh;  /* second entry of `scatter` */
  int transmittance_shape[2];     /* [height, elevation] */
  int surface_radiance_shape[2];  /* [height, sun elevation] */
  int ray_scatter_shape[4];       /* [height, elevation, sun elevation, sun heading] */
  int ray_steps;            /* midpoint samples per ray integral */
  int sphere_steps;         /* point-scatter sphere steps (theta rings = steps/2) */
  int iterations;           /* multiple-scattering iterations after the first order */
  int precision;            /* SFSIM_ATMO_FP32 or SFSIM_ATMO_FP64 */
  int flags;                /* SFSIM_ATMO_* flag bits; 0 follows the reference */
} sfsim_atmo_config;

/* Fills `cfg` with the reference's production values
 * (atmosphere_lut.clj:20-63: R 6378 km, H 35 km, T 64x255, E 16x63,
 * S 32x127x32x8, 100 ray steps, 15 sphere steps, 5 iterations), FP32. */
void sfsim_atmo_default_config(sfsim_atmo_config* cfg);

/* Checks a configuration; 0 when it is usable. */
int sfsim_atmo_validate(const sfsim_atmo_config* cfg);

/* Number of floats in each output table (RGB included). */
int sfsim_atmo_table_sizes(const sfsim_atmo_config* cfg, size_t* n_transmittance,
                           size_t* n_surface_radiance, size_t* n_ray_scatter,
                           size_t* n_mie_strength);

/* Builds all four tables; replaces generate-atmosphere-luts
 * (atmosphere_lut.clj:43-105) up to, not including, spit-floats.
 * Output pointers are HOST memory sized by sfsim_atmo_table_sizes. */
int sfsim_atmo_build(const sfsim_atmo_config* cfg, float* transmittance,
                     float* surface_radiance, float* ray_scatter, float* mie_strength);

/* As sfsim_atmo_build, but the outputs are DEVICE pointers and the work is
 * queued on `stream` (a cudaStream_t, NULL for the legacy stream).  The call
 * returns once the work is queued.  Scratch tables stay allocated inside the
 * library between calls, keyed by device. */
int sfsim_atmo_build_device(const sfsim_atmo_config* cfg, float* transmittance,
                            float* surface_radiance, float* ray_scatter,
                            float* mie_strength, void* stream);

/* A build that allocates nothing.  No counterpart in the reference.  It is
 * for callers that cannot call cudaMalloc: engines whose own allocator
 * reserves all device memory at start-up, or that run under a fixed device
 * budget, where a library that allocates on its own would fail or break the
 * budget.  All scratch tables live in one static device array of 64 MiB
 * (67108864 bytes) that every GPU loading the library holds until the process
 * exits; a configuration that needs more (roughly 3e5 ray-scatter cells in
 * FP32, half that in FP64; the small FP64 case and the 12^4 shader-test
 * tables fit, the production tables do not) is rejected with
 * SFSIM_ATMO_ETOOBIG and a message naming the bytes it needs.  The first call
 * on a device looks up the array's device address (cudaGetSymbolAddress, with
 * that device current); make that first call before any stream capture.  The
 * parameters and quadrature directions are copied from host memory on every
 * call.  Outputs are DEVICE pointers, work is queued on `stream`, and the call
 * returns once it is queued.  Every call uses the same array, so calls that
 * overlap on the GPU (different streams, or different host threads) race and
 * corrupt each other; order them on one stream.  FP64 builds equal
 * sfsim_atmo_build_device's bit for bit.  FP32 builds integrate every sun ray
 * directly; sfsim_atmo_build_device does the same for builds whose
 * ray-scatter cells times ray steps stay below about 1.9e7 (then the tables
 * are equal) and reads the sun rays from tables above that size, where the
 * two agree within 2e-5 relative.  Stage timings are not recorded. */
int sfsim_atmo_build_static(const sfsim_atmo_config* cfg, float* transmittance,
                            float* surface_radiance, float* ray_scatter,
                            float* mie_strength, void* stream);

/* Plans: a build prepared once for one configuration on the current device
 * (its scratch allocated, its parameters and quadrature directions uploaded;
 * synchronous).  sfsim_atmo_plan_build then only launches kernels on
 * `stream` into DEVICE outputs in the .scatter layout: no allocation, copy or
 * synchronisation, so it may run inside a CUDA stream capture, and the
 * captured graph rebuilds the tables on every launch.  Asynchronous.  Builds
 * of one plan share its scratch: order them on one stream.  No counterpart in
 * the reference. */
typedef struct sfsim_atmo_plan sfsim_atmo_plan;
int sfsim_atmo_plan_create(const sfsim_atmo_config* cfg, sfsim_atmo_plan** plan);
int sfsim_atmo_plan_build(sfsim_atmo_plan* plan, float* transmittance, float* surface_radiance,
                          float* ray_scatter, float* mie_strength, void* stream);
int sfsim_atmo_plan_destroy(sfsim_atmo_plan* plan);

/* Builds `n` independent atmospheres that share shapes, steps, iterations,
 * precision and flags (they may differ in every physical parameter) in one
 * pass of batched kernels, 1 <= n <= 65535 (SFSIM_ATMO_ETOOBIG above).
 * Outputs are HOST arrays of n consecutive tables each. */
int sfsim_atmo_build_batch(const sfsim_atmo_config* cfgs, int n, float* transmittance,
                           float* surface_radiance, float* ray_scatter,
                           float* mie_strength);

/* Intermediate tables of one build, for validation.  Every pointer may be NULL.
 * 4-D tables use the plain [height][elevation][sun elevation][sun heading][3]
 * order, 2-D tables [height][second][3]; per-iteration arrays hold
 * `iterations` consecutive tables. */
typedef struct sfsim_atmo_intermediates {
  float* transmittance_nodes;   /* T sampled at the nodes, before re-interpolation */
  float* surface_base;          /* E0, surface-radiance-base table */
  float* rayleigh_first;        /* first-order Rayleigh ray scatter table */
  float* mie_first;             /* first-order Mie strength table */
  float* point_scatter;         /* J of each iteration */
  float* surface_delta;         /* dE of each iteration */
  float* ray_scatter_delta;     /* dS of each iteration */
} sfsim_atmo_intermediates;

/* As sfsim_atmo_build, and also copies intermediate tables to host memory. */
int sfsim_atmo_build_debug(const sfsim_atmo_config* cfg, float* transmittance,
                           float* surface_radiance, float* ray_scatter,
                           float* mie_strength, const sfsim_atmo_intermediates* inter);

/* The state of a build between two iterations: the four tables the loop of
 * atmosphere_lut.clj:86-97 carries from one iteration to the next (the last
 * iteration's ray-scatter and surface-radiance deltas and both sums so far),
 * as the build holds them.  Each table is one record of four values (RGB
 * and an unused fourth) per node, in [height][elevation][sun elevation]
 * [sun heading] order (4-D) or [height][sun elevation] (2-D), of the build's
 * precision: float for SFSIM_ATMO_FP32, double for SFSIM_ATMO_FP64.  They
 * are node values, before the outputs' re-interpolation, so a state saved by
 * one build resumes another build of the same config with the same results
 * as an uninterrupted build.  (The reference keeps no such state: a failed
 * run restarts from the first iteration.) */
typedef struct sfsim_atmo_iteration_state {
  int iteration;            /* iterations done, 1 .. iterations */
  void* ray_scatter_delta;  /* dS of that iteration: ray_scatter nodes x 4 values */
  void* surface_delta;      /* dE of that iteration: surface_radiance nodes x 4 */
  void* ray_scatter_sum;    /* S so far, the first-order Rayleigh term included */
  void* surface_sum;        /* E so far */
} sfsim_atmo_iteration_state;

/* Bytes of each 4-D and each 2-D table of an iteration state of `cfg`. */
int sfsim_atmo_iteration_state_bytes(const sfsim_atmo_config* cfg, size_t* ray_scatter_bytes,
                                     size_t* surface_bytes);

/* Called after each iteration with the state in host memory; a nonzero
 * return stops the build, which then returns SFSIM_ATMO_ESTOPPED without
 * writing its outputs.  It runs while the library holds its build lock, so
 * it must not call the library's build entry points. */
typedef int (*sfsim_atmo_iteration_fn)(const sfsim_atmo_iteration_state* state, void* user);

/* As sfsim_atmo_build (HOST outputs), with a state per iteration and resume.
 * resume:   NULL, or a state saved by an earlier build of the same config
 *           (iteration in 1 .. iterations); the build redoes the set-up and
 *           the first order (milliseconds) and continues with the next
 *           iteration.
 * state:    NULL, or caller-owned host buffers that receive the state after
 *           each iteration; `iteration` is set before on_iteration (which
 *           may be NULL) is called with it.  It may share `resume`'s buffers.
 * Each state costs a device-to-host copy of two 4-D and two 2-D tables and a
 * stream synchronisation. */
int sfsim_atmo_build_resumable(const sfsim_atmo_config* cfg, const sfsim_atmo_iteration_state* resume,
                               sfsim_atmo_iteration_state* state, sfsim_atmo_iteration_fn on_iteration,
                               void* user, float* transmittance, float* surface_radiance,
                               float* ray_scatter, float* mie_strength);

/* Device time of each stage of the last build, in ms, measured with CUDA
 * events on the build stream when timing is enabled.  Stage order: set-up
 * (node maps, view rows, sphere directions), transmittance, surface base,
 * first order, reserved (0), point scatter, surface radiance, ray scatter,
 * accumulate, output.  Returns the number of stages written (at most `n`);
 * for sfsim_atmo_build_device it waits for the build's last event.  With
 * timing on every stage runs on the build stream, so the stages add up to the
 * build; with timing off each iteration's surface radiance and accumulation
 * run on a second stream beside point scatter and ray scatter. */
int sfsim_atmo_set_timing(int enabled);
int sfsim_atmo_last_timings(double* ms, int n);

/* Number of kernel launches of the last build. */
int sfsim_atmo_last_launch_count(void);

/* Bytes the last build copied from host to device (its parameters and
 * quadrature directions) and from device to host (the four tables of
 * sfsim_atmo_build, plus the intermediates of sfsim_atmo_build_debug).  A plan
 * build copies nothing.  Either pointer may be NULL.  No counterpart in the
 * reference. */
int sfsim_atmo_last_transfer_bytes(unsigned long long* h2d, unsigned long long* d2h);

/* ---- Queries of a built atmosphere ---------------------------------------
 * A context builds the four tables of `cfg` on the current device and keeps
 * them, with the point-scatter tables summed over the iterations, for
 * queries.  Query inputs and outputs are DEVICE arrays of n [3] vectors; the
 * work is queued on `stream`. */
typedef struct sfsim_atmo_context sfsim_atmo_context;

int sfsim_atmo_context_create(const sfsim_atmo_config* cfg, sfsim_atmo_context** ctx);
int sfsim_atmo_context_destroy(sfsim_atmo_context* ctx);

/* Device pointers (owned by the context) of the four tables, .scatter layout. */
int sfsim_atmo_context_tables(const sfsim_atmo_context* ctx, float** transmittance,
                              float** surface_radiance, float** ray_scatter, float** mie_strength);

/* Device pointer of the point-scatter table summed over all iterations,
 * [height][elevation][sun elevation][heading][4] floats (RGB + pad); NULL
 * when the build has no iterations. */
int sfsim_atmo_context_point_scatter_sum(const sfsim_atmo_context* ctx, float** jsum);

/* Table lookups as sfsim's shaders perform them (FP32, clamped bilinear
 * texture filtering; weight_bits 0 for exact weights or 8 for GL's 8-bit
 * fixed-point weights), replacing resources/shaders/atmosphere/:
 *   kind 0  transmittance-track.glsl  transmittance_track(a, b)
 *   kind 1  transmittance-outer.glsl  transmittance_outer(a, b = direction)
 *   kind 2  ray-scatter-track.glsl    ray_scatter_track(light, a, b)
 *   kind 3  ray-scatter-outer.glsl    ray_scatter_outer(light, a, b = direction)
 *   kind 4  in-scatter S + M phase(mie g, b.light) at point a, direction b,
 *           table half chosen by is_above_horizon(a, b) */
int sfsim_atmo_query_table(const sfsim_atmo_context* ctx, int kind, long long n, const float* a,
                           const float* b, const float* light, float* out, int weight_bits,
                           void* stream);

/* Attenuation of light along view rays as sfsim's shaders compute it from the
 * tables (resources/shaders/atmosphere/, FP32, weights as in
 * sfsim_atmo_query_table), one RGBA result per query in out [n][4]:
 *   kind 0  attenuation-outer.glsl   attenuation_outer(light, p, d, s[0], incoming.rgb);
 *           alpha = incoming.a
 *   kind 1  attenuation-track.glsl   attenuation_track(light, p, d, (s[0], s[1]), incoming)
 *           (p the ray origin, d its direction, s the segment's start and length)
 *   kind 2  attenuation-point.glsl   attenuation_point(p, incoming) with the shader's
 *           uniforms origin = d (the eye) and light_direction = light
 *   kind 3  transmittance-point.glsl transmittance_point(p), uniform light_direction
 *           = light; alpha = 1
 * DEVICE arrays: light, p, d [n][3]; s [n][2]; incoming [n][4] (d, s and incoming
 * may be NULL where the kind does not read them).  `amplification` is the
 * shaders' uniform of that name. */
int sfsim_atmo_query_attenuation(const sfsim_atmo_context* ctx, int kind, long long n, const float* light,
                                 const float* p, const float* d, const float* s, const float* incoming,
                                 float amplification, float* out, int weight_bits, void* stream);

/* Rendered in-scatter S + M phase(mie g, v.l) at position x, unit view v and
 * unit sun l (FP64 inputs) by direct quadrature, without the 4-D table: the
 * first order integrated at the point as atmosphere.clj:154-200 does, plus
 * ray scatter of the summed point-scatter table (the higher orders). */
int sfsim_atmo_query_direct(const sfsim_atmo_context* ctx, long long n, const double* x,
                            const double* v, const double* l, float* out, void* stream);

/* The surrogate's ten coordinates in [0, 1] of (x, v, l): the table
 * coordinates height, elevation, sun elevation and sun heading as
 * core/ray-scatter-forward.glsl forms them (FP32), with the table half chosen
 * by is_above_horizon; then (1 + sin of the sun elevation) / 2 without the
 * lookup's clamp, the table half (0 upper, 1 lower), and the four cell phases
 * frac(coordinate * (size - 1)) of the lookup.  coords is a DEVICE [n][10]. */
int sfsim_atmo_query_coords(const sfsim_atmo_context* ctx, long long n, const double* x, const double* v,
                            const double* l, float* coords, void* stream);

/* ---- Surrogate of the rendered in-scatter ----------------------------------
 * An MLP over ten coordinates in [0, 1] of a query (sfsim_atmo_query_coords:
 * the four table coordinates as the in-scatter lookup forms them, the
 * unclamped sun elevation, the table half and the four cell phases): sin/cos
 * Fourier features (256) -> 4 x 256 SiLU -> 4 outputs, three log-space
 * corrections to the table lookup and the log of their expected squared
 * error (sfsim_atmo_surrogate_parameters).  BF16 weights and activations,
 * FP32 accumulation and master weights; the hidden layers run on tcgen05
 * tensor cores in the forward and both backward GEMMs.  No counterpart in the
 * reference. */
typedef struct sfsim_atmo_surrogate_config {
  int steps;                /* Adam steps */
  int batch;                /* rows per step, a multiple of 1024 */
  long long direct_samples; /* off-grid training points integrated by sfsim_atmo_query_direct */
  float node_fraction;      /* share of each batch drawn from the table nodes */
  float lr;                 /* initial learning rate, cosine decay to 0 */
  unsigned long long seed;
  float huber_delta;        /* > 0: Huber loss of the corrections with this threshold; 0: squared error */
} sfsim_atmo_surrogate_config;

/* Trains (or continues training) the context's surrogate on the GPU;
 * loss_history (host, `steps` floats, may be NULL) receives each step's loss.
 * Returns SFSIM_ATMO_ENUMERIC when the run diverged (a non-finite last loss;
 * learning rates above about 3e-3 can do that at batch 65536). */
int sfsim_atmo_surrogate_train(sfsim_atmo_context* ctx, const sfsim_atmo_surrogate_config* cfg,
                               float* loss_history);

/* Parameter vector (FP32, W1 [256][256], b1, W2, b2, W3, b3, W4, b4 [256][256],
 * W5 [4][256], b5 [4]): *count receives its length; `get` copies it out, `set`
 * replaces it (host arrays, either may be NULL).  Outputs 0-2 are corrections
 * r = log(value + 1e-7) - log(table + 1e-7) to the in-scatter lookup, output 3
 * the log of their expected squared error. */
int sfsim_atmo_surrogate_parameters(sfsim_atmo_context* ctx, float* get, const float* set, long long* count);

/* Loss (mean squared error of the corrections) and parameter gradients of
 * one batch (host coords [n][10], target corrections [n][3]; n a multiple of
 * 1024) without updating, for validation.  The gradients also carry the
 * Gaussian negative log-likelihood of the squared error under the predicted
 * variance, weighted 0.01. */
int sfsim_atmo_surrogate_gradients(sfsim_atmo_context* ctx, long long n, const float* coords,
                                   const float* targets, float* loss, float* grads);

/* Rendered in-scatter at (x, v, l) from the surrogate (DEVICE arrays as in
 * sfsim_atmo_query_direct), one fused tensor-core kernel: coordinates, the
 * table lookup, features, the four hidden layers (tcgen05 MMA into tensor
 * memory) and the head per 256 queries; the value is the lookup corrected by
 * the network, (table + 1e-7) exp(r) - 1e-7.  With threshold > 0, points whose
 * predicted relative error (the square root of the variance output) exceeds
 * `threshold` are recomputed by direct quadrature; *n_fallback receives their
 * number.  Without a threshold the call is asynchronous on `stream`; with one
 * it synchronises and also reports a tensor-core wait that timed out. */
int sfsim_atmo_query_surrogate(sfsim_atmo_context* ctx, long long n, const double* x, const double* v,
                               const double* l, float* out, float threshold, long long* n_fallback,
                               void* stream);

/* ---- Conditioned surrogate ------------------------------------------------
 * One network for a family of atmospheres: the surrogate above whose first
 * layer also takes eight inputs describing the atmosphere (z1 = W1 F + b1 +
 * U g with U [256][8]).  It is trained on several contexts at once and
 * corrects the table lookup of any context, including atmospheres it was not
 * trained on.  No counterpart in the reference. */
typedef struct sfsim_atmo_cond_surrogate sfsim_atmo_cond_surrogate;

/* The eight inputs g of an atmosphere, each about [-1, 1] over the
 * parameter sweep: log2 of the Rayleigh coefficients (RGB) relative to
 * (5.8, 13.5, 33.1)e-6 /m, log2 of the red Mie coefficient relative to
 * 2e-5 /m, (Rayleigh scale height - 8 km) / 2 km, (Mie scale height -
 * 1.4 km) / 0.6 km, (Mie g - 0.725) / 0.125, (radius - 5000 km) / 2000 km;
 * each clamped to [-8, 8].  Host-only. */
int sfsim_atmo_condition_inputs(const sfsim_atmo_config* cfg, float* inputs);

/* Creates an untrained conditioned surrogate on the current device
 * (Xavier-uniform weights from `seed`, U zero). */
int sfsim_atmo_cond_surrogate_create(unsigned long long seed, sfsim_atmo_cond_surrogate** out);
int sfsim_atmo_cond_surrogate_destroy(sfsim_atmo_cond_surrogate* cs);

/* Trains on n_ctx (1..256) FP32 contexts sharing one ray-scatter shape.  Each
 * batch row picks a context uniformly, then a sample of it as
 * sfsim_atmo_surrogate_train draws one; `direct_samples` counts per context. */
int sfsim_atmo_cond_surrogate_train(sfsim_atmo_cond_surrogate* cs, sfsim_atmo_context* const* ctxs, int n_ctx,
                                    const sfsim_atmo_surrogate_config* cfg, float* loss_history);

/* Parameter vector: the surrogate's (sfsim_atmo_surrogate_parameters) followed
 * by U [256][8]. */
int sfsim_atmo_cond_surrogate_parameters(sfsim_atmo_cond_surrogate* cs, float* get, const float* set,
                                         long long* count);

/* Loss and gradients of one batch as sfsim_atmo_surrogate_gradients, row i
 * belonging to group groups[i] < n_groups whose eight inputs are
 * inputs[groups[i]][0..7] (host arrays). */
int sfsim_atmo_cond_surrogate_gradients(sfsim_atmo_cond_surrogate* cs, long long n, const float* coords,
                                        const int* groups, int n_groups, const float* inputs, const float* targets,
                                        float* loss, float* grads);

/* Rendered in-scatter of the atmosphere `ctx` as sfsim_atmo_query_surrogate
 * computes it, with the conditioned network at ctx's inputs (folded into the
 * first-layer bias, so the fused kernel is the same).  Calls on one
 * surrogate are ordered on one stream. */
int sfsim_atmo_query_cond_surrogate(sfsim_atmo_cond_surrogate* cs, const sfsim_atmo_context* ctx, long long n,
                                    const double* x, const double* v, const double* l, float* out, float threshold,
                                    long long* n_fallback, void* stream);

/* The surrogate's tensor-core GEMM, exposed for validation: C = A * B^T with
 * A [M][K] and B [N][K] row-major bf16 DEVICE arrays and C [M][N] float,
 * FP32 accumulation on tcgen05 tensor cores.  N <= 256; K a multiple of
 * 64 * splits; splits > 1 divides K over CTAs and sums into C atomically. */
int sfsim_atmo_gemm_bf16(const void* A, const void* B, float* C, int M, int N, long long K, int splits,
                         void* stream);

/* Poll limit of every mbarrier wait in the tensor-core kernels (the
 * surrogate's training GEMMs and its fused inference).  A wait that is not
 * satisfied within `polls` polls gives up: the CTA records an error, tells
 * its other warps to stop (their waits give up too), waits for the copies
 * and MMAs it has in flight, frees its tensor memory and returns; the next
 * synchronising call (training, gradients, a query with a threshold) returns
 * SFSIM_ATMO_ECUDA.  polls <= 0 restores the default, 4194304.  Returns the
 * limit that was in force.  Applies to launches after the call.  No
 * counterpart in the reference. */
long long sfsim_atmo_set_wait_limit(long long polls);

/* Self-test of that timeout path, for validation: launches the GEMM kernel of
 * sfsim_atmo_gemm_bf16 once (one CTA, 128 x 256 x 4096 zero operands that it
 * allocates) with its epilogue first waiting `polls` polls (1 .. 1000000) on
 * an mbarrier that nothing arrives on, and synchronises.  That wait gives up
 * and the kernel returns through the path above, so the call returns
 * SFSIM_ATMO_ECUDA with a message naming the timed-out wait; the device and
 * the library stay usable.  A return of 0 would mean the wait did not time
 * out.  No counterpart in the reference. */
int sfsim_atmo_wait_selftest(int polls);

/* Work census of one build (no tables are written).  counts[0] = first-order
 * sun-ray integrals (node, ray-sample pairs with the sun above the sample's
 * horizon), [1] = their extinction samples, [2] = view-ray extinction
 * samples, [3] = point-scatter direction evaluations, [4] = ray-scatter
 * J lookups, [5] = surface-radiance direction evaluations, [6] = the pairs
 * of [0] whose sun ray climbs (FP32 builds whose ray-scatter cells times ray
 * steps exceed about 1.9e7 read the optical depths of every pair of [0] from
 * two tables, one for climbing and one for descending sun rays, instead of
 * integrating them; smaller builds integrate them), [7] = the point-scatter
 * direction
 * evaluations of [3] that end on the ground, [8] = those of the first
 * iteration (which also reads the Mie strength), [9] = those of [7] whose
 * ground point has height coordinate exactly 0 in the surface-radiance
 * table (their dE lookup reads one height row).  Returns the number of
 * counts written (at most n). */
int sfsim_atmo_census(const sfsim_atmo_config* cfg, unsigned long long* counts, int n);

/* Measures the SFU throughput of the current device (ex2.approx.f32
 * operations per second, best of 4 timed launches over all SMs), the
 * denominator of the quadrature kernels' roofline. */
int sfsim_atmo_sfu_peak(double* ex2_per_second);

/* Measured shared-memory read bandwidth of this GPU (bytes per second, all
 * SMs, conflict-free 16-byte reads), the roofline denominator of the
 * shared-memory-gather kernels (point scatter).  No counterpart in the
 * reference. */
int sfsim_atmo_smem_peak(double* bytes_per_second);

/* Frees the cached scratch tables of the current device. */
int sfsim_atmo_release(void);

/* Text for an error code. */
const char* sfsim_atmo_strerror(int code);

/* Detailed message of the last failure on the calling thread. */
const char* sfsim_atmo_last_error(void);

/* Library version string. */
const char* sfsim_atmo_version(void);

#ifdef __cplusplus
}
#endif

#endif /* SFSIM_ATMO_H */
