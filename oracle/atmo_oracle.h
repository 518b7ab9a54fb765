/*
 * atmo_oracle.h -- exported functions of the FP64 CPU oracle (test
 * infrastructure only; see atmo_oracle.c).
 */
#ifndef ATMO_ORACLE_H
#define ATMO_ORACLE_H

#include "../include/sfsim_atmo.h"

#ifdef __cplusplus
extern "C" {
#endif

/* planet map of the reference: :sfsim.sphere/centre, :sfsim.sphere/radius,
 * :sfsim.atmosphere/height, :sfsim.atmosphere/brightness */
typedef struct {
  double centre[3];
  double radius;
  double height;
  double brightness[3];
} oracle_planet;

/* scatter component: base, scale, quotient (1.0 if absent), g (0.0 if absent) */
typedef struct {
  double base[3];
  double scale;
  double quotient;
  double g;
} oracle_component;

/* Optional intermediate tables (doubles, plain [..][3] order). */
typedef struct {
  double* transmittance_nodes;
  double* surface_base;
  double* rayleigh_first;
  double* mie_first;
  double* point_scatter;      /* iterations x 4-D */
  double* surface_delta;      /* iterations x 2-D */
  double* ray_scatter_delta;  /* iterations x 4-D */
} oracle_intermediates;

/* Whole build (atmosphere_lut.clj:43-105); outputs in the .scatter layout. */
int oracle_build(const sfsim_atmo_config* cfg, int nthreads, double* T_out, double* E_out, double* S_out,
                 double* M_out, const oracle_intermediates* inter);

/* Single nodes against supplied tables ([..][3] doubles, plain order). */
void oracle_transmittance_node(const sfsim_atmo_config* cfg, int i, int j, double* out);
void oracle_surface_base_node(const sfsim_atmo_config* cfg, int i, int k, double* out);
void oracle_first_order_node(const sfsim_atmo_config* cfg, int i, int j, int k, int a, double* rayleigh,
                             double* mie);
void oracle_point_scatter_node(const sfsim_atmo_config* cfg, const double* dS, const double* mie_first,
                               const double* dE, int i, int j, int k, int a, double* out);
void oracle_ray_scatter_node(const sfsim_atmo_config* cfg, const double* J, int i, int j, int k, int a,
                             double* out);
void oracle_surface_radiance_node(const sfsim_atmo_config* cfg, const double* dS, const double* mie_first, int i,
                                  int k, double* out);
void oracle_remap4_node(const sfsim_atmo_config* cfg, const double* table, int i, int j, int k, int a,
                        double* out);

/* Rendered in-scatter S + M phase at an arbitrary (x, v, l); Jsum is the
 * point-scatter table summed over the iterations or NULL. */
void oracle_rendered_inscatter(const sfsim_atmo_config* cfg, const double* Jsum, const double* x, const double* v,
                               const double* l, double* out);

/* Tables for the GLSL restatement. */
typedef struct {
  float radius, max_height;
  int t_height_size, t_elevation_size;
  int height_size, elevation_size, light_elevation_size, heading_size;
  const float* transmittance;
  const float* ray_scatter;
  const float* mie_strength;
  int weight_bits;
} oracle_glsl_tables;

void oracle_glsl_query(const oracle_glsl_tables* t, int kind, const float* light, const float* p, const float* q,
                       float* out);
void oracle_glsl_query_batch(const oracle_glsl_tables* t, int kind, long n, const float* light, const float* p,
                             const float* q, float* out, int* above);
/* n attenuation queries of atmosphere/attenuation-*.glsl and
 * transmittance-point.glsl (kinds 0-3; see atmo_oracle.c). */
void oracle_glsl_attenuation_batch(const oracle_glsl_tables* t, int kind, long n, const float* light, const float* p,
                                   const float* d, const float* s, const float* incoming, float amplification,
                                   float* out);

#ifdef __cplusplus
}
#endif

#endif
