/* A native caller of the C ABI: builds the small FP32 tables through
 * sfsim_atmo_build with host buffers, as sfsim's Clojure host would through
 * coffi, and writes them to the file named by argv[1] (transmittance,
 * surface radiance, ray scatter, Mie strength, float32, one after another).
 * Exit status 0 on success; on failure the library's message goes to stderr. */
#include <stdio.h>
#include <stdlib.h>

#include "sfsim_atmo.h"

int main(int argc, char** argv) {
  if (argc < 2) return 2;
  sfsim_atmo_config cfg;
  sfsim_atmo_default_config(&cfg);
  cfg.height = 100000.0;
  cfg.transmittance_shape[0] = 32, cfg.transmittance_shape[1] = 32;
  cfg.surface_radiance_shape[0] = 16, cfg.surface_radiance_shape[1] = 32;
  cfg.ray_scatter_shape[0] = 8, cfg.ray_scatter_shape[1] = 16;
  cfg.ray_scatter_shape[2] = 8, cfg.ray_scatter_shape[3] = 4;
  cfg.ray_steps = 64;
  cfg.sphere_steps = 16;
  cfg.iterations = 2;
  cfg.precision = SFSIM_ATMO_FP32;
  size_t n[4];
  if (sfsim_atmo_table_sizes(&cfg, &n[0], &n[1], &n[2], &n[3])) return 3;
  float* t[4];
  for (int i = 0; i < 4; i++) {
    t[i] = (float*)malloc(sizeof(float) * n[i]);
    if (!t[i]) return 4;
  }
  int rc = sfsim_atmo_build(&cfg, t[0], t[1], t[2], t[3]);
  if (rc) {
    fprintf(stderr, "%s: %s\n", sfsim_atmo_strerror(rc), sfsim_atmo_last_error());
    return 5;
  }
  FILE* f = fopen(argv[1], "wb");
  if (!f) return 6;
  for (int i = 0; i < 4; i++) fwrite(t[i], sizeof(float), n[i], f);
  fclose(f);
  for (int i = 0; i < 4; i++) free(t[i]);
  return 0;
}
