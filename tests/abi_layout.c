/* Prints the byte layout of the configuration structs that include/sfsim_atmo.h
 * declares: one line "name offset size" per field, flattened (nested
 * component fields as mie.scatter_base ...), then "sizeof N".  A binding on
 * the other side of the C ABI (coffi in Clojure, ctypes in Python) must lay
 * the struct out the same way; tests/test_abi_layout.py compares them. */
#include <stddef.h>
#include <stdio.h>

#include "sfsim_atmo.h"

#define FIELD(path, member) \
  printf("%s %zu %zu\n", path, offsetof(sfsim_atmo_config, member), sizeof(((sfsim_atmo_config*)0)->member))

int main(void) {
  FIELD("radius", radius);
  FIELD("height", height);
  FIELD("brightness", brightness);
  FIELD("intensity", intensity);
  FIELD("mie.scatter_base", mie.scatter_base);
  FIELD("mie.scatter_scale", mie.scatter_scale);
  FIELD("mie.scatter_quotient", mie.scatter_quotient);
  FIELD("mie.scatter_g", mie.scatter_g);
  FIELD("rayleigh.scatter_base", rayleigh.scatter_base);
  FIELD("rayleigh.scatter_scale", rayleigh.scatter_scale);
  FIELD("rayleigh.scatter_quotient", rayleigh.scatter_quotient);
  FIELD("rayleigh.scatter_g", rayleigh.scatter_g);
  FIELD("transmittance_shape", transmittance_shape);
  FIELD("surface_radiance_shape", surface_radiance_shape);
  FIELD("ray_scatter_shape", ray_scatter_shape);
  FIELD("ray_steps", ray_steps);
  FIELD("sphere_steps", sphere_steps);
  FIELD("iterations", iterations);
  FIELD("precision", precision);
  FIELD("flags", flags);
  printf("sizeof %zu\n", sizeof(sfsim_atmo_config));
  printf("component_sizeof %zu\n", sizeof(sfsim_atmo_component));
  return 0;
}
