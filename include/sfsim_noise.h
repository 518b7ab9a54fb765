/*
 * sfsim_noise.h -- C ABI of the GPU cloud-noise table builders in
 * libsfsim_atmo.so (sm_103a).
 *
 * These replace the bodies of the reference's offline build tasks `worley`,
 * `perlin` and `bluenoise` (build.clj:34-51): the random inputs stay on the
 * host (the caller draws them, as the reference's tests inject them), the
 * per-voxel and per-pixel work runs on the GPU.  All arrays are HOST memory;
 * every call is synchronous.  Return codes are the SFSIM_ATMO_E* codes of
 * sfsim_atmo.h; sfsim_atmo_last_error() holds the message.
 */
#ifndef SFSIM_NOISE_H
#define SFSIM_NOISE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Worley noise, replaces worley-noise (src/clj/sfsim/worley.clj:96-109)
 * after random-point-grid (:27-46).  grid: [divisions]^3 points (x, y, z) in
 * [k][j][i] order, the point of cell (i, j, k) inside
 * [i, i+1) x [j, j+1) x [k, k+1) times size/divisions; size must be a
 * multiple of divisions.  out: size^3 floats in the reference's order
 * (index (k size + j) size + i holds the voxel centre (k, j, i) + 0.5),
 * 1 - distance / maximum distance. */
int sfsim_noise_worley(int divisions, int size, const double* grid, float* out);

/* Perlin noise, replaces perlin-noise (src/clj/sfsim/perlin.clj:122-133)
 * after random-gradient-grid (:37-48).  gradients: [divisions]^3 indices
 * 0..11 into the twelve gradient vectors of random-gradient (:24-34), in
 * [z][y][x] order.  out: size^3 floats, index (k size + j) size + i holds
 * the sample at (i, j, k) + 0.5, scaled to [0, 1]. */
int sfsim_noise_perlin(int divisions, int size, const int* gradients, float* out);

/* Blue noise by void and cluster, replaces blue-noise
 * (src/clj/sfsim/bluenoise.clj:162-172).  seed: the n distinct pixel
 * indices in [0, m*m) that pick-n chose, 1 <= n <= m*m/2, 2 <= m <= 256; sigma: the width of the Gauss
 * density function.  dither: m*m ranks (the reference's dither array).  The
 * densities are FP64 with the reference's order of operations per pixel. */
int sfsim_noise_blue(int m, int n, const int* seed, double sigma, int* dither);

#ifdef __cplusplus
}
#endif

#endif
