/*
 * noise_oracle.h -- the FP64 CPU restatement of sfsim's cloud-noise
 * builders (test infrastructure only; see noise_oracle.c).
 */
#ifndef NOISE_ORACLE_H
#define NOISE_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* grid: [divisions]^3 points (x, y, z), grid[k][j][i]; out: size^3 */
void noise_worley(int divisions, int size, const double* grid, double* out);
double noise_worley_closest(const double* grid, int divisions, int size, const double* point);
/* the same on a grid of nk x nj x ni cells (the reference's unit facts use such grids) */
double noise_worley_closest_grid(const double* grid, int nk, int nj, int ni, int divisions, int size,
                                 const double* point);

/* gradients: [divisions]^3 indices 0..11 into the twelve gradient vectors */
void noise_perlin(int divisions, int size, const int* gradients, double* out);
double noise_perlin_sample(const int* gradients, int divisions, int size, const double* cell);
double noise_perlin_ease(double t);
void noise_perlin_gradient(int index, double* g);

/* void and cluster on an m x m torus from the n seed pixels; dither: m*m ranks */
int noise_blue(int m, int n, const int* seed, double sigma, int* dither);
int noise_blue_wrap(int x, int m);
double noise_blue_density(double sigma, int dx, int dy);
void noise_blue_table(int m, double sigma, double* table);
void noise_blue_density_array(const unsigned char* mask, int m, const double* table, double* density);
void noise_blue_seed_pattern(unsigned char* mask, int m, const double* table);
void noise_blue_phase(int phase, unsigned char* mask, int m, int n, double sigma, int* dither);

#ifdef __cplusplus
}
#endif

#endif
