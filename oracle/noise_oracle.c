/*
 * noise_oracle.c -- FP64 CPU restatement of sfsim's cloud-noise table
 * builders (test infrastructure only: the checker of the GPU kernels in
 * sfsim_gb300/csrc/k_noise.cu, never a product path).
 *
 * Followed line by line:
 *   Worley noise   src/clj/sfsim/worley.clj:27-109
 *   Perlin noise   src/clj/sfsim/perlin.clj:24-133
 *   blue noise     src/clj/sfsim/bluenoise.clj:25-176 (void and cluster,
 *                  Ulichney 1993)
 * The reference draws its random inputs inside the builders (rand,
 * rand-nth, shuffle); here they are arguments, as the reference's own tests
 * inject them (random-point-grid with `random`, random-gradient-grid with a
 * selector, pick-n with `order`).
 */
#include "noise_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* ---------------------------------------------------------------- Worley */

/* clipped-index-and-offset, worley.clj:49-56: an index one beyond either end
 * of the grid wraps around and shifts the point by the texture size. */
static void clipped_index_and_offset(int divisions, int size, int index, int* clipped, double* offset) {
  if (index < divisions) {
    if (index >= 0) {
      *clipped = index;
      *offset = 0.0;
    } else {
      *clipped = index + divisions;
      *offset = -(double)size;
    }
  } else {
    *clipped = index - divisions;
    *offset = (double)size;
  }
}

/* extract-point-from-grid, worley.clj:59-66; grid[k][j][i] holds (x, y, z)
 * and has nk x nj x ni cells. */
static void extract_point(const double* grid, int nk, int nj, int ni, int size, int k, int j, int i, double* p) {
  int ic, jc, kc;
  double xo, yo, zo;
  clipped_index_and_offset(ni, size, i, &ic, &xo);
  clipped_index_and_offset(nj, size, j, &jc, &yo);
  clipped_index_and_offset(nk, size, k, &kc, &zo);
  const double* q = grid + 3 * (((size_t)kc * nj + jc) * ni + ic);
  p[0] = q[0] + xo;
  p[1] = q[1] + yo;
  p[2] = q[2] + zo;
}

/* closest-distance-to-point-in-grid, worley.clj:69-79. */
double noise_worley_closest_grid(const double* grid, int nk, int nj, int ni, int divisions, int size,
                                 const double* point) {
  const double cellsize = (double)(size / divisions);
  /* (long (quot x cellsize)): truncation toward zero */
  const int i = (int)trunc(point[0] / cellsize), j = (int)trunc(point[1] / cellsize),
            k = (int)trunc(point[2] / cellsize);
  double best = INFINITY;
  for (int dk = -1; dk <= 1; dk++)
    for (int dj = -1; dj <= 1; dj++)
      for (int di = -1; di <= 1; di++) {
        double p[3];
        extract_point(grid, nk, nj, ni, size, k + dk, j + dj, i + di, p);
        const double dx = point[0] - p[0], dy = point[1] - p[1], dz = point[2] - p[2];
        const double d = sqrt(dx * dx + dy * dy + dz * dz);
        if (d < best) best = d;
      }
  return best;
}

double noise_worley_closest(const double* grid, int divisions, int size, const double* point) {
  return noise_worley_closest_grid(grid, divisions, divisions, divisions, divisions, size, point);
}

/* worley-noise, worley.clj:96-109: closest distances at the cell centres in
 * pfor order [k j i] with the point (k + 0.5, j + 0.5, i + 0.5), scaled by
 * their maximum (normalize-vector, :82-87) and inverted (:90-93). */
void noise_worley(int divisions, int size, const double* grid, double* out) {
  const size_t n = (size_t)size * size * size;
  double maximum = -INFINITY;
  for (int k = 0; k < size; k++)
    for (int j = 0; j < size; j++)
      for (int i = 0; i < size; i++) {
        const double p[3] = {k + 0.5, j + 0.5, i + 0.5};
        const double d = noise_worley_closest(grid, divisions, size, p);
        out[((size_t)k * size + j) * size + i] = d;
        if (d > maximum) maximum = d;
      }
  for (size_t t = 0; t < n; t++) out[t] = 1.0 - out[t] / maximum;
}

/* ---------------------------------------------------------------- Perlin */

/* the twelve gradient vectors of random-gradient, perlin.clj:24-34 */
static const double kGradients[12][3] = {{1, 1, 0},  {-1, 1, 0},  {1, -1, 0}, {-1, -1, 0},
                                         {1, 0, 1},  {-1, 0, 1},  {1, 0, -1}, {-1, 0, -1},
                                         {0, 1, 1},  {0, -1, 1},  {0, 1, -1}, {0, -1, -1}};

void noise_perlin_gradient(int index, double* g) {
  g[0] = kGradients[index][0];
  g[1] = kGradients[index][1];
  g[2] = kGradients[index][2];
}

/* ease-curve, perlin.clj:85-88: ((6 t - 15) t + 10) t t t, left to right */
double noise_perlin_ease(double t) { return (((t * 6.0 - 15.0) * t + 10.0) * t) * t * t; }

/* perlin-noise-sample, perlin.clj:111-119, with corner-vectors (:58-64),
 * corner-gradients (:67-74, the upper corner wraps modulo the grid),
 * influence-values (:77-80) and interpolation-weights (:91-100);
 * gradients[z][y][x] index the twelve vectors. */
double noise_perlin_sample(const int* gradients, int divisions, int size, const double* cell) {
  const double scale = (double)divisions / (double)size;
  const double p[3] = {cell[0] * scale, cell[1] * scale, cell[2] * scale};
  const int x = (int)floor(p[0]), y = (int)floor(p[1]), z = (int)floor(p[2]);
  const int xs[2] = {x, (x + 1) % divisions}, ys[2] = {y, (y + 1) % divisions}, zs[2] = {z, (z + 1) % divisions};
  const double f[3] = {p[0] - x, p[1] - y, p[2] - z};
  double sum = 0.0;
  int c = 0;
  for (int zc = 0; zc < 2; zc++)
    for (int yc = 0; yc < 2; yc++)
      for (int xc = 0; xc < 2; xc++, c++) {
        const double v[3] = {p[0] - (x + xc), p[1] - (y + yc), p[2] - (z + zc)};
        double g[3];
        noise_perlin_gradient(gradients[((size_t)zs[zc] * divisions + ys[yc]) * divisions + xs[xc]], g);
        const double influence = g[0] * v[0] + g[1] * v[1] + g[2] * v[2];
        const double wz = noise_perlin_ease(zc ? f[2] : 1.0 - f[2]);
        const double wy = noise_perlin_ease(yc ? f[1] : 1.0 - f[1]);
        const double wx = noise_perlin_ease(xc ? f[0] : 1.0 - f[0]);
        const double w = wz * wy * wx;
        sum = c == 0 ? w * influence : sum + w * influence;
      }
  return sum;
}

/* perlin-noise, perlin.clj:122-133: samples at (i + 0.5, j + 0.5, k + 0.5) in
 * pfor order [k j i], scaled to [0, 1] (normalize-vector, :103-108). */
void noise_perlin(int divisions, int size, const int* gradients, double* out) {
  const size_t n = (size_t)size * size * size;
  double lo = INFINITY, hi = -INFINITY;
  for (int k = 0; k < size; k++)
    for (int j = 0; j < size; j++)
      for (int i = 0; i < size; i++) {
        const double cell[3] = {i + 0.5, j + 0.5, k + 0.5};
        const double v = noise_perlin_sample(gradients, divisions, size, cell);
        out[((size_t)k * size + j) * size + i] = v;
        if (v < lo) lo = v;
        if (v > hi) hi = v;
      }
  for (size_t t = 0; t < n; t++) out[t] = (out[t] - lo) / (hi - lo);
}

/* ------------------------------------------------------------ blue noise */

/* wrap, bluenoise.clj:72-76: x into [-m/2, m/2) */
int noise_blue_wrap(int x, int m) {
  const int offset = m / 2;
  int r = (x + offset) % m;
  if (r < 0) r += m;
  return r - offset;
}

/* density-function, bluenoise.clj:50-53 */
double noise_blue_density(double sigma, int dx, int dy) {
  return exp(-((double)(dx * dx + dy * dy) / (2.0 * sigma * sigma)));
}

/* Gauss weights by |dx|, |dy| (both at most m/2): the table the GPU reads. */
void noise_blue_table(int m, double sigma, double* table) {
  const int h = m / 2 + 1;
  for (int y = 0; y < h; y++)
    for (int x = 0; x < h; x++) table[y * h + x] = noise_blue_density(sigma, x, y);
}

static double f_at(const double* table, int m, int dx, int dy) {
  const int h = m / 2 + 1;
  return table[abs(dy) * h + abs(dx)];
}

/* argmax-with-mask / argmin-with-mask, bluenoise.clj:56-69: max-key and
 * min-key return the last of equal elements. */
static int argmax_mask(const double* a, const unsigned char* mask, int n) {
  int best = -1;
  for (int t = 0; t < n; t++)
    if (mask[t] && (best < 0 || a[t] >= a[best])) best = t;
  return best;
}
static int argmin_mask(const double* a, const unsigned char* mask, int n) {
  int best = -1;
  for (int t = 0; t < n; t++)
    if (!mask[t] && (best < 0 || a[t] <= a[best])) best = t;
  return best;
}

/* density-array with density-sample, bluenoise.clj:79-96: per pixel, the sum
 * over set pixels in row-major order */
static void density_array(const unsigned char* mask, int m, const double* table, double* density) {
  for (int cy = 0; cy < m; cy++)
    for (int cx = 0; cx < m; cx++) {
      double s = 0.0;
      for (int y = 0; y < m; y++)
        for (int x = 0; x < m; x++)
          if (mask[y * m + x]) s += f_at(table, m, noise_blue_wrap(x - cx, m), noise_blue_wrap(y - cy, m));
      density[cy * m + cx] = s;
    }
}

/* density-change, bluenoise.clj:99-109 */
static void density_change(double* density, int m, int sign, const double* table, int index) {
  const int cy = index / m, cx = index % m;
  for (int y = 0; y < m; y++)
    for (int x = 0; x < m; x++) {
      const double f = f_at(table, m, noise_blue_wrap(x - cx, m), noise_blue_wrap(y - cy, m));
      if (sign > 0)
        density[y * m + x] += f;
      else
        density[y * m + x] -= f;
    }
}

/* seed-pattern, bluenoise.clj:112-124 */
static void seed_pattern(unsigned char* mask, int m, const double* table, double* density) {
  const int n = m * m;
  density_array(mask, m, table, density);
  for (;;) {
    const int cluster = argmax_mask(density, mask, n);
    mask[cluster] = 0;
    density_change(density, m, -1, table, cluster);
    const int vd = argmin_mask(density, mask, n);
    mask[vd] = 1;
    if (cluster == vd) return;
    density_change(density, m, +1, table, vd);
  }
}

/* dither-phase1, bluenoise.clj:127-140: remove the n set pixels of mask,
 * tightest cluster first, with ranks n-1 .. 0; mask and density change. */
static void phase1(unsigned char* mask, int m, int n, const double* table, double* density, int* dither) {
  for (int r = n; r > 0; r--) {
    const int cluster = argmax_mask(density, mask, m * m);
    density_change(density, m, -1, table, cluster);
    mask[cluster] = 0;
    dither[cluster] = r - 1;
  }
}

/* dither-phase2, bluenoise.clj:143-154: fill the largest voids with ranks
 * n .. m*m/2 - 1; mask and density change. */
static void phase2(unsigned char* mask, int m, int n, const double* table, double* density, int* dither) {
  for (int r = n; r < m * m / 2; r++) {
    const int vd = argmin_mask(density, mask, m * m);
    density_change(density, m, +1, table, vd);
    mask[vd] = 1;
    dither[vd] = r;
  }
}

/* dither-phase3, bluenoise.clj:157-169: on the complement of mask, remove the
 * tightest clusters with ranks n .. m*m - 1; mask is complemented in place. */
static void phase3(unsigned char* mask, int m, int n, const double* table, double* density, int* dither) {
  for (int t = 0; t < m * m; t++) mask[t] = !mask[t];
  density_array(mask, m, table, density);
  for (int r = n; r < m * m; r++) {
    const int cluster = argmax_mask(density, mask, m * m);
    density_change(density, m, -1, table, cluster);
    mask[cluster] = 0;
    dither[cluster] = r;
  }
}

/* blue-noise, bluenoise.clj:162-172.  seed holds the n pixel indices pick-n
 * chose; dither receives m*m ranks. */
int noise_blue(int m, int n, const int* seed, double sigma, int* dither) {
  const int total = m * m;
  unsigned char* mask = calloc(total, 1);
  unsigned char* work = calloc(total, 1);
  double* table = malloc(sizeof(double) * (m / 2 + 1) * (m / 2 + 1));
  double* density0 = malloc(sizeof(double) * total);
  double* density = malloc(sizeof(double) * total);
  if (!mask || !work || !table || !density0 || !density) {
    free(mask), free(work), free(table), free(density0), free(density);
    return -1;
  }
  noise_blue_table(m, sigma, table);
  for (int t = 0; t < n; t++) mask[seed[t]] = 1;
  seed_pattern(mask, m, table, density);
  density_array(mask, m, table, density0);
  memset(dither, 0, sizeof(int) * total);
  memcpy(work, mask, total);
  memcpy(density, density0, sizeof(double) * total);
  phase1(work, m, n, table, density, dither);
  memcpy(work, mask, total);
  memcpy(density, density0, sizeof(double) * total);
  phase2(work, m, n, table, density, dither);
  phase3(work, m, total / 2, table, density, dither);
  free(mask), free(work), free(table), free(density0), free(density);
  return 0;
}

/* One phase from a mask (the reference's shorter arities, which start from
 * density-array of the mask): phase 1, 2 or 3. */
void noise_blue_phase(int phase, unsigned char* mask, int m, int n, double sigma, int* dither) {
  double* table = malloc(sizeof(double) * (m / 2 + 1) * (m / 2 + 1));
  double* density = malloc(sizeof(double) * m * m);
  if (table && density) {
    noise_blue_table(m, sigma, table);
    if (phase == 3) {
      phase3(mask, m, n, table, density, dither);
    } else {
      density_array(mask, m, table, density);
      if (phase == 1) phase1(mask, m, n, table, density, dither);
      else phase2(mask, m, n, table, density, dither);
    }
  }
  free(table), free(density);
}

/* Unit pieces for the reference's facts. */
void noise_blue_density_array(const unsigned char* mask, int m, const double* table, double* density) {
  density_array(mask, m, table, density);
}
void noise_blue_seed_pattern(unsigned char* mask, int m, const double* table) {
  double* density = malloc(sizeof(double) * m * m);
  if (!density) return;
  seed_pattern(mask, m, table, density);
  free(density);
}
