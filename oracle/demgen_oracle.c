/* Synthetic DEMs for the CPU side (test and baseline infrastructure only).
 *
 * The reference ships one real DEM (dem.bin); its larger workloads are seeded
 * fractal terrains: fBm value noise (octave k has frequency f0*lacunarity^k
 * and weight persistence^k, f0 = 1/base_wavelength), optionally blended with
 * ridged noise 1-|2n-1| at `ridged_weight`, min-max scaled to [0, range_max]
 * and rounded half-up into row-major uint16 — the raw format of
 * siting.cpp:726-730.  This file restates that recipe independently of the
 * library's generator so that the CPU timing baseline never loads the
 * library; a test checks that both give the same bytes for the workloads'
 * recipes.  Only integer hashing (a splitmix64 finaliser on the lattice
 * coordinates) and IEEE double add/multiply are used, built with
 * -ffp-contract=off, so x86-64 and aarch64 hosts give the same bytes.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>

#define SPLITMIX_GAMMA 0x9e3779b97f4a7c15ull

static uint64_t splitmix(uint64_t z) {
  z += SPLITMIX_GAMMA;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

/* uniform value in [0, 1) at lattice point (i, j) of the noise keyed by `key` */
static double corner(uint64_t key, int64_t i, int64_t j) {
  const uint64_t cell = splitmix(((uint64_t)i * 0xd6e8feb86659fd93ull) ^ (uint64_t)j);
  return (double)(splitmix(key ^ cell) >> 11) / 9007199254740992.0; /* 2^53 */
}

/* smoothstep-weighted bilinear interpolation of the four corners */
static double noise2(uint64_t key, double u, double v) {
  const double u0 = floor(u), v0 = floor(v);
  const int64_t i = (int64_t)u0, j = (int64_t)v0;
  const double tu = u - u0, tv = v - v0;
  const double wu = tu * tu * (3.0 - 2.0 * tu);
  const double wv = tv * tv * (3.0 - 2.0 * tv);
  const double c00 = corner(key, i, j), c10 = corner(key, i + 1, j);
  const double c01 = corner(key, i, j + 1), c11 = corner(key, i + 1, j + 1);
  const double lo = c00 + (c10 - c00) * wu;
  const double hi = c01 + (c11 - c01) * wu;
  return lo + (hi - lo) * wv;
}

int oracle_fbm_dem(uint16_t *dem, int nrows, uint64_t seed, int octaves, double persistence,
                   double lacunarity, double base_wavelength, double ridged_weight,
                   int range_max) {
  if (!dem || nrows <= 0 || octaves < 1 || octaves > 30 || base_wavelength <= 0.0 ||
      range_max < 0 || range_max > 65535 || ridged_weight < 0.0 || ridged_weight > 1.0)
    return 1;
  double freq[30], weight[30], wsum = 0.0;
  uint64_t key[30], rkey[30];
  {
    double f = 1.0 / base_wavelength, a = 1.0;
    const uint64_t base = seed * 0x2545f4914f6cdd1dull;
    for (int k = 0; k < octaves; k++) {
      freq[k] = f;
      weight[k] = a;
      wsum += a;
      key[k] = splitmix(base + 2 * (uint64_t)k + 1);
      rkey[k] = splitmix(base + 2 * (uint64_t)k + 2);
      f *= lacunarity;
      a *= persistence;
    }
  }
  const double norm = 1.0 / wsum;
  const long long ncell = (long long)nrows * nrows;
  double *height = (double *)malloc(sizeof(double) * (size_t)ncell);
  if (!height) return 2;
  double gmin = INFINITY, gmax = -INFINITY;
#pragma omp parallel for schedule(static) reduction(min : gmin) reduction(max : gmax)
  for (int row = 0; row < nrows; row++) {
    double *out = height + (long long)row * nrows;
    for (int col = 0; col < nrows; col++) {
      double fbm = 0.0, ridge = 0.0;
      for (int k = 0; k < octaves; k++) {
        const double u = row * freq[k], v = col * freq[k];
        fbm += weight[k] * noise2(key[k], u, v);
        if (ridged_weight > 0.0) {
          const double m = 2.0 * noise2(rkey[k], u, v) - 1.0;
          ridge += weight[k] * (1.0 - fabs(m));
        }
      }
      double h = fbm * norm;
      if (ridged_weight > 0.0) h = (1.0 - ridged_weight) * h + ridged_weight * (ridge * norm);
      out[col] = h;
      if (h < gmin) gmin = h;
      if (h > gmax) gmax = h;
    }
  }
  const double scale = gmax > gmin ? (double)range_max / (gmax - gmin) : 0.0;
#pragma omp parallel for schedule(static)
  for (long long c = 0; c < ncell; c++) {
    const int q = (int)((height[c] - gmin) * scale + 0.5);
    dem[c] = (uint16_t)(q < 0 ? 0 : (q > range_max ? range_max : q));
  }
  free(height);
  return 0;
}
