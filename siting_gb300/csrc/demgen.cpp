// Seeded synthetic terrain: fractal (fBm) value noise, optionally blended with
// ridged noise, min-max scaled to [0, range] and stored as row-major uint16 —
// the raw DEM format the reference reads (2-byte unsigned shorts, 0.1 m units,
// README.md:17).  The reference ships one real DEM only; these DEMs stand in
// for the larger workloads.
//
// The generator uses integer hashing and IEEE double add/multiply only (no
// libm transcendental calls) and is compiled with -ffp-contract=off, so the
// same seed gives the same bytes on x86-64 and aarch64 hosts.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "siting.h"

namespace {

inline uint64_t mix64(uint64_t z) {
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

// Lattice value in [0, 1) for integer lattice point (ix, iy) of one octave.
inline double lattice(uint64_t salt, int64_t ix, int64_t iy) {
  uint64_t h = mix64(salt ^ mix64((uint64_t)ix * 0xd6e8feb86659fd93ull ^
                                  (uint64_t)iy));
  return (double)(h >> 11) * (1.0 / 9007199254740992.0);
}

inline double fade(double t) { return t * t * (3.0 - 2.0 * t); }

// Bilinearly interpolated value noise at (u, v), in [0, 1).
inline double value_noise(uint64_t salt, double u, double v) {
  const double fu = std::floor(u), fv = std::floor(v);
  const int64_t iu = (int64_t)fu, iv = (int64_t)fv;
  const double su = fade(u - fu), sv = fade(v - fv);
  const double a = lattice(salt, iu, iv), b = lattice(salt, iu + 1, iv);
  const double c = lattice(salt, iu, iv + 1), d = lattice(salt, iu + 1, iv + 1);
  const double top = a + (b - a) * su;
  const double bot = c + (d - c) * su;
  return top + (bot - top) * sv;
}

}  // namespace

extern "C" int siting_fbm_dem(uint16_t *out, int nrows, uint64_t seed,
                              int octaves, double persistence,
                              double lacunarity, double base_wavelength,
                              double ridged_weight, int range_max) {
  if (!out || nrows <= 0 || octaves < 1 || octaves > 30 ||
      base_wavelength <= 0.0 || range_max < 0 || range_max > 65535 ||
      ridged_weight < 0.0 || ridged_weight > 1.0)
    return SITING_EINVAL;
  const size_t ncell = (size_t)nrows * nrows;
  std::vector<double> h(ncell);
  std::vector<double> freq(octaves), amp(octaves);
  std::vector<uint64_t> salt(octaves), rsalt(octaves);
  double f = 1.0 / base_wavelength, a = 1.0, asum = 0.0;
  for (int k = 0; k < octaves; k++) {
    freq[k] = f;
    amp[k] = a;
    asum += a;
    salt[k] = mix64(seed * 0x2545f4914f6cdd1dull + 2 * (uint64_t)k + 1);
    rsalt[k] = mix64(seed * 0x2545f4914f6cdd1dull + 2 * (uint64_t)k + 2);
    f *= lacunarity;
    a *= persistence;
  }
  const double inv = 1.0 / asum;
  const double w = ridged_weight;
#pragma omp parallel for schedule(static)
  for (int x = 0; x < nrows; x++) {
    for (int y = 0; y < nrows; y++) {
      double s = 0.0, r = 0.0;
      for (int k = 0; k < octaves; k++) {
        const double u = x * freq[k], v = y * freq[k];
        s += amp[k] * value_noise(salt[k], u, v);
        if (w > 0.0) {
          const double n = 2.0 * value_noise(rsalt[k], u, v) - 1.0;
          r += amp[k] * (1.0 - (n < 0.0 ? -n : n));
        }
      }
      double val = s * inv;
      if (w > 0.0) val = (1.0 - w) * val + w * (r * inv);
      h[(size_t)x * nrows + y] = val;
    }
  }
  double lo = h[0], hi = h[0];
  for (size_t i = 1; i < ncell; i++) {
    lo = h[i] < lo ? h[i] : lo;
    hi = h[i] > hi ? h[i] : hi;
  }
  const double scale = hi > lo ? (double)range_max / (hi - lo) : 0.0;
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < (long long)ncell; i++) {
    const double q = (h[i] - lo) * scale + 0.5;
    int v = (int)q;
    out[i] = (uint16_t)(v < 0 ? 0 : (v > range_max ? range_max : v));
  }
  return SITING_OK;
}
