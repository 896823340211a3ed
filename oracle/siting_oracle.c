/*
 * CPU restatement of the reference observer-siting pipeline
 * VIX -> FINDMAX -> VIEWSHED -> SITE, with seqsite semantics.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity oracle and the timed CPU
 * baseline.  Only the tests, the smoke check and the bench's CPU-baseline leg
 * load it; the product library never links or calls it.
 *
 * Every function restates the reference's algorithm (wenlili/siting,
 * siting.cpp) in the same floating-point evaluation order, so its outputs are
 * bit-identical to the reference's `seqsite` (pinned by tests that compare it
 * with the reference built from its own sources, and with the known answers of
 * the reference's sample DEM).  Build with -ffp-contract=off: the reference is
 * compiled without FMA contraction on x86-64, and aarch64 compilers contract
 * by default.
 *
 * Parallelism: OpenMP over independent cells / blocks / observers / update
 * candidates.  Every parallel loop writes disjoint outputs, and SITE's argmax
 * is the sequential lowest-index scan of siting.cpp:553-562, so results do not
 * depend on the thread count.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_RANDOM_MAX 0x7fffffff /* siting.cpp:27 */

static inline int isq(int v) { return v * v; }
static inline int iabs_(int v) { return v < 0 ? -v : v; }

/* glibc-constant LCG step on 31 bits: siting.cpp:29-33. */
static inline int lcg_step(int seed) {
  return (int)((1103515245u * ((unsigned)seed & 0x7fffffffu) + 12345u) &
               0x7fffffffu);
}

int oracle_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void oracle_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

/*
 * Block geometry: siting.cpp:688-695.  Returns 1 when the last block is too
 * small for the per-block observer count (the reference dies there).
 */
int oracle_geometry(int nrows, int bw, int nwanted0, float *bs_out,
                    int *nb_out, int *npb_out, int *nwanted_out) {
  float bs = (float)nrows / (int)((float)nrows / bw + 0.5f);
  int nb = (int)(nrows / bs + 0.5f);
  int npb = (int)((float)nwanted0 / isq(nb) + 0.99999f);
  int last = nrows - (int)(bs * (nb - 1));
  *bs_out = bs;
  *nb_out = nb;
  *npb_out = npb;
  *nwanted_out = npb * isq(nb);
  return isq(last) < npb ? 1 : 0;
}

/*
 * Line-of-sight test between observer (ox,oy,oz) and target (tx,ty,tz):
 * siting.cpp:54-135.  The four octant cases of the reference are one walk
 * along the major axis here: sample offsets 1,2,4,8,... (times the sign of the
 * major delta) strictly inside the segment, minor coordinate
 * o + round(slope*id), slope and zslope scaled by (float)(1.0/d), and the
 * target is hidden when a sample's ground is above oz + id*zslope.
 */
static int los_visible(int nrows, const uint16_t *elev, int ox, int oy, int oz,
                       int tx, int ty, int tz) {
  if (iabs_(ox - tx) <= 1 && iabs_(oy - ty) <= 1) return 1;
  const int major_is_x = iabs_(tx - ox) >= iabs_(ty - oy);
  const int d = major_is_x ? tx - ox : ty - oy;
  const int m = major_is_x ? ty - oy : tx - ox;
  const float drecip = (float)(1.0 / d);
  const float slope = m * drecip;
  const float zslope = (tz - oz) * drecip;
  const int dir = d > 0 ? 1 : -1;
  for (int step = 1; step < d * dir; step <<= 1) {
    const int id = step * dir;
    const int off = (int)roundf(slope * id);
    const int x = major_is_x ? ox + id : ox + off;
    const int y = major_is_x ? oy + off : oy + id;
    const float z = elev[x * nrows + y];
    if (z > oz + id * zslope) return 0;
  }
  return 1;
}

/* One cell's visibility index: siting.cpp:137-190. */
static uint8_t vix_one(int cell, int nrows, const uint16_t *elev, int roi,
                       int oht, int tht, int ntests) {
  const int ox = cell / nrows, oy = cell % nrows;
  const int oz = elev[cell] + oht;
  const float span = 2 * roi + 0.99999f;
  int r = cell, nvis = 0;
  for (int t = 0; t < ntests; t++) {
    r = lcg_step(r);
    int tx = (int)(span * r / ORC_RANDOM_MAX) + (ox - roi);
    r = lcg_step(r);
    int ty = (int)(span * r / ORC_RANDOM_MAX) + (oy - roi);
    if (isq(tx - ox) + isq(ty - oy) > isq(roi)) { /* fold inside: cpp:162-166 */
      tx = ox + (tx - ox) / 3;
      ty = oy + (ty - oy) / 3;
    }
    if (tx >= 0 && tx < nrows && ty >= 0 && ty < nrows)
      nvis += los_visible(nrows, elev, ox, oy, oz, tx, ty,
                          elev[tx * nrows + ty] + tht);
  }
  const float v = (float)nvis / ntests;
  const int q = (int)(v * 255.999f);
  return (uint8_t)(q < 255 ? q : 255);
}

/* calc_vix: siting.cpp:192-198. */
void oracle_calc_vix(int nrows, const uint16_t *elev, int roi, int oht,
                     int tht, int ntests, uint8_t *vix) {
  const long long ncell = (long long)nrows * nrows;
#pragma omp parallel for schedule(dynamic, 256)
  for (long long c = 0; c < ncell; c++)
    vix[c] = vix_one((int)c, nrows, elev, roi, oht, tht, ntests);
}

/* calc_vix restricted to a list of cells (the same per-cell computation,
 * siting.cpp:137-190): spot checks of full-size rasters. */
void oracle_vix_cells(int nrows, const uint16_t *elev, int roi, int oht,
                      int tht, int ntests, const int64_t *cells, int count,
                      uint8_t *out) {
#pragma omp parallel for schedule(dynamic, 64)
  for (int i = 0; i < count; i++)
    out[i] = vix_one((int)cells[i], nrows, elev, roi, oht, tht, ntests);
}

/* Number of VIX targets that land in the DEM and of LOS samples they read
 * (work accounting for the VIX roofline; same walk as los_visible). */
void oracle_vix_work(int nrows, const uint16_t *elev, int roi, int oht,
                     int tht, int ntests, long long *targets_in,
                     long long *samples) {
  long long tin = 0, smp = 0;
  const long long ncell = (long long)nrows * nrows;
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : tin, smp)
  for (long long c = 0; c < ncell; c++) {
    const int ox = (int)(c / nrows), oy = (int)(c % nrows);
    const int oz = elev[c] + oht;
    const float span = 2 * roi + 0.99999f;
    int r = (int)c;
    for (int t = 0; t < ntests; t++) {
      r = lcg_step(r);
      int tx = (int)(span * r / ORC_RANDOM_MAX) + (ox - roi);
      r = lcg_step(r);
      int ty = (int)(span * r / ORC_RANDOM_MAX) + (oy - roi);
      if (isq(tx - ox) + isq(ty - oy) > isq(roi)) {
        tx = ox + (tx - ox) / 3;
        ty = oy + (ty - oy) / 3;
      }
      if (!(tx >= 0 && tx < nrows && ty >= 0 && ty < nrows)) continue;
      tin++;
      if (iabs_(ox - tx) <= 1 && iabs_(oy - ty) <= 1) continue;
      const int tz = elev[tx * nrows + ty] + tht;
      const int major_is_x = iabs_(tx - ox) >= iabs_(ty - oy);
      const int d = major_is_x ? tx - ox : ty - oy;
      const int m = major_is_x ? ty - oy : tx - ox;
      const float drecip = (float)(1.0 / d);
      const float slope = m * drecip, zslope = (tz - oz) * drecip;
      const int dir = d > 0 ? 1 : -1;
      for (int step = 1; step < d * dir; step <<= 1) {
        const int id = step * dir;
        const int off = (int)roundf(slope * id);
        const int x = major_is_x ? ox + id : ox + off;
        const int y = major_is_x ? oy + off : oy + id;
        smp++;
        if ((float)elev[x * nrows + y] > oz + id * zslope) break;
      }
    }
  }
  *targets_in = tin;
  *samples = smp;
}

/*
 * FINDMAX for one block: siting.cpp:204-233.  Each round scans the block in
 * row-major order for the largest (vix, h) with h = x*(x+y)*010101010101
 * wrapping in 32 bits; the first cell reaching the maximum wins.  The winner's
 * vix is then cleared (so a zero-vix winner can repeat).
 */
static void findmax_block(int bx, int by, int nrows, uint8_t *vix, float bs,
                          int npb, int32_t *obs) {
  const int x0 = (int)(bs * bx), y0 = (int)(bs * by);
  int x1 = (int)(bs * (bx + 1)), y1 = (int)(bs * (by + 1));
  if (x1 > nrows) x1 = nrows;
  if (y1 > nrows) y1 = nrows;
  for (int k = 0; k < npb; k++) {
    int bestx = x0, besty = y0;
    int bestv = vix[x0 * nrows + y0];
    int32_t besth = (int32_t)((uint32_t)x0 * (uint32_t)(x0 + y0) * 0x41041041u);
    for (int x = x0; x < x1; x++)
      for (int y = y0; y < y1; y++) {
        const int v = vix[x * nrows + y];
        const int32_t h =
            (int32_t)((uint32_t)x * (uint32_t)(x + y) * 0x41041041u);
        if (bestv < v || (bestv == v && besth < h)) {
          bestx = x;
          besty = y;
          bestv = v;
          besth = h;
        }
      }
    obs[k] = bestx * nrows + besty;
    vix[bestx * nrows + besty] = 0;
  }
}

/* find_max: siting.cpp:235-241; observers are block-major, obs[b*npb+k]. */
void oracle_find_max(int nrows, uint8_t *vix, float bs, int nb, int npb,
                     int32_t *obs) {
#pragma omp parallel for schedule(dynamic, 16)
  for (int b = 0; b < nb * nb; b++)
    findmax_block(b / nb, b % nb, nrows, vix, bs, npb, &obs[(size_t)b * npb]);
}

/* Bit (row, col) of a viewshed: word row*nwpr+col/64, MSB first
 * (siting.cpp:247-250). */
static inline void shed_set(uint64_t *shed, int nwpr, int row, int col) {
  shed[(size_t)row * nwpr + col / 64] |= 1ull << (63 - col % 64);
}

/*
 * Viewshed of one observer: siting.cpp:252-347.  Rays go from the observer to
 * each of the 8*roi perimeter cells of the (2roi+1)^2 box, stepping the major
 * axis; each ray keeps the running maximum horizon slope, stops at the DEM
 * edge or outside the roi circle, and marks a cell when its ground plus the
 * target height is at or above the horizon altitude.
 */
static void shed_one(int ob, int nrows, const uint16_t *elev, int roi,
                     int oht, int tht, uint64_t *shed) {
  const int ox = ob / nrows, oy = ob % nrows;
  const int nwpr = (2 * roi + 1 + 63) / 64;
  const int side = 2 * roi;
  const int xmin = ox - roi, ymin = oy - roi, xmax = ox + roi, ymax = oy + roi;
  const int oalt = elev[ob] + oht;
  shed_set(shed, nwpr, roi, roi);
  for (int ip = 0; ip < 4 * side; ip++) {
    int tx, ty; /* perimeter order of siting.cpp:291-304 */
    if (ip < side) {
      tx = xmin + ip;
      ty = ymin;
    } else if (ip < 2 * side) {
      tx = 1 + xmin - side + ip;
      ty = ymax;
    } else if (ip < 3 * side) {
      tx = xmin;
      ty = 1 + ymin - 2 * side + ip;
    } else {
      tx = xmax;
      ty = ymin - 3 * side + ip;
    }
    if (tx == ox && ty == oy) continue;
    const int dx = tx - ox, dy = ty - oy;
    const int major_is_y = iabs_(dx) < iabs_(dy);
    const int dmaj = major_is_y ? dy : dx, dmin = major_is_y ? dx : dy;
    const float slope = (float)dmin / (float)dmaj;
    const int dir = dmaj > 0 ? 1 : -1;
    float hslope = -99999.f;
    for (int i = dir; i != dmaj + dir; i += dir) {
      const int off = (int)roundf(i * slope);
      const int px = major_is_y ? ox + off : ox + i;
      const int py = major_is_y ? oy + i : oy + off;
      if (px < 0 || px >= nrows || py < 0 || py >= nrows) break;
      if (isq(px - ox) + isq(py - oy) > isq(roi)) break;
      const int pelev = elev[px * nrows + py];
      const int ai = iabs_(i);
      const float s = (float)(pelev - oalt) / (float)ai;
      if (hslope < s) hslope = s;
      const float halt = oalt + hslope * ai;
      if (pelev + tht >= halt)
        shed_set(shed, nwpr, px - ox + roi, py - oy + roi);
    }
  }
}

/* calc_sheds: siting.cpp:349-360. */
void oracle_calc_sheds(int nrows, const uint16_t *elev, int roi, int oht,
                       int tht, int nsheds, const int32_t *obs,
                       uint64_t *sheds) {
  const size_t per = (size_t)(2 * roi + 1) * ((2 * roi + 1 + 63) / 64);
  memset(sheds, 0, per * nsheds * sizeof(uint64_t));
#pragma omp parallel for schedule(dynamic, 4)
  for (int t = 0; t < nsheds; t++)
    shed_one(obs[t], nrows, elev, roi, oht, tht, &sheds[per * t]);
}

/* Word alignment of a shed placed with its column 0 at global column c0:
 * floor division by 64 (siting.cpp:400-405). */
static inline void shed_align(int c0, int *firstword, int *firstbit) {
  int w = c0 / 64, b = c0 % 64;
  if (b < 0) {
    w--;
    b += 64;
  }
  *firstword = w;
  *firstbit = b;
}

/* OR a shed into the cumulative coverage bitmap: siting.cpp:393-419. */
static void cover_union(int nrows, int roi, int ox, int oy,
                        const uint64_t *shed, uint64_t *cum) {
  const int nr = 2 * roi + 1, nwpr = (nr + 63) / 64, cw = (nrows + 63) / 64;
  int fw, fb;
  shed_align(oy - roi, &fw, &fb);
  for (int row = 0; row < nr; row++) {
    const int crow = ox - roi + row;
    if (crow < 0 || crow >= nrows) continue;
    uint64_t *dst = &cum[(size_t)crow * cw];
    for (int w = 0; w < nwpr; w++) {
      const uint64_t v = shed[(size_t)row * nwpr + w];
      const int cword = fw + w;
      if (cword >= 0 && cword < cw) dst[cword] |= v >> fb;
      if (fb != 0 && cword + 1 >= 0 && cword + 1 < cw)
        dst[cword + 1] |= v << (64 - fb);
    }
  }
}

/* Bit of cell (x,y) in the coverage bitmap: siting.cpp:421-428. */
static inline int covered(int cw, const uint64_t *cum, int x, int y) {
  const int i = x * cw * 64 + y;
  return (cum[i / 64] >> (63 - i % 64)) & 1;
}

/* Cells a shed would add to the coverage: siting.cpp:430-499 (without the
 * intervis gate, which the caller applies). */
static int cover_gain(int nrows, int roi, int ox, int oy, const uint64_t *shed,
                      const uint64_t *cum) {
  const int nr = 2 * roi + 1, nwpr = (nr + 63) / 64, cw = (nrows + 63) / 64;
  int fw, fb;
  shed_align(oy - roi, &fw, &fb);
  const int lw = (oy + roi) / 64;
  int total = 0;
  for (int row = 0; row < nr; row++) {
    const int crow = ox - roi + row;
    if (crow < 0 || crow >= nrows) continue;
    const uint64_t *srow = &shed[(size_t)row * nwpr];
    const uint64_t *crw = &cum[(size_t)crow * cw];
    for (int cword = fw < 0 ? 0 : fw; cword <= lw && cword < cw; cword++) {
      const int w = cword - fw;
      const uint64_t cur = w < nwpr ? srow[w] : 0ull;
      const uint64_t prev = w > 0 ? srow[w - 1] : 0ull;
      uint64_t placed = cur >> fb;
      if (fb != 0) placed |= prev << (64 - fb);
      total += __builtin_popcountll(placed & ~crw[cword]);
    }
  }
  return total;
}

/*
 * Greedy selection: siting.cpp:501-626 with the sequential argmax.  Each
 * round rescores the unused candidates (all of them in the first round, else
 * those within 2*roi of the last pick), zeroes a rescored candidate's gain when
 * intervis is on and its cell is not yet covered, picks the lowest index with
 * the largest positive gain, ORs its shed into the coverage and stops at zero
 * gain or once coverage exceeds 95%.
 *
 * selected[i] = 1 for picked candidates.  Returns the number picked; the
 * covered cell count goes to *cumarea_out and, when pick_order is not NULL,
 * the picks in order to pick_order[0..n).
 */
int oracle_site_it(int nrows, int roi, int intervis, int nsheds,
                   const int32_t *obs, const uint64_t *sheds,
                   uint8_t *selected, long long *cumarea_out,
                   int32_t *pick_order) {
  const int nr = 2 * roi + 1, nwpr = (nr + 63) / 64, cw = (nrows + 63) / 64;
  const size_t per = (size_t)nr * nwpr;
  uint64_t *cum = (uint64_t *)calloc((size_t)nrows * cw, sizeof(uint64_t));
  int *gain = (int *)calloc(nsheds, sizeof(int));
  int *todo = (int *)malloc(sizeof(int) * (nsheds > 0 ? nsheds : 1));
  memset(selected, 0, nsheds);
  int nused = 0, lastx = 0, lasty = 0;
  long long cumarea = 0;
  const double ncells = (double)nrows * nrows;
  for (;;) {
    int ntodo = 0;
    for (int c = 0; c < nsheds; c++) {
      if (selected[c]) continue;
      const int cx = obs[c] / nrows, cy = obs[c] % nrows;
      if (nused == 0 || isq(cx - lastx) + isq(cy - lasty) <= isq(2 * roi))
        todo[ntodo++] = c;
    }
#pragma omp parallel for schedule(dynamic, 8)
    for (int k = 0; k < ntodo; k++) {
      const int c = todo[k];
      const int cx = obs[c] / nrows, cy = obs[c] % nrows;
      if (intervis && nused > 0 && !covered(cw, cum, cx, cy))
        gain[c] = 0;
      else
        gain[c] = cover_gain(nrows, roi, cx, cy, &sheds[per * c], cum);
    }
    int best = -1, bestgain = 0;
    for (int c = 0; c < nsheds; c++)
      if (!selected[c] && gain[c] > bestgain) {
        bestgain = gain[c];
        best = c;
      }
    if (bestgain == 0) break;
    const int bx = obs[best] / nrows, by = obs[best] % nrows;
    cover_union(nrows, roi, bx, by, &sheds[per * best], cum);
    if (pick_order) pick_order[nused] = best;
    nused++;
    selected[best] = 1;
    lastx = bx;
    lasty = by;
    cumarea += bestgain;
    if (100.0 * cumarea / ncells > 95) break;
  }
  free(cum);
  free(gain);
  free(todo);
  *cumarea_out = cumarea;
  return nused;
}

/* Coverage bitmap of a set of selected sheds (used to cross-check cumarea). */
long long oracle_union_count(int nrows, int roi, int nsheds, const int32_t *obs,
                             const uint64_t *sheds, const uint8_t *selected) {
  const int nr = 2 * roi + 1, nwpr = (nr + 63) / 64, cw = (nrows + 63) / 64;
  const size_t per = (size_t)nr * nwpr;
  uint64_t *cum = (uint64_t *)calloc((size_t)nrows * cw, sizeof(uint64_t));
  for (int c = 0; c < nsheds; c++)
    if (selected[c])
      cover_union(nrows, roi, obs[c] / nrows, obs[c] % nrows, &sheds[per * c],
                  cum);
  long long n = 0;
  for (size_t i = 0; i < (size_t)nrows * cw; i++)
    n += __builtin_popcountll(cum[i]);
  free(cum);
  return n;
}
