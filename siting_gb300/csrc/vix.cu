// VIX: approximate visibility index of every DEM cell (siting.cpp:137-198).
//
// Each cell tests `ntests` random targets within roi; a target is visible when
// no sampled ground point on the line of sight (offsets 1,2,4,8,... along the
// major axis) rises above the sight line.  VIX = min(255, (int)(nvis/ntests *
// 255.999f)).
//
// GB300 mapping: one CTA per T x T cell tile.  The tile's halo (T+2roi rows,
// T+2roi+7 columns rounded to 8) is loaded into shared memory by TMA
// bulk-tensor copies, so every line-of-sight sample is a shared-memory gather.
// Each thread keeps one cell per pass and takes every L-th of its targets
// (L threads a cell); the target of item (cell, t) comes from the LCG state
// after 2t+1 steps from the seed, obtained by an affine jump-ahead table
// instead of a serial chain.  Per-cell hit counts accumulate in shared memory
// and become VIX bytes through a host-computed table.  When the halo does not
// fit in shared memory (large roi) the same code reads the DEM through the
// read-only L1 path instead.
//
// Bit-exactness: every FP32 operation is separately rounded (no FMA), the
// reference's drecip = (float)(1.0/d) comes from a host table, and C's
// truncating integer division and round-half-away-from-zero are kept.
#include <algorithm>

#include "common.cuh"
#include "kernels.h"

namespace siting {
namespace {

struct VixArgs {
  const uint16_t *dem;
  int pitch, n, roi, oht, tht, ntests;
  uint8_t *vix;
  int tile, tiles_per_row;
  int halo_w, box_rows, nboxes;
  const uint32_t *jump;  // ntests pairs: LCG map of 2t+1 steps
  const float *rtab;     // roi+1
  const uint8_t *vtab;   // ntests+1
  int *err;
};

// DEM accessors by linear offset: `base` is the observer cell's offset, a cell
// (dx, dy) away is at base + dx*stride + dy.
struct SmemDem {
  static constexpr bool kShared = true;
  const uint16_t *s;
  int w, x0, y0;
  __device__ __forceinline__ int base(int x, int y) const { return (x - x0) * w + (y - y0); }
  __device__ __forceinline__ int stride() const { return w; }
  __device__ __forceinline__ int at(int o) const { return s[o]; }
};

struct GlobalDem {
  static constexpr bool kShared = false;
  const uint16_t *g;
  int pitch;
  __device__ __forceinline__ int base(int x, int y) const { return x * pitch + y; }
  __device__ __forceinline__ int stride() const { return pitch; }
  __device__ __forceinline__ int at(int o) const { return __ldg(g + o); }
};

// One random target of one cell (siting.cpp:155-175 and 54-135).  kInterior:
// every cell of the tile is at least roi from the DEM edge, so no target can
// fall outside it and the bounds test is dropped.
template <bool kInterior, class Dem>
__device__ __forceinline__ int vix_target(const Dem &dem, int obase, int n, int roi, int roi2,
                                          int tht, unsigned long long span2, int ox, int oy,
                                          int oz, float foz, uint32_t r1,
                                          const unsigned long long *rtab2) {
  const uint32_t r2 = lcg_step(r1);
  // (int)((2*roi+0.99999f)*r/RANDOM_MAX): the divisor is 2^31, and scaling
  // by a power of two commutes with rounding (no overflow or underflow
  // here), so RN(span*r)/2^31 = RN((span*2^-31)*r): span arrives pre-scaled,
  // paired with itself, and both draws are scaled by one packed multiply.
  const unsigned long long dd = f2_mul(span2, f2_pack(i2f((int)r1), i2f((int)r2)));
  int dx = f2i(f2_lo(dd)) - roi;
  int dy = f2i(f2_hi(dd)) - roi;
  if (dx * dx + dy * dy > roi2) {  // fold into the circle (siting.cpp:162-166)
    dx /= 3;
    dy /= 3;
  }
  if (!kInterior &&
      ((unsigned)(ox + dx) >= (unsigned)n || (unsigned)(oy + dy) >= (unsigned)n))
    return 0;
  const int adx = abs(dx), ady = abs(dy);
  if (adx <= 1 && ady <= 1) return 1;
  const int W = dem.stride();
  const int tz = dem.at(obase + dx * W + dy) + tht;
  const bool mx = adx >= ady;
  const int d = mx ? dx : dy, m = mx ? dy : dx, ad = mx ? adx : ady;
  // Sample offsets are id = +-1, 2, 4, ... along the major axis (the sign of
  // d).  slope*id = m*drecip*id = (m*|drecip|)*|id| exactly (negation and
  // scaling by a power of two are exact in FP32), likewise id*zslope, so both
  // are carried by doubling from m*|drecip| and (tz-oz)*|drecip|, bit-identical
  // to the reference's products.  They travel as one pair P = {slope*|id|,
  // zslope*|id|}: one packed add doubles both, and one packed add with
  // C = {copysign(pred(0.5), slope), oz} gives the rounding sum of the minor
  // offset and the sight-line height oz + id*zslope.  The sample's offset
  // from the observer is id*(major stride) + round(slope*id)*(minor stride).
  unsigned long long P = f2_mul(f2_pack(i2f(m), i2f(tz - oz)), rtab2[ad]);  // |drecip|, siting.cpp:91
  const unsigned long long C = f2_pack(round_addend(f2_lo(P)), foz);  // the sign never changes
  const int smin = mx ? 1 : W;
  int q = obase + (mx ? (d > 0 ? W : -W) : (d > 0 ? 1 : -1));  // observer + id*(major stride)
  if constexpr (Dem::kShared) {
    // With the halo in shared memory every sample is tested: a blocked
    // target's lane would idle until its warp's other lanes finish anyway, and
    // no branch is left for the lanes to diverge on.  (Through L1 the extra
    // loads cost more than the branch.)
    bool vis = true;
    // the sample's shared-memory byte address, doubled about the observer's
    // (no scaling of an element offset at every sample)
    const uint32_t sb = smem_u32(dem.s);
    uint32_t qb = sb + 2u * (uint32_t)q;
    const uint32_t ob2 = sb + 2u * (uint32_t)obase;
    const int sminb = 2 * smin;
    for (int step = 1; step < ad; step <<= 1) {
      const unsigned long long Q = f2_add(P, C);
      const int off = f2i(f2_lo(Q));  // round(slope*id), half away from zero
      unsigned short ev;
      asm("ld.shared.u16 %0, [%1];" : "=h"(ev) : "r"(qb + off * sminb));
      vis &= !(i2f(ev) > f2_hi(Q));
      P = f2_add(P, P);
      qb = 2u * qb - ob2;  // id doubles
    }
    return vis;
  } else {
    for (int step = 1; step < ad; step <<= 1) {
      const unsigned long long Q = f2_add(P, C);
      const int off = f2i(f2_lo(Q));  // round(slope*id), half away from zero
      if (i2f(dem.at(q + off * smin)) > f2_hi(Q)) return 0;
      P = f2_add(P, P);
      q = 2 * q - obase;  // id doubles
    }
    return 1;
  }
}

// The tile's (cell, target) items: L = blockDim/T^2 consecutive threads share
// a cell (T = 16: 4) and take every L-th of its targets, so a thread keeps one
// cell for the whole pass (no per-item bookkeeping) and a warp's lanes run the
// same number of targets; the L partial counts are summed by shuffles.
template <bool kInterior, class Dem>
__device__ __forceinline__ void vix_tile_work(const Dem &dem, const VixArgs &a,
                                              const int4 *cinfo, const uint2 *jump,
                                              const unsigned long long *rtab2, int *cnt) {

  const int ncell = a.tile * a.tile;
  const int L = max(1, (int)blockDim.x / ncell);  // a power of two: tiles are 16, 32, 64
  const int per_pass = blockDim.x / L;
  const float span = fmul(fadd(i2f(2 * a.roi), 0.99999f), 0x1p-31f);  // scaled by 2^-31
  const unsigned long long span2 = f2_pack(span, span);
  const int roi2 = a.roi * a.roi;
  const int sub = threadIdx.x & (L - 1);
  for (int c0 = 0; c0 < ncell; c0 += per_pass) {
    const int cell = c0 + threadIdx.x / L;
    int acc = 0;
    if (cell < ncell) {
      const int4 ci = cinfo[cell];
      if (ci.w >= 0) {
        const int obase = ci.x, oz = ci.y, ox = ci.w >> 16, oy = ci.w & 0xffff;
        const float foz = i2f(oz);
        const uint32_t seed = (uint32_t)ci.z;
        for (int t = sub; t < a.ntests; t += L) {
          const uint2 j = jump[t];
          const uint32_t r1 = (j.x * seed + j.y) & 0x7fffffffu;
          acc += vix_target<kInterior>(dem, obase, a.n, a.roi, roi2, a.tht, span2, ox, oy, oz,
                                       foz, r1, rtab2);
        }
      }
    }
    for (int o = 1; o < L; o <<= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (sub == 0 && cell < ncell) cnt[cell] = acc;
  }
}

// One T x T tile of cells: `map` is the halo's tensor map (kSmem), `tile` the
// tile's index (row-major over tiles_per_row^2), `sm` the CTA's dynamic
// shared memory (vix_smem_bytes), `mbar` the halo's mbarrier (shared
// memory).  Every thread of the CTA calls it.
template <bool kSmem>
__device__ __forceinline__ void vix_tile(const CUtensorMap *map, const VixArgs &a, int tile,
                                         unsigned char *sm, uint64_t *mbar) {
  const int T = a.tile;
  const int tx0 = (tile / a.tiles_per_row) * T;
  const int ty0 = (tile % a.tiles_per_row) * T;
  const int hx0 = tx0 - a.roi;
  const int hy0 = (ty0 - a.roi) & ~7;  // TMA inner coordinate: 16-byte aligned
  size_t off = 0;
  uint16_t *halo = reinterpret_cast<uint16_t *>(sm);
  const uint32_t halo_bytes = kSmem ? (uint32_t)a.nboxes * a.box_rows * a.halo_w * 2u : 0u;
  off += halo_bytes + 16;  // (the per-tile kernel's mbarrier)
  uint2 *jump = reinterpret_cast<uint2 *>(sm + off);
  off += (size_t)a.ntests * 8;
  unsigned long long *rtab2 = reinterpret_cast<unsigned long long *>(sm + off);  // {r, r} pairs
  off += (size_t)(a.roi + 1) * 8;
  int *cnt = reinterpret_cast<int *>(sm + off);
  off += (size_t)T * T * 4;
  off = (off + 15) & ~(size_t)15;
  int4 *cinfo = reinterpret_cast<int4 *>(sm + off);  // per cell: base, oz, seed, row<<16|col
  off += (size_t)T * T * 16;
  uint8_t *vtab = sm + off;

  if (kSmem && threadIdx.x == 0) {
    mbar_init(mbar, 1);
    mbar_expect_tx(mbar, halo_bytes);
    for (int b = 0; b < a.nboxes; b++)
      tma_load_window(halo + (size_t)b * a.box_rows * a.halo_w, map, hy0, hx0 + b * a.box_rows,
                      mbar);
  }
  for (int i = threadIdx.x; i < a.ntests; i += blockDim.x)
    jump[i] = make_uint2(a.jump[2 * i], a.jump[2 * i + 1]);
  for (int i = threadIdx.x; i <= a.roi; i += blockDim.x) rtab2[i] = f2_pack(a.rtab[i], a.rtab[i]);
  for (int i = threadIdx.x; i <= a.ntests; i += blockDim.x) vtab[i] = a.vtab[i];
  __syncthreads();

  // targets lie within roi of their cell (after the fold, |dx|,|dy| <= roi)
  const bool interior = tx0 >= a.roi && ty0 >= a.roi && tx0 + T + a.roi <= a.n &&
                        ty0 + T + a.roi <= a.n;
  // per-cell constants, once per tile (rows and columns are below 2^16)
  auto fill_cells = [&](const auto &dem) {
    for (int i = threadIdx.x; i < T * T; i += blockDim.x) {
      const int x = tx0 + i / T, y = ty0 + i % T;
      int4 ci = make_int4(0, 0, 0, -1);
      if (x < a.n && y < a.n) {
        ci.x = dem.base(x, y);
        ci.y = dem.at(ci.x) + a.oht;
        ci.z = x * a.n + y;  // the LCG seed is the cell index (siting.cpp:150, r = tid)
        ci.w = (x << 16) | y;
      }
      cinfo[i] = ci;
    }
    __syncthreads();
  };
  if (kSmem) {
    if (!mbar_wait(mbar, 0)) {
      if (threadIdx.x == 0) atomicOr(a.err, kErrTmaTimeout);
      return;
    }
    const SmemDem dem{halo, a.halo_w, hx0, hy0};
    fill_cells(dem);
    if (interior)
      vix_tile_work<true>(dem, a, cinfo, jump, rtab2, cnt);
    else
      vix_tile_work<false>(dem, a, cinfo, jump, rtab2, cnt);
  } else {
    const GlobalDem dem{a.dem, a.pitch};
    fill_cells(dem);
    if (interior)
      vix_tile_work<true>(dem, a, cinfo, jump, rtab2, cnt);
    else
      vix_tile_work<false>(dem, a, cinfo, jump, rtab2, cnt);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < T * T; i += blockDim.x) {
    const int lx = i / T;
    const int x = tx0 + lx, y = ty0 + (i - lx * T);
    if (x < a.n && y < a.n) a.vix[x * a.n + y] = vtab[cnt[i]];
  }
}

template <bool kSmem>
__global__ void __launch_bounds__(1024) vix_kernel(const __grid_constant__ CUtensorMap map,
                                                  const VixArgs a) {
  extern __shared__ __align__(128) unsigned char sm[];
  const uint32_t halo_bytes = kSmem ? (uint32_t)a.nboxes * a.box_rows * a.halo_w * 2u : 0u;
  vix_tile<kSmem>(&map, a, blockIdx.x, sm, reinterpret_cast<uint64_t *>(sm + halo_bytes));
}

// ---- VIX of many jobs in one launch (batched form) ---------------------------
// One grid covers the (job, tile) items of many jobs, so a job's last tiles
// overlap the next job's first ones instead of each job ending a grid of its
// own.  The job table travels as the kernel's parameters, and a CTA finds its
// job from its index: every value derived from the table is then the same in
// all threads and is read from the constant bank, as in the one-job kernel.

struct VixQJob {
  CUtensorMap map;  // halo map of a staged job
  VixArgs a;
  unsigned first;   // grid index of the job's first tile
};

struct VixQTable {
  VixQJob jobs[kStageQueueMaxJobs];
  int njobs;
};
static_assert(sizeof(VixQTable) <= 32000, "kernel parameters are limited to 32 KB");

// One CTA per (job, tile) item.  kSmem: every job of the launch has its halo
// staged (else none has): one kernel per staging keeps each within 32
// registers a thread.
template <bool kSmem>
__global__ void __launch_bounds__(1024, 2) vixq_kernel(const __grid_constant__ VixQTable tab) {
  extern __shared__ __align__(128) unsigned char sm[];
  __shared__ __align__(8) uint64_t mbar;
  const unsigned it = blockIdx.x;
  int lo = 0, hi = tab.njobs - 1;  // the last job whose first tile is at or before `it`
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (tab.jobs[mid].first <= it)
      lo = mid;
    else
      hi = mid - 1;
  }
  const VixQJob &J = tab.jobs[lo];
  vix_tile<kSmem>(&J.map, J.a, (int)(it - J.first), sm, &mbar);
}

int round8(int v) { return (v + 7) & ~7; }

struct HaloGeom {
  int w, box_rows, nboxes;
};

HaloGeom halo_geom(int tile, int roi) {
  HaloGeom g;
  g.w = round8(tile + 2 * roi + 7);
  const int h = tile + 2 * roi;
  g.nboxes = (h + 255) / 256;
  g.box_rows = round8((h + g.nboxes - 1) / g.nboxes);
  return g;
}

size_t tables_tail_bytes(int tile, int roi, int ntests) {
  // mbarrier, jump table, reciprocal pairs, counts, then the int4 cell table
  // (16-byte aligned: the offsets before it are multiples of 4), VIX bytes
  size_t b = 16 + (size_t)ntests * 8 + (size_t)(roi + 1) * 8 + (size_t)tile * tile * 4;
  b = (b + 15) & ~(size_t)15;
  return b + (size_t)tile * tile * 16 + ntests + 1;
}

}  // namespace

size_t vix_table_bytes(int roi, int ntests) {
  return (((size_t)ntests * 8 + (size_t)(roi + 1) * 4 + ntests + 1) + 15) & ~(size_t)15;
}

void vix_fill_tables(void *host_buf, int roi, int ntests) {
  uint32_t *jump = static_cast<uint32_t *>(host_buf);
  const uint32_t a = 1103515245u, c = 12345u;
  uint32_t A = a, C = c;  // map of 1 step
  for (int t = 0; t < ntests; t++) {
    jump[2 * t] = A;  // map of 2t+1 steps
    jump[2 * t + 1] = C;
    A = a * (a * A);  // advance by two steps
    C = a * (a * C + c) + c;
  }
  float *rtab = reinterpret_cast<float *>(jump + 2 * ntests);
  rtab[0] = 0.f;
  for (int d = 1; d <= roi; d++) rtab[d] = (float)(1.0 / d);  // siting.cpp:91
  uint8_t *vtab = reinterpret_cast<uint8_t *>(rtab + roi + 1);
  for (int v = 0; v <= ntests; v++) {
    const float f = (float)v / ntests;  // siting.cpp:186-189
    const int q = (int)(f * 255.999f);
    vtab[v] = (uint8_t)(q < 255 ? q : 255);
  }
}

size_t vix_smem_bytes(const VixPlan &p, int roi, int ntests) {
  size_t b = tables_tail_bytes(p.tile, roi, ntests);
  if (p.use_smem) {
    const HaloGeom g = halo_geom(p.tile, roi);
    b += (size_t)g.nboxes * g.box_rows * g.w * 2;
  }
  return b;
}

// Two 1024-thread CTAs share an SM when each takes at most half of its 228 KB
// shared memory (at most 32 registers a thread); the second CTA fills the
// issue slots that the first leaves while its warps drain at the end of a tile.
constexpr size_t kVixTwoCtaSmem = 112 * 1024;
constexpr size_t kVixMaxSmem = 220 * 1024;

VixPlan vix_default_plan(int nrows, int roi, int ntests) {
  (void)nrows;
  // 32x32 tiles (one cell a thread) are fastest wherever their halo fits two
  // CTAs per SM, then 16x16 (four threads a cell); else the L1 path, where
  // the halo costs nothing.  64x64 tiles (four cells a thread) never won.
  for (int tile : {32, 16}) {
    VixPlan q{tile, 1024, true};
    if (vix_smem_bytes(q, roi, ntests) <= kVixTwoCtaSmem) return q;
  }
  VixPlan p{32, 1024, false};
  if (vix_smem_bytes(p, roi, ntests) > kVixMaxSmem) p.tile = 16;
  return p;
}

VixPlan vix_plan_for(int nrows, int roi, int ntests, int tile, int smem) {
  VixPlan p = vix_default_plan(nrows, roi, ntests);
  if (tile == 16 || tile == 32 || tile == 64) {
    p.tile = tile;
    p.use_smem = smem != 0;
    const HaloGeom g = halo_geom(tile, roi);
    if (p.use_smem && (g.w > 2048 || vix_smem_bytes(p, roi, ntests) > kVixMaxSmem)) p.use_smem = false;
    if (!p.use_smem && vix_smem_bytes(p, roi, ntests) > kVixMaxSmem) p = vix_default_plan(nrows, roi, ntests);
  } else if (smem == 0) {
    p.use_smem = false;
  }
  return p;
}

namespace {

// Kernel arguments and halo map of one job; false if the map cannot be made.
bool vix_args(const DemView &dem, int roi, int oht, int tht, int ntests, uint8_t *vix,
              const void *d_tables, const VixPlan &plan, int *d_err, VixArgs *out,
              CUtensorMap *map, bool *smem) {
  VixArgs a{};
  a.dem = dem.data;
  a.pitch = dem.pitch;
  a.n = dem.nrows;
  a.roi = roi;
  a.oht = oht;
  a.tht = tht;
  a.ntests = ntests;
  a.vix = vix;
  a.tile = plan.tile;
  a.tiles_per_row = ceil_div(dem.nrows, plan.tile);
  a.jump = static_cast<const uint32_t *>(d_tables);
  a.rtab = reinterpret_cast<const float *>(a.jump + 2 * ntests);
  a.vtab = reinterpret_cast<const uint8_t *>(a.rtab + roi + 1);
  a.err = d_err;
  memset(map, 0, sizeof(*map));
  *smem = plan.use_smem && dem.tma_ok;
  if (*smem) {
    const HaloGeom g = halo_geom(plan.tile, roi);
    a.halo_w = g.w;
    a.box_rows = g.box_rows;
    a.nboxes = g.nboxes;
    if (!make_dem_tensor_map(map, dem, g.w, g.box_rows)) return false;
  }
  *out = a;
  return true;
}

}  // namespace

cudaError_t launch_vix(const DemView &dem, int roi, int oht, int tht, int ntests, uint8_t *vix,
                       const void *d_tables, const VixPlan &plan, int *d_err, cudaStream_t st) {
  VixArgs a;
  CUtensorMap map;
  bool smem;
  if (!vix_args(dem, roi, oht, tht, ntests, vix, d_tables, plan, d_err, &a, &map, &smem))
    return cudaErrorInvalidValue;
  VixPlan eff = plan;
  eff.use_smem = smem;
  const size_t shm = vix_smem_bytes(eff, roi, ntests);
  const int grid = a.tiles_per_row * a.tiles_per_row;
  cudaError_t e;
  if (smem) {
    e = cudaFuncSetAttribute(vix_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)shm);
    if (e != cudaSuccess) return e;
    vix_kernel<true><<<grid, plan.threads, shm, st>>>(map, a);
  } else {
    e = cudaFuncSetAttribute(vix_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)shm);
    if (e != cudaSuccess) return e;
    vix_kernel<false><<<grid, plan.threads, shm, st>>>(map, a);
  }
  return cudaGetLastError();
}

cudaError_t launch_vix_queue(const StageJob *jobs, int njobs, cudaStream_t st) {
  // jobs whose halo is staged, then those read through L1: one launch for
  // each kind, at most kStageQueueMaxJobs jobs a launch
  static thread_local VixQTable tab;  // 20 KB: not on the host stack
  for (int kind = 0; kind < 2; kind++) {
    int j = 0;
    while (j < njobs) {
      tab.njobs = 0;
      size_t shm = 0;
      unsigned total = 0;
      for (; j < njobs && tab.njobs < kStageQueueMaxJobs; j++) {
        const StageJob &J = jobs[j];
        VixQJob &q = tab.jobs[tab.njobs];
        memset(&q, 0, sizeof(q));
        bool smem;
        if (!vix_args(J.dem, J.roi, J.oht, J.tht, J.ntests, J.vix, J.vix_tables, J.vplan, J.err,
                      &q.a, &q.map, &smem))
          return cudaErrorInvalidValue;
        if ((smem ? 0 : 1) != kind) continue;
        q.first = total;
        VixPlan eff = J.vplan;
        eff.use_smem = smem;
        shm = std::max(shm, vix_smem_bytes(eff, J.roi, J.ntests));
        total += (unsigned)(q.a.tiles_per_row * q.a.tiles_per_row);
        tab.njobs++;
      }
      if (!tab.njobs) continue;
      auto kern = kind == 0 ? vixq_kernel<true> : vixq_kernel<false>;
      cudaError_t e =
          cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm);
      if (e != cudaSuccess) return e;
      kern<<<total, 1024, shm, st>>>(tab);
      e = cudaGetLastError();
      if (e != cudaSuccess) return e;
    }
  }
  return cudaSuccess;
}

}  // namespace siting
