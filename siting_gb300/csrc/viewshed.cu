// VIEWSHED: bit-packed viewshed of every tentative observer
// (siting.cpp:247-360).
//
// From observer o, rays go to each of the 8*roi perimeter cells of the
// (2roi+1)^2 box (perimeter order of siting.cpp:291-304).  A ray steps the
// major axis, puts the minor coordinate at o + round(i*slope), stops at the
// DEM edge or outside the roi circle, keeps the running maximum horizon slope
// s = (elev - oalt)/|i| and marks the cell when elev + tht >= oalt + hs*|i|.
// Bit (row, col) of a shed is word row*nwpr + col/64, bit 63 - col%64.
//
// GB300 mapping: one CTA per observer.  The observer's window (2roi+1 rows,
// 2roi+8 columns from an 8-aligned start) is loaded into shared memory by one
// TMA bulk-tensor copy; each thread sweeps rays (adjacent threads take
// adjacent perimeter cells, so a warp's lanes touch neighbouring cells each
// step and have nearly equal ray lengths).  Visible cells are OR-ed into a
// shared-memory image of the shed (32-bit halves of the reference's 64-bit
// words), which is then written to HBM with coalesced stores.  For windows
// too large for two CTAs per SM the DEM is read through the read-only L1 path.
//
// Half windows: every ray to a target row tx <= ox stays in rows ox-roi..ox,
// every other ray in rows ox..ox+roi, so an observer can also be swept by two
// CTAs that each stage roi+1 rows (half the bytes: twice the resident CTAs,
// and windows up to roi ~150 staged).  The upper CTA writes shed rows 0..roi,
// the lower one rows roi+1..2roi.  Row ox is the upper CTA's: the lower CTA's
// rays meet it only in a prefix of steps k with round(k*slope) = 0, and such a
// prefix samples the cells (ox, oy+-k) in the order and at the steps of the
// straight ray to (ox, oy+-roi) of the upper CTA, with the same horizons, so
// its marks there are a subset of that ray's.
//
// Bit-exactness: separately rounded FP32 operations, IEEE division for the
// slopes, round-half-away-from-zero for the minor coordinate.  The horizon
// slope s = RN(a/k) (a an integer elevation difference, k the step) is
// q0 = RN(a*y), s = RN(q0 + RN(a - k*q0)*y) with y = RN(1/k) from a per-CTA
// table: one fused correction of a quotient within an ulp, given a correctly
// rounded reciprocal, yields the correctly rounded quotient (Markstein's
// theorem), and an exhaustive check of every |a| <= 2^21, k <= 2048 (the
// validated heights and rois) against IEEE division agrees bit for bit.
// Beyond that range the kernel divides.
#include <algorithm>

#include "common.cuh"
#include "kernels.h"

namespace siting {
namespace {

// Word strides of the two shed images (odd, so consecutive rows/columns fall in
// distinct banks); the column image has 32-column padding for the transpose.
__host__ __device__ __forceinline__ int shed_row_stride(int nr) {
  const int w = 2 * ((nr + 63) / 64);  // reference words per row, in halves
  return w | 1;
}
__host__ __device__ __forceinline__ int shed_col_stride(int nr) { return ((nr + 31) / 32) | 1; }
__host__ __device__ __forceinline__ int shed_col_count(int nr) { return (nr + 31) / 32 * 32; }

struct ShedArgs {
  const uint16_t *dem;
  int pitch, n, roi, oht, tht, nsheds;
  const int32_t *obs;
  uint64_t *sheds;
  int win_w, box_rows, nboxes;
  int *err;
};

// DEM accessors by linear offset: `base` is the observer cell's offset, a cell
// (dx, dy) away is at base + dx*stride + dy.
struct SmemDem {
  static constexpr bool kShared = true;
  uint32_t s;  // shared-memory address of the window
  int w, x0, y0;
  __device__ __forceinline__ int base(int x, int y) const { return (x - x0) * w + (y - y0); }
  __device__ __forceinline__ int stride() const { return w; }
  __device__ __forceinline__ int at(int o) const {
    unsigned short v;
    asm("ld.shared.u16 %0, [%1];" : "=h"(v) : "r"(s + 2u * (uint32_t)o));
    return v;
  }
};

struct GlobalDem {
  static constexpr bool kShared = false;
  const uint16_t *g;
  int pitch;
  __device__ __forceinline__ int base(int x, int y) const { return x * pitch + y; }
  __device__ __forceinline__ int stride() const { return pitch; }
  __device__ __forceinline__ int at(int o) const { return __ldg(g + o); }
};

// The shed is assembled in two shared-memory bit images.  Rays that step
// along y put a warp's lanes on different rows at each step; they mark cells in
// the row-major image R (word = row*rs + col/32, bit 31 - col%32, i.e. the
// reference's words split into 32-bit halves, bit col%32 LSB-first; the
// halves are bit-reversed into the reference's MSB-first order on the way
// out).  Rays that step along x put the lanes on one row; they mark the
// column-major image C (word = col*cs + row/32, bit row%32), where their words
// differ.  rs and cs are odd, so distinct words also fall in distinct banks.
// C is transposed into R at the end, 32x32 bits per warp.
struct ShedImage {
  unsigned *R, *C;
  int rs, cs;
};

__device__ __forceinline__ void mark_row_major(const ShedImage &im, int row, int col) {
  atomicOr(&im.R[row * im.rs + (col >> 5)], 1u << (col & 31));
}

// Perimeter index of ray t of a half window, in perimeter order: the upper
// half (0) takes the 4roi+1 targets with tx <= ox, the lower half (1) the
// other 4roi-1.
__device__ __forceinline__ int half_ray(int t, int roi, int half) {
  if (!half) return t + (t <= roi ? 0 : t <= 2 * roi ? roi - 1 : 2 * roi - 1);
  return t + (t < roi - 1 ? roi + 1 : t < 2 * roi - 1 ? 2 * roi + 1 : 4 * roi + 1);
}

// Rays of this CTA; the images hold shed rows r0.. (r0 = roi for a lower half).
template <bool kRcp, bool kHalf, class Dem>
__device__ __forceinline__ void sweep_rays(const Dem &dem, const ShedArgs &a, int ox, int oy,
                                           const ShedImage &im, uint32_t rcp, int half) {
  const int roi = a.roi, n = a.n, side = 2 * roi;
  const int roi2 = roi * roi;
  const int xmin = ox - roi, ymin = oy - roi, xmax = ox + roi, ymax = oy + roi;
  const int W = dem.stride();
  const int obase = dem.base(ox, oy);
  const int oalt = dem.at(obase) + a.oht;
  const float foalt = i2f(oalt), ftht = i2f(a.tht);
  const int r0 = kHalf && half ? roi : 0;
  const int nrays = !kHalf ? 4 * side : half ? 4 * roi - 1 : 4 * roi + 1;
  for (int t = threadIdx.x; t < nrays; t += blockDim.x) {
    const int ip = kHalf ? half_ray(t, roi, half) : t;
    int tx, ty;
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
    const bool my = abs(dx) < abs(dy);
    const int dmaj = my ? dy : dx, dmin = my ? dx : dy;
    const float slope = fdiv(i2f(dmin), i2f(dmaj));
    const int dir = dmaj > 0 ? 1 : -1;
    // i*slope = |i| * (dir*slope) exactly (negation is exact), so the minor
    // offset of step k is round(k * sl).
    const float sl = dir > 0 ? slope : -slope;
    const int omaj = my ? oy : ox, omin = my ? ox : oy;
    // The ray stops at the DEM edge along the major axis (kedge steps), when
    // the minor coordinate leaves the DEM, or outside the roi circle
    // (siting.cpp:333-334).  |round(k*sl)| never decreases with k, so the last
    // two hold from some step on and a binary search finds the last step.
    int lo = 0, hi = min(dmaj * dir, dir > 0 ? n - 1 - omaj : omaj);
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      const int off = round_i(fmul(i2f(mid), sl));
      if ((unsigned)(omin + off) < (unsigned)n && mid * mid + off * off <= roi2)
        lo = mid;
      else
        hi = mid - 1;
    }
    const int kend = lo;
    const int smaj = my ? dir : dir * W, smin = my ? W : 1;
    // y-major rays mark the row-major image (line = row), x-major rays the
    // column-major one (line = column); pos is the cell's coordinate along
    // the ray's axis, bit pos%32 of word line*stride + pos/32
    const uint32_t img = smem_u32(my ? im.R : im.C);  // shared-memory address
    const int stride = my ? im.rs : im.cs;
    // the image line of minor offset 0 and the start's position along the
    // line, rows counted from r0
    const int lroi = my ? roi - r0 : roi;
    int pb = obase, pos = my ? roi : roi - r0;
    const float fend = i2f(kend);
    // elevations and offsets are integers below 2^24: their differences and
    // sums are exact in FP32, so (float)(pelev - oalt) = pelev_f - foalt
    float hs = -99999.f;
    if constexpr (kRcp && Dem::kShared) {
      // the sign of |i|*slope is the slope's: round's addend is fixed per ray
      const float hsl = round_addend(sl);
      // The table division costs a few instructions: every step divides and
      // takes the larger slope (s > hs ? s : hs, the reference's update),
      // with no branch for the lanes of a warp to diverge on (window in
      // shared memory; through L1 the extra table read per step costs more).
      uint32_t rp = rcp + 4u;  // &rcp[|i|]
      // the cell's shared-memory byte address, advanced by byte strides (no
      // scaling of an element offset at every step)
      uint32_t pbb = dem.s + 2u * (uint32_t)obase;
      const int smajb = 2 * smaj, sminb = 2 * smin;
#pragma unroll 2  // two steps a trip: half the loop tests and branches
      for (float fai = 1.f; fai <= fend; fai = fadd(fai, 1.f)) {  // fai = (float)|i|, exact
        pbb += smajb;
        pos += dir;
        const int off = f2i(fadd(fmul(fai, sl), hsl));  // round(|i|*slope), half away from zero
        unsigned short ev;
        asm("ld.shared.u16 %0, [%1];" : "=h"(ev) : "r"(pbb + off * sminb));
        const float fe = i2f(ev);
        const float fa = __fsub_rn(fe, foalt);
        float y;
        asm("ld.shared.f32 %0, [%1];" : "=f"(y) : "r"(rp));
        rp += 4u;
        const float q0 = __fmul_rn(fa, y);
        const float sn = __fmaf_rn(__fmaf_rn(-q0, fai, fa), y, q0);
        hs = hs < sn ? sn : hs;
        const float t = fmul(hs, fai);
        // pelev + tht against oalt + hs*|i|: both sums in one packed add
        const unsigned long long V = f2_add(f2_pack(fe, foalt), f2_pack(ftht, t));
        if (f2_lo(V) >= f2_hi(V))
          asm volatile("red.shared.or.b32 [%0], %1;" ::"r"(img + 4u * (uint32_t)((off + lroi) * stride + (pos >> 5))),
                       "r"(__funnelshift_l(0u, 1u, pos)) : "memory");  // 1 << (pos & 31)
      }
    } else {
      for (float fai = 1.f; fai <= fend; fai = fadd(fai, 1.f)) {  // fai = (float)|i|, exact
        pb += smaj;
        pos += dir;
        const int off = round_i(fmul(fai, sl));
        const float fe = i2f(dem.at(pb + off * smin));
        const float fa = __fsub_rn(fe, foalt);
        // s = RN(a/|i|) can exceed hs only if a > hs*|i|, and then t = RN(hs*|i|)
        // <= a (rounding is monotone and a is a float): the division runs only
        // when the horizon may rise, and t serves the visibility test as well
        float t = fmul(hs, fai);
        if (t <= fa) {
          float sn;
          if (kRcp) {
            float y;
            asm("ld.shared.f32 %0, [%1];" : "=f"(y) : "r"(rcp + 4u * (uint32_t)__float2int_rz(fai)));
            const float q0 = __fmul_rn(fa, y);
            sn = __fmaf_rn(__fmaf_rn(-q0, fai, fa), y, q0);
          } else {
            sn = fdiv(fa, fai);
          }
          if (hs < sn) {
            hs = sn;
            t = fmul(hs, fai);
          }
        }
        const unsigned long long V = f2_add(f2_pack(fe, foalt), f2_pack(ftht, t));
        if (f2_lo(V) >= f2_hi(V))
          asm volatile("red.shared.or.b32 [%0], %1;" ::"r"(img + 4u * (uint32_t)((off + lroi) * stride + (pos >> 5))),
                       "r"(1u << (pos & 31)) : "memory");
      }
    }
  }
}

// One observer (whole window) or one half of one (kHalf: block 2o is the
// upper half of observer o, block 2o+1 the lower).
template <bool kSmem, bool kRcp, bool kHalf>
__device__ __forceinline__ void shed_body(const CUtensorMap &map, const ShedArgs &a) {
  extern __shared__ __align__(128) unsigned char sm[];
  const int nr = 2 * a.roi + 1, nwpr = (nr + 63) / 64, nwords = nr * nwpr;
  const int half = kHalf ? (int)(blockIdx.x & 1u) : 0;
  const int obi = kHalf ? (int)(blockIdx.x >> 1) : (int)blockIdx.x;
  const int r0 = half * a.roi;          // first shed row of this CTA's images
  const int nri = kHalf ? a.roi + 1 : nr;  // rows of its images and window
  // the shed rows this CTA writes: the upper half owns row roi
  const int wr0 = kHalf && half ? a.roi + 1 : 0, wr1 = kHalf && !half ? a.roi + 1 : nr;
  const int ob = a.obs[obi];
  if (ob < 0 || ob >= a.n * a.n) {  // invalid observer: empty shed, flagged
    uint64_t *dst = a.sheds + (size_t)obi * nwords;
    for (int i = wr0 * nwpr + threadIdx.x; i < wr1 * nwpr; i += blockDim.x) dst[i] = 0ull;
    if (threadIdx.x == 0) atomicOr(a.err, kErrBadInput);
    return;
  }
  const int ox = ob / a.n, oy = ob - (ob / a.n) * a.n;
  const int hx0 = ox - a.roi + r0, hy0 = (oy - a.roi) & ~7;  // window origin, 16-byte aligned
  uint16_t *win = reinterpret_cast<uint16_t *>(sm);
  const uint32_t win_bytes = kSmem ? (uint32_t)a.nboxes * a.box_rows * a.win_w * 2u : 0u;
  uint64_t *mbar = reinterpret_cast<uint64_t *>(sm + win_bytes);
  ShedImage im;
  im.rs = shed_row_stride(nr);
  im.cs = shed_col_stride(nri);
  im.R = reinterpret_cast<unsigned *>(sm + win_bytes + 16);
  im.C = im.R + nri * im.rs;
  const int img_words = nri * im.rs + shed_col_count(nr) * im.cs;
  float *rcp = reinterpret_cast<float *>(im.R + img_words);  // rcp[k] = RN(1/k)
  if (kRcp)
    for (int i = threadIdx.x; i <= a.roi; i += blockDim.x) rcp[i] = i ? __frcp_rn((float)i) : 0.f;
  if (kSmem && threadIdx.x == 0) {
    mbar_init(mbar, 1);
    mbar_expect_tx(mbar, win_bytes);
    for (int b = 0; b < a.nboxes; b++)
      tma_load_window(win + (size_t)b * a.box_rows * a.win_w, &map, hy0, hx0 + b * a.box_rows,
                      mbar);
  }
  for (int i = threadIdx.x; i < img_words; i += blockDim.x) im.R[i] = 0u;
  __syncthreads();
  if (threadIdx.x == 0 && !half) mark_row_major(im, a.roi, a.roi);  // siting.cpp:279
  if (kSmem) {
    if (!mbar_wait(mbar, 0)) {
      if (threadIdx.x == 0) atomicOr(a.err, kErrTmaTimeout);
      return;
    }
    sweep_rays<kRcp, kHalf>(SmemDem{smem_u32(win), a.win_w, hx0, hy0}, a, ox, oy, im,
                            smem_u32(rcp), half);
  } else {
    sweep_rays<kRcp, kHalf>(GlobalDem{a.dem, a.pitch}, a, ox, oy, im, smem_u32(rcp), half);
  }
  __syncthreads();
  // fold C into R: one warp per 32x32 block; lane j holds column cb*32+j's
  // bits of rows rb*32..+31, a 5-stage butterfly transpose leaves row rb*32+i
  // in lane i (bit j = column cb*32+j), R's own bit order
  const int nbr = (nri + 31) / 32, nbc = (nr + 31) / 32;
  const int lane = threadIdx.x & 31;
  for (int blk = threadIdx.x >> 5; blk < nbr * nbc; blk += blockDim.x >> 5) {
    const int rb = blk / nbc, cb = blk - rb * nbc;
    unsigned x = im.C[(cb * 32 + lane) * im.cs + rb];
    if (!__any_sync(0xffffffffu, x != 0u)) continue;
#pragma unroll
    for (int sh = 16; sh >= 1; sh >>= 1) {
      const unsigned m = sh == 16 ? 0x0000FFFFu : sh == 8 ? 0x00FF00FFu : sh == 4 ? 0x0F0F0F0Fu
                         : sh == 2 ? 0x33333333u : 0x55555555u;
      const unsigned o = __shfl_xor_sync(0xffffffffu, x, sh);
      x = (lane & sh) ? (x & ~m) | ((o >> sh) & m) : (x & m) | ((o << sh) & ~m);
    }
    const int row = rb * 32 + lane;
    if (row < nri && x) im.R[row * im.rs + cb] |= x;
  }
  __syncthreads();
  uint64_t *dst = a.sheds + (size_t)obi * nwords;
  for (int i = wr0 * nwpr + threadIdx.x; i < wr1 * nwpr; i += blockDim.x) {
    const int r = i / nwpr, q = i - r * nwpr;
    const unsigned *src = im.R + (r - r0) * im.rs + 2 * q;
    dst[i] = ((uint64_t)__brev(src[0]) << 32) | __brev(src[1]);
  }
}

// CTAs of at most 800 threads compiled for two resident CTAs per SM (two
// observers' windows in flight; the per-partition register file then allows
// 32 registers per thread).
template <bool kSmem, bool kRcp>
__global__ void __launch_bounds__(800, 2)
    shed_kernel2(const __grid_constant__ CUtensorMap map, const ShedArgs a) {
  shed_body<kSmem, kRcp, false>(map, a);
}

// Half windows, staged, one ray a thread: kThreads = 32*ceil((4roi+1)/32),
// compiled for kMinBlocks resident CTAs per SM (what the window allows).
template <int kThreads, int kMinBlocks>
__global__ void __launch_bounds__(kThreads, kMinBlocks)
    shed_half_kernel(const __grid_constant__ CUtensorMap map, const ShedArgs a) {
  shed_body<true, true, true>(map, a);
}

int round8(int v) { return (v + 7) & ~7; }

struct WinGeom {
  int w, box_rows, nboxes;
};

WinGeom win_geom(int roi, bool half) {
  WinGeom g;
  const int nr = half ? roi + 1 : 2 * roi + 1;  // window rows
  g.w = round8(2 * roi + 8);
  g.nboxes = (nr + 255) / 256;
  g.box_rows = round8((nr + g.nboxes - 1) / g.nboxes);
  return g;
}

// Half windows are launched for roi 60..151 (4roi+1 rays in at most 608
// threads).  16384 observers on a 2048^2 DEM, half against whole windows:
// roi 25 +8%, 50 +0.5%, 75 -1.5%, 100 -8% (staged whole window); 110-120
// -23..25%, 125-150 -9..13% (whole window through L1).  Below roi 60 the
// halves' CTAs are too small (a few warps) to gain.
constexpr int kHalfMinRoi = 60, kHalfMaxRoi = 151;

}  // namespace

size_t shed_smem_bytes(const ShedPlan &p, int roi) {
  const int nr = 2 * roi + 1, nri = p.half ? roi + 1 : nr;  // image rows
  size_t b = 16 + 4 * ((size_t)nri * shed_row_stride(nr) + (size_t)shed_col_count(nr) * shed_col_stride(nri));
  b += 4 * ((size_t)roi + 1);  // reciprocal table
  if (p.use_smem) {
    const WinGeom g = win_geom(roi, p.half);
    b += (size_t)g.nboxes * g.box_rows * g.w * 2;
  }
  return b;
}

namespace {

// One CTA an observer: one ray per thread up to 800 rays (two resident CTAs
// per SM at 32 registers a thread), else an even split into rounds of at most
// 800 (a single 1024-thread CTA per SM ran 1.5x slower per ray step, roi
// 104-128).  The window is staged only while two CTAs of a full round of rays
// still share an SM: a ray's steps form one dependent chain, so fewer
// resident warps cannot hide the shared-memory latency and the L1 path, with
// more resident CTAs, is faster.
ShedPlan shed_whole_plan(int roi) {
  const int rays = 8 * roi;
  const int rounds = (rays + 799) / 800;
  const int threads = std::min(800, ((rays + rounds - 1) / rounds + 31) / 32 * 32);
  ShedPlan p{std::max(threads, 64), true, false};
  if (rounds > 1 || shed_smem_bytes(p, roi) > 112 * 1024) p.use_smem = false;
  return p;
}

// Two CTAs an observer, each staging its half window, one ray a thread.
ShedPlan shed_half_plan(int roi) { return ShedPlan{(4 * roi + 1 + 31) / 32 * 32, true, true}; }

}  // namespace

ShedPlan shed_default_plan(int roi) {
  return roi >= kHalfMinRoi && roi <= kHalfMaxRoi ? shed_half_plan(roi) : shed_whole_plan(roi);
}

// smem: 1 half windows (up to roi 151, else as 2), 2 the whole window,
// staged where it fits, 0 the whole window through L1, -1 the default.
ShedPlan shed_plan_for(int roi, int smem) {
  if (smem == 1 && roi >= 1 && roi <= kHalfMaxRoi) return shed_half_plan(roi);
  if (smem == 1 || smem == 2) return shed_whole_plan(roi);
  if (smem == 0) {
    ShedPlan p = shed_whole_plan(roi);
    p.use_smem = false;
    return p;
  }
  return shed_default_plan(roi);
}

cudaError_t launch_sheds(const DemView &dem, int roi, int oht, int tht, int nsheds,
                         const int32_t *obs, uint64_t *sheds, const ShedPlan &plan, int *d_err,
                         cudaStream_t st) {
  if (nsheds <= 0) return cudaSuccess;
  ShedArgs a{};
  a.dem = dem.data;
  a.pitch = dem.pitch;
  a.n = dem.nrows;
  a.roi = roi;
  a.oht = oht;
  a.tht = tht;
  a.nsheds = nsheds;
  a.obs = obs;
  a.sheds = sheds;
  a.err = d_err;
  // the reciprocal-table division is exhaustively checked for |a| <= 2^21
  // (heights up to 10^6 over 16-bit elevations) and steps up to 2048
  const bool rcp = roi <= 2048 && oht >= 0 && oht <= 1000000;
  // half windows need the staged window and the table division
  ShedPlan eff = plan;
  if (eff.half && (!rcp || !dem.tma_ok || roi < 1 || roi > kHalfMaxRoi)) eff = shed_whole_plan(roi);
  eff.use_smem = eff.use_smem && dem.tma_ok;
  CUtensorMap map;
  memset(&map, 0, sizeof(map));
  if (eff.use_smem) {
    const WinGeom g = win_geom(roi, eff.half);
    a.win_w = g.w;
    a.box_rows = g.box_rows;
    a.nboxes = g.nboxes;
    if (!make_dem_tensor_map(&map, dem, g.w, g.box_rows)) return cudaErrorInvalidValue;
  }
  const size_t shm = shed_smem_bytes(eff, roi);
  auto launch = [&](auto kern, int ctas) -> cudaError_t {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm);
    if (e != cudaSuccess) return e;
    kern<<<ctas, eff.threads, shm, st>>>(map, a);
    return cudaSuccess;
  };
  cudaError_t e;
  if (eff.half) {
    // the variant compiled for as many resident CTAs as the window allows
    e = eff.threads <= 416   ? launch(shed_half_kernel<416, 4>, 2 * nsheds)
        : eff.threads <= 512 ? launch(shed_half_kernel<512, 3>, 2 * nsheds)
                             : launch(shed_half_kernel<608, 2>, 2 * nsheds);
  } else if (eff.use_smem) {
    e = rcp ? launch(shed_kernel2<true, true>, nsheds) : launch(shed_kernel2<true, false>, nsheds);
  } else {
    e = rcp ? launch(shed_kernel2<false, true>, nsheds) : launch(shed_kernel2<false, false>, nsheds);
  }
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

}  // namespace siting
