// SITE: greedy observer selection (siting.cpp:366-626, seqsite argmax).
//
// Reference semantics reproduced exactly:
//   * gain(c) = cells of c's viewshed not yet covered (popcount of the shed
//     shifted into the coverage bitmap, AND-NOT coverage);
//   * round 1 scores every candidate; later rounds rescore only unused
//     candidates within 2*roi of the last pick (a viewshed is a disc of
//     radius roi, so no other gain can change);
//   * with intervis, a rescored candidate whose own cell is not covered gets
//     area 0; a candidate never rescored keeps its round-1 area;
//   * pick = lowest index with the largest area > 0; stop at area 0 or when
//     100.0*cumarea/n^2 > 95 (after adding the pick).
//
// GB300 mapping: one cooperative persistent kernel of G CTAs (one per SM).
// Candidate c is owned by CTA c % G, which keeps its true gain, area, cell and
// used flag in shared memory and a per-32-slot max tree of the keys
// (area << 32 | ~c).  Each round every CTA
//   1. reads the G published CTA maxima {key, cell} and reduces them to the
//      pick (all CTAs agree; no second barrier is needed),
//   2. computes the pick's newly covered bits N = placed(shed_p) & ~cum into
//      shared memory (self-check: popcount(N) must equal the pick's area),
//   3. finds its own unused candidates within 2*roi of the pick (block
//      rectangle of the FINDMAX geometry, stepping by G) and subtracts
//      popcount(placed(shed_c) & N) from their gains: exact, because
//      |V_c \ (C u N)| = |V_c \ C| - |V_c n N| when N n C is empty,
//   4. applies the intervis gate, refreshes the touched groups of its max
//      tree and publishes its new maximum into the other parity slot.
// CTA 0 also ORs N (and the previous round's N) into the second coverage
// buffer, so the buffer read in a round is never written in it; one bounded
// barrier per round orders everything.  The initial scores (popcount of every
// shed, 128-bit loads) stream all sheds once at HBM bandwidth.
#include <algorithm>
#include <cmath>

#include "common.cuh"
#include "kernels.h"

namespace siting {
namespace {

constexpr int kSiteThreads = 1024;
constexpr int kMaxSlots = 4096;  // candidates owned by one CTA

struct SiteArgs {
  int n, roi, intervis, nsheds, G;
  const int32_t *obs;
  const uint64_t *sheds;
  float bs;
  int nb, npb;
  uint64_t *cum0, *cum1;
  unsigned long long *slots;  // [2][G] x {key, cell}
  unsigned *bar;
  long long *out;
  int32_t *order;
  uint8_t *selected;
  const int *gains;  // round-1 gains, from site_score_kernel
  int *err;
  int nslots, list_cap;
  long long stop_area;  // smallest cumarea with 100.0*cumarea/n^2 > 95 (host-computed)
};

__device__ __forceinline__ void shed_align(int c0, int &fw, int &fb) {
  fw = c0 >> 6;  // floor division by 64 (siting.cpp:400-405)
  fb = c0 & 63;
}

// Word `j` (0..nwpr) of a shed row shifted so that the shed's column 0 lands
// at bit position fb of word 0.
__device__ __forceinline__ uint64_t placed_word(const uint64_t *row, int j, int nwpr, int fb) {
  const uint64_t cur = j < nwpr ? __ldg(row + j) : 0ull;
  const uint64_t prev = j > 0 ? __ldg(row + j - 1) : 0ull;
  uint64_t v = cur >> fb;
  if (fb) v |= prev << (64 - fb);
  return v;
}

__device__ __forceinline__ unsigned long long make_key(int area, int c) {
  return ((unsigned long long)(unsigned)area << 32) | (unsigned long long)(0xFFFFFFFFu - (unsigned)c);
}

struct KeyPos {
  unsigned long long key;
  int pos;
};

__device__ __forceinline__ KeyPos warp_argmax(KeyPos v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long k = __shfl_xor_sync(0xffffffffu, v.key, o);
    const int p = __shfl_xor_sync(0xffffffffu, v.pos, o);
    if (k > v.key) {
      v.key = k;
      v.pos = p;
    }
  }
  return v;
}

// Round 1 (siting.cpp:537-549 with nusedsheds == 0): the gain of every
// candidate against an empty coverage is the popcount of its shed.  One warp
// per shed, 128-bit loads, grid-stride: a pure HBM stream over all sheds.
__global__ void __launch_bounds__(256) site_score_kernel(const uint64_t *sheds, int nsheds,
                                                         int per, int *gains) {
  const int lane = threadIdx.x & 31;
  const int warps = gridDim.x * (blockDim.x >> 5);
  for (int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < nsheds; c += warps) {
    const uint64_t *sh = sheds + (size_t)c * per;
    int cnt = 0;
    if ((per & 1) == 0) {
      const ulonglong2 *v = reinterpret_cast<const ulonglong2 *>(sh);
      for (int i = lane; i < per / 2; i += 32) {
        const ulonglong2 q = __ldg(v + i);
        cnt += __popcll(q.x) + __popcll(q.y);
      }
    } else {
      for (int i = lane; i < per; i += 32) cnt += __popcll(__ldg(sh + i));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    if (lane == 0) gains[c] = cnt;
  }
}

__global__ void __launch_bounds__(kSiteThreads, 1) site_kernel(const SiteArgs a) {
  extern __shared__ __align__(16) unsigned char sm[];
  __shared__ unsigned long long s_rkey[32];
  __shared__ int s_rpos[32];
  __shared__ unsigned long long s_bestkey;
  __shared__ int s_bestpos, s_nlist, s_flag, s_ncount;

  const int G = a.G, k = blockIdx.x;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
  const int n = a.n, roi = a.roi, nr = 2 * roi + 1, nwpr = (nr + 63) / 64, nbw = nwpr + 1;
  const int cw = (n + 63) / 64;
  const size_t per = (size_t)nr * nwpr;
  const int my_slots = k < a.nsheds ? (a.nsheds - k + G - 1) / G : 0;
  const int ngroups = (a.nslots + 31) / 32;

  // shared-memory carve-up (sizes mirrored by site_smem_bytes)
  unsigned char *p = sm;
  uint64_t *nbuf0 = reinterpret_cast<uint64_t *>(p);
  p += (size_t)nr * nbw * 8;
  uint64_t *nbuf1 = reinterpret_cast<uint64_t *>(p);
  p += (size_t)nr * nbw * 8;
  unsigned long long *s_gmax = reinterpret_cast<unsigned long long *>(p);
  p += (size_t)ngroups * 8;
  int *s_gain = reinterpret_cast<int *>(p);
  p += (size_t)a.nslots * 4;
  int *s_area = reinterpret_cast<int *>(p);
  p += (size_t)a.nslots * 4;
  int *s_pos = reinterpret_cast<int *>(p);
  p += (size_t)a.nslots * 4;
  int *s_list = reinterpret_cast<int *>(p);
  p += (size_t)a.list_cap * 4;
  int *s_delta = reinterpret_cast<int *>(p);
  p += (size_t)a.list_cap * 4;
  unsigned char *s_cov = p;
  p += a.list_cap;
  unsigned char *s_used = p;
  p += a.nslots;
  unsigned char *s_dirty = p;

  GroupBarrier gb{a.bar, (unsigned)G, 0u};
  // tracing: device cycles per phase, accumulated by CTA 0's thread 0
  long long ph[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  long long tmark = clock64();
  auto mark = [&](int i) {
    if (k == 0 && tid == 0) {
      const long long now = clock64();
      ph[i] += now - tmark;
      tmark = now;
    }
  };

  // ---- own candidates: round-1 gains from the scoring kernel ----------------
  for (int s = tid; s < a.nslots; s += blockDim.x) {
    if (s < my_slots) {
      const int c = s * G + k;
      const int g = __ldcg(a.gains + c);
      s_gain[s] = g;
      s_area[s] = g;
      s_pos[s] = __ldg(a.obs + c);
      s_used[s] = 0;
    } else {
      s_gain[s] = 0;
      s_area[s] = 0;
      s_pos[s] = 0;
      s_used[s] = 1;
    }
  }
  for (int g = tid; g < ngroups; g += blockDim.x) s_dirty[g] = 1;
  __syncthreads();
  mark(0);

  long long cumarea = 0;
  int npicks = 0;
  uint64_t *X = a.cum0, *Y = a.cum1;
  uint64_t *ncur = nbuf0, *nprev = nbuf1;
  int prev_px = 0, prev_fw = 0, cur_px = 0, cur_fw = 0;

  for (;;) {
    // ---- refresh dirty groups and publish this CTA's maximum --------------
    for (int g = warp; g < ngroups; g += nwarps) {
      if (!s_dirty[g]) continue;
      const int s = g * 32 + lane;
      unsigned long long key = 0;
      if (s < my_slots && !s_used[s]) key = make_key(s_area[s], s * G + k);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long w = __shfl_xor_sync(0xffffffffu, key, o);
        key = w > key ? w : key;
      }
      if (lane == 0) {
        s_gmax[g] = key;
        s_dirty[g] = 0;
      }
    }
    __syncthreads();
    if (warp == 0) {
      unsigned long long key = 0;
      for (int g = lane; g < ngroups; g += 32) key = s_gmax[g] > key ? s_gmax[g] : key;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long w = __shfl_xor_sync(0xffffffffu, key, o);
        key = w > key ? w : key;
      }
      if (lane == 0) {
        int pos = 0;
        if (key) {
          const int c = (int)(0xFFFFFFFFu - (unsigned)(key & 0xFFFFFFFFull));
          pos = s_pos[c / G];
        }
        unsigned long long *slot = a.slots + ((size_t)(npicks & 1) * G + k) * 2;
        __stcg(slot, key);
        __stcg(slot + 1, (unsigned long long)pos);
      }
    }
    mark(1);
    if (!group_sync(gb, a.err, &s_flag)) return;
    mark(2);
    if (npicks > 0) {  // the buffer written last round is complete: read it now
      uint64_t *tmp = X;
      X = Y;
      Y = tmp;
      uint64_t *tb = ncur;
      ncur = nprev;
      nprev = tb;
      prev_px = cur_px;
      prev_fw = cur_fw;
    }

    // ---- 1. agree on the pick ---------------------------------------------
    if (warp * 32 < G) {
      KeyPos v{0ull, 0};
      if (tid < G) {
        const unsigned long long *slot = a.slots + ((size_t)(npicks & 1) * G + tid) * 2;
        v.key = __ldcg(slot);
        v.pos = (int)__ldcg(slot + 1);
      }
      v = warp_argmax(v);
      if (lane == 0) {
        s_rkey[warp] = v.key;
        s_rpos[warp] = v.pos;
      }
    }
    if (G > 32) __syncthreads();
    if (warp == 0) {
      KeyPos w{0ull, 0};
      if (lane * 32 < G) {
        w.key = s_rkey[lane];
        w.pos = s_rpos[lane];
      }
      w = warp_argmax(w);
      if (lane == 0) {
        s_bestkey = w.key;
        s_bestpos = w.pos;
        s_nlist = 0;
        s_ncount = 0;
      }
    }
    __syncthreads();
    mark(3);
    const unsigned long long bkey = s_bestkey;
    const int area = (int)(bkey >> 32);
    if (area <= 0) break;
    const int pc = (int)(0xFFFFFFFFu - (unsigned)(bkey & 0xFFFFFFFFull));
    const int bpos = s_bestpos;
    cumarea += area;
    if (tid == 0) {
      if (pc % G == k) {
        const int s = pc / G;
        s_used[s] = 1;
        s_dirty[s >> 5] = 1;
        a.selected[pc] = 1;
      }
      if (k == 0) a.order[npicks] = pc;
    }
    npicks++;
    if (cumarea >= a.stop_area) break;  // 100.0*cumarea/n^2 > 95 (siting.cpp:602-604)

    // ---- 2. newly covered bits of the pick --------------------------------
    const int px = bpos / n, py = bpos - (bpos / n) * n;
    int fwp, fbp;
    shed_align(py - roi, fwp, fbp);
    cur_px = px;
    cur_fw = fwp;
    {
      const uint64_t *shp = a.sheds + (size_t)pc * per;
      int cnt = 0;
      for (int i = tid; i < nr * nbw; i += blockDim.x) {
        const int prow = i / nbw, j = i - prow * nbw;
        const int gr = px - roi + prow, W = fwp + j;
        uint64_t v = 0;
        if (gr >= 0 && gr < n && W >= 0 && W < cw)
          v = placed_word(shp + (size_t)prow * nwpr, j, nwpr, fbp) & ~__ldcg(X + (size_t)gr * cw + W);
        ncur[i] = v;
        cnt += __popcll(v);
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
      if (lane == 0 && cnt) atomicAdd(&s_ncount, cnt);
    }

    // ---- 3a. own unused candidates within 2*roi of the pick ---------------
    {
      const float r2f = (float)(2 * roi);
      const int bxl = max(0, (int)floorf(((float)px - r2f) / a.bs) - 2);
      const int bxh = min(a.nb - 1, (int)floorf(((float)px + r2f) / a.bs) + 2);
      const int byl = max(0, (int)floorf(((float)py - r2f) / a.bs) - 2);
      const int byh = min(a.nb - 1, (int)floorf(((float)py + r2f) / a.bs) + 2);
      const int run = (byh - byl + 1) * a.npb;  // contiguous indices per block row
      const int per_run = run / G + 2;
      const int items = (bxh - bxl + 1) * per_run;
      const int lim = 4 * roi * roi;
      for (int i = tid; i < items; i += blockDim.x) {
        const int r = i / per_run, m = i - r * per_run;
        const int start = ((bxl + r) * a.nb + byl) * a.npb;
        const int c = start + ((k - start % G) + G) % G + m * G;
        if (c >= start + run || c >= a.nsheds) continue;
        const int s = c / G;
        if (s_used[s]) continue;
        const int cp = s_pos[s];
        const int dx = cp / n - px, dy = cp - (cp / n) * n - py;
        if (dx * dx + dy * dy > lim) continue;
        const int idx = atomicAdd(&s_nlist, 1);
        if (idx < a.list_cap) {
          s_list[idx] = s;
          s_delta[idx] = 0;
          s_cov[idx] = 0;
        } else {
          atomicOr(a.err, kErrCapacity);
        }
      }
    }
    __syncthreads();
    mark(4);
    if (tid == 0 && s_ncount != area) atomicOr(a.err, kErrSiteMismatch);
    const int nlist = min(s_nlist, a.list_cap);

    // ---- coverage buffer for next round: this CTA's rows of N_t and N_{t-1}
    for (int i = tid; i < nr * nbw; i += blockDim.x) {
      const int prow = i / nbw;
      if (prow % G != k) continue;
      const int j = i - prow * nbw;
      uint64_t v = ncur[i];
      int gr = cur_px - roi + prow, W = cur_fw + j;
      if (v && gr >= 0 && gr < n && W >= 0 && W < cw)
        atomicOr(reinterpret_cast<unsigned long long *>(Y + (size_t)gr * cw + W), v);
      if (npicks > 1) {
        v = nprev[i];
        gr = prev_px - roi + prow;
        W = prev_fw + j;
        if (v && gr >= 0 && gr < n && W >= 0 && W < cw)
          atomicOr(reinterpret_cast<unsigned long long *>(Y + (size_t)gr * cw + W), v);
      }
    }

    // ---- 3b. subtract the overlap with N; coverage bit of own cell ----------
    for (int i = tid; i < nlist * nr; i += blockDim.x) {
      const int li = i / nr, r = i - li * nr;
      const int s = s_list[li];
      const int cp = s_pos[s];
      const int cx = cp / n, cy = cp - cx * n;
      const int gr = cx - roi + r, prow = gr - (px - roi);
      if (a.intervis && r == roi) {  // the candidate's own cell: covered after p?
        int cov = (int)((__ldcg(X + (size_t)cx * cw + (cy >> 6)) >> (63 - (cy & 63))) & 1ull);
        const int j = (cy >> 6) - fwp;
        if (!cov && prow >= 0 && prow < nr && j >= 0 && j < nbw)
          cov = (int)((ncur[prow * nbw + j] >> (63 - (cy & 63))) & 1ull);
        s_cov[li] = (unsigned char)cov;
      }
      if (prow < 0 || prow >= nr || gr < 0 || gr >= n) continue;
      int fwc, fbc;
      shed_align(cy - roi, fwc, fbc);
      const int lwc = (cy + roi) >> 6;
      const int lo = max(max(fwc, fwp), 0), hi = min(min(lwc, fwp + nwpr), cw - 1);
      if (lo > hi) continue;
      const uint64_t *row = a.sheds + (size_t)(s * G + k) * per + (size_t)r * nwpr;
      const uint64_t *nrow = ncur + prow * nbw;
      int d = 0;
      for (int W = lo; W <= hi; W++)
        d += __popcll(placed_word(row, W - fwc, nwpr, fbc) & nrow[W - fwp]);
      if (d) atomicAdd(&s_delta[li], d);
    }
    __syncthreads();
    mark(5);

    // ---- 4. new gains, intervis gate, dirty groups --------------------------
    for (int li = tid; li < nlist; li += blockDim.x) {
      const int s = s_list[li];
      const int g = s_gain[s] - s_delta[li];
      s_gain[s] = g;
      s_area[s] = (!a.intervis || s_cov[li]) ? g : 0;
      s_dirty[s >> 5] = 1;
    }
    __syncthreads();
    mark(6);
  }

  if (k == 0 && tid == 0) {
    a.out[0] = npicks;
    a.out[1] = cumarea;
    a.out[2] = npicks;
    for (int i = 0; i < 7; i++) a.out[3 + i] = ph[i];
  }
}

struct SiteGeomLimits {
  int list_cap;
};

int site_list_cap(int roi, int nsheds, int G, int nb, int npb, float bs) {
  const int span_blocks = (int)std::ceil((4.0 * roi + 1.0) / bs) + 4;
  const int nbx = std::min(nb, span_blocks);
  const int run = std::min(nb, span_blocks) * npb;
  long long cap = (long long)nbx * (run / G + 2);
  cap = std::min<long long>(cap, (nsheds + G - 1) / G);
  return (int)std::max<long long>(cap, 1);
}

}  // namespace

// The reference stops once 100.0 * cumarea / square(nrows) > 95, evaluated in
// double (siting.cpp:602-604).  The expression is non-decreasing in cumarea,
// so the first cumarea where it holds is found once, on the host, with the
// same double arithmetic; the kernel then compares integers.
long long site_stop_area(int nrows) {
  const int sq = nrows * nrows;
  auto over = [&](long long c) { return 100.0 * (int)c / sq > 95; };
  long long lo = 0, hi = (long long)sq + 1;  // over(hi) is true
  while (lo < hi) {
    const long long mid = lo + (hi - lo) / 2;
    if (over(mid))
      hi = mid;
    else
      lo = mid + 1;
  }
  return lo;
}

size_t site_scratch_bytes(int nrows, int nsheds, int nctas) {
  const size_t cw = (size_t)(nrows + 63) / 64;
  size_t b = 2 * (size_t)nrows * cw * 8;
  b += (size_t)2 * nctas * 2 * 8;
  b += 256;  // barrier + out
  b += 2 * (((size_t)nsheds * 4 + 255) & ~(size_t)255);  // order + gains
  return b + 1024;
}

void site_carve_scratch(void *base, int nrows, int nsheds, int nctas, SiteScratch *s) {
  const size_t cw = (size_t)(nrows + 63) / 64;
  unsigned char *p = static_cast<unsigned char *>(base);
  auto take = [&](size_t bytes) {
    unsigned char *q = p;
    p += (bytes + 255) & ~(size_t)255;
    return q;
  };
  s->cum[0] = reinterpret_cast<uint64_t *>(take((size_t)nrows * cw * 8));
  s->cum[1] = reinterpret_cast<uint64_t *>(take((size_t)nrows * cw * 8));
  s->slots = reinterpret_cast<uint64_t *>(take((size_t)2 * nctas * 2 * 8));
  s->bar = reinterpret_cast<unsigned *>(take(64));
  s->out = reinterpret_cast<long long *>(take(64));
  s->order = reinterpret_cast<int32_t *>(take((size_t)nsheds * 4));
  s->gains = reinterpret_cast<int32_t *>(take((size_t)nsheds * 4));
}

// Few CTAs keep the per-round barrier and the redundant reads of the pick's
// shed cheap; enough CTAs keep each one's candidates within kMaxSlots.
int site_default_ctas(int nsheds, int sm_count) {
  int g = std::max(32, (nsheds + kMaxSlots - 1) / kMaxSlots);
  g = std::min(g, std::max(1, nsheds));
  return std::min(g, sm_count);
}

size_t site_smem_bytes(int roi, int nsheds, int nctas, int nblocks, int npb, float blocksize) {
  const int nr = 2 * roi + 1, nwpr = (nr + 63) / 64, nbw = nwpr + 1;
  const int nslots = (nsheds + nctas - 1) / nctas;
  const int ngroups = (nslots + 31) / 32;
  const int cap = site_list_cap(roi, nsheds, nctas, nblocks, npb, blocksize);
  size_t b = 2 * (size_t)nr * nbw * 8;
  b += (size_t)ngroups * 8;
  b += (size_t)nslots * 12;
  b += (size_t)cap * 9;
  b += nslots + ngroups;
  return (b + 15) & ~(size_t)15;
}

bool site_supported(int roi, int nsheds, int nctas) {
  const int nslots = (nsheds + nctas - 1) / nctas;
  return nslots <= kMaxSlots && roi <= 1000;
}

cudaError_t launch_site(int nrows, int roi, int intervis, int nsheds, const int32_t *obs,
                        const uint64_t *sheds, float blocksize, int nblocks, int npb,
                        uint8_t *selected, const SiteScratch &s, int nctas, int *d_err,
                        cudaStream_t st) {
  SiteArgs a{};
  a.n = nrows;
  a.roi = roi;
  a.intervis = intervis;
  a.nsheds = nsheds;
  a.G = nctas;
  a.obs = obs;
  a.sheds = sheds;
  a.bs = blocksize;
  a.nb = nblocks;
  a.npb = npb;
  a.cum0 = s.cum[0];
  a.cum1 = s.cum[1];
  a.slots = reinterpret_cast<unsigned long long *>(s.slots);
  a.bar = s.bar;
  a.out = s.out;
  a.order = s.order;
  a.selected = selected;
  a.gains = s.gains;
  a.err = d_err;
  a.nslots = (nsheds + nctas - 1) / nctas;
  a.list_cap = site_list_cap(roi, nsheds, nctas, nblocks, npb, blocksize);
  a.stop_area = site_stop_area(nrows);
  const size_t shm = site_smem_bytes(roi, nsheds, nctas, nblocks, npb, blocksize);
  const int nr = 2 * roi + 1, per = nr * ((nr + 63) / 64);
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int sgrid = std::max(1, std::min(sms * 8, (nsheds + 7) / 8));
  site_score_kernel<<<sgrid, 256, 0, st>>>(sheds, nsheds, per, s.gains);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(site_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm);
  if (e != cudaSuccess) return e;
  void *args[] = {&a};
  return cudaLaunchCooperativeKernel((void *)site_kernel, dim3(nctas), dim3(kSiteThreads), args,
                                     shm, st);
}

}  // namespace siting
