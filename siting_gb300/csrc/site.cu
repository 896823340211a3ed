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
// GB300 mapping: one persistent kernel of G co-resident CTAs (one per SM)
// with a bounded group barrier.  Candidate c is owned by CTA c % G, which
// keeps its true gain, area, cell and flags in shared memory and a top-K key
// list per 32 slots (key = area << 32 | ~c, K = kTopK).  A round:
//   A. every CTA publishes its own top-K keys; one barrier;
//   B. every CTA merges the G lists identically and accepts the longest
//      prefix of the global key order whose members are pairwise > 2*roi
//      apart, up to the exactness threshold (the largest K-th key of any list:
//      unpublished keys are below it) and the 95% stop.  A candidate > 2*roi
//      from every earlier pick of the round keeps its key, every other key
//      can only fall, so the prefix equals the sequential greedy's next picks;
//   C. each CTA lists its unused candidates within 2*roi of each pick;
//   D. and computes |V_c n N_p| for each such pair, N_p = placed(V_p) \ cum
//      the pick's new bits: the exact gain decrease, since the picks' new
//      bits are disjoint.  Small rounds compute N in every CTA's shared
//      memory; larger ones spread its rows over the CTAs (a global buffer
//      read after one more barrier);
//   E. with intervis, a candidate of area 0 whose cell a pick covers can
//      become eligible: each CTA finds the first prefix position it would
//      overtake, and a second barrier takes the minimum (the round's cut);
//   F. the picks before the cut are applied: gains fall by the summed
//      deltas, the intervis gate is re-evaluated, and the coverage bitmap is
//      OR-ed in place (rows spread over the CTAs).  A self-check compares each
//      pick's count of new bits with its area.
// The round-1 gains (popcount of every shed) come from a separate streaming
// kernel at HBM bandwidth.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "kernels.h"
#include "siting.h"

namespace siting {
namespace {

// Threads a CTA: 512 allow 128 registers a thread and suit jobs with few
// candidates per CTA and narrow sheds; 1024 (64 registers) keep more items
// in flight for many candidates per CTA or wide sheds (measured, SITE ms at
// 512 and 1024 threads: 4096^2/roi 100 7.41 vs 7.65; 16384^2/roi 200 51.5 vs
// 42.7).
int site_threads_for(int nslots, int roi) { return (nslots > 1024 || roi > 127) ? 1024 : 512; }
constexpr int kMaxSlots = 4096;  // candidates owned by one CTA
// Keys each CTA publishes per round.  Rounds end at distance conflicts and
// intervis cuts long before the threshold of K keys binds (4096^2: 343
// rounds with 3, 4, 6 or 8), and fewer keys make each merge cheaper; with 2
// the threshold binds (16384^2: 725 -> 1015 rounds).
constexpr int kTopK = 3;
constexpr int kMaxPicks = 64;    // picks accepted in one round at most
constexpr int kSmallRecip = 128; // reciprocals tabled in shared memory (>= kMaxPicks)
constexpr int kMaxPairs = 8192;  // (candidate, pick) pairs one CTA updates per round
constexpr int kMaskCap = 8192;   // shared bytes for a spread round's new-bit word masks

struct SiteArgs {
  int n, roi, intervis, nsheds, G;
  const int32_t *obs;
  const uint64_t *sheds;
  float bs;
  int nb, npb;
  uint64_t *cum0;   // coverage bitmap, updated in place
  uint64_t *nbits;  // [kMaxPicks][nr][nwpr+1]: the round's new bits of each pick
  unsigned char *nmask;  // [kMaxPicks][nr]: bit j set when word j of that row is nonzero
  int ncap_words;   // shared-memory words for a small round's new bits
  unsigned long long *topk;  // [2][G][kTopK] x {key, cell}
  int *cuts;                 // [2][G]: per-CTA cut of the round's prefix (intervis)
  int *ncount;               // [2][kMaxPicks]: popcount of each pick's new bits
  unsigned *bar;
  long long *out;
  int32_t *order;
  uint8_t *selected;
  const int *gains;  // round-1 gains, from site_score_kernel
  int *err;
  int nslots, pick_items, pick_cap, pair_cap;
  long long stop_area;  // smallest cumarea with 100.0*cumarea/n^2 > 95 (host-computed)
  int block0;           // first CTA of this job's group in the launch
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
__device__ __forceinline__ int key_index(unsigned long long key) {
  return (int)(0xFFFFFFFFu - (unsigned)(key & 0xFFFFFFFFull));
}
// Division by an invariant divisor d >= 1: r = ceil(2^64/d) (0 for d = 1)
// gives floor(n/d) = high 64 bits of n*r for every n < 2^32, since n*r/2^64
// exceeds n/d by less than n/2^64 < 1/d (Granlund and Montgomery, 1994).
__host__ __device__ __forceinline__ unsigned long long div_recip(int d) {
  return d > 1 ? ~0ull / (unsigned long long)d + 1ull : 0ull;
}
__device__ __forceinline__ int div_by(int n, unsigned long long r) {
  return r ? (int)__umul64hi((unsigned long long)(unsigned)n, r) : n;
}

// Largest 64-bit key of a full warp by two 32-bit reductions: the largest
// high word, then the largest low word among the lanes that hold it.
__device__ __forceinline__ unsigned long long warp_max_key(unsigned long long key) {
  const unsigned hi = (unsigned)(key >> 32), lo = (unsigned)key;
  const unsigned mh = __reduce_max_sync(0xffffffffu, hi);
  const unsigned ml = __reduce_max_sync(0xffffffffu, hi == mh ? lo : 0u);
  return ((unsigned long long)mh << 32) | ml;
}

// Slot flags
constexpr unsigned char kUsed = 1, kInel = 4;

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

// One launch runs the greedy selection of one or more jobs (DEMs): CTA b
// belongs to job block_job[b]; each job's CTAs form their own group with
// their own barrier, scratch and outputs.
template <int kThreads>
__global__ void __launch_bounds__(kThreads, 1)
    site_kernel(const SiteArgs *__restrict__ jobs, const int *__restrict__ block_job) {
  extern __shared__ __align__(16) unsigned char sm[];
  __shared__ SiteArgs s_args;
  if (threadIdx.x == 0) s_args = jobs[block_job[blockIdx.x]];
  __syncthreads();
  const SiteArgs &a = s_args;
  __shared__ int s_m, s_mcut, s_stop_at, s_done, s_flagv, s_roundcut, s_npair, s_nvalid;
  __shared__ long long s_cum;
  __shared__ int s_poff[kMaxPicks + 1];
  // reciprocals (div_recip) of the kernel's divisors and of each pick's run
  __shared__ unsigned long long s_rG, s_rnr, s_rpcap, s_rm, s_rrows, s_rnb2;
  __shared__ unsigned long long s_rrun[kMaxPicks];
  __shared__ unsigned long long s_rsmall[kSmallRecip + 1];  // div_recip(d), d <= kSmallRecip
  __shared__ int4 s_pbox[kMaxPicks];  // per pick: start of its first block row, run, per_run, items
  __shared__ unsigned long long s_red[32];
  __shared__ int s_rank[kMaxPicks], s_rpos[kMaxPicks];

  const int G = a.G, k = blockIdx.x - a.block0;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
  const int n = a.n, roi = a.roi, nr = 2 * roi + 1, nwpr = (nr + 63) / 64;
  const int nb2 = nwpr + 1;            // words of a placed row
  const int nch = (nb2 + 3) / 4;       // 4-word chunks of a placed row
  const int cw = (n + 63) / 64;
  const size_t per = (size_t)nr * nwpr;
  const int my_slots = k < a.nsheds ? (a.nsheds - k + G - 1) / G : 0;
  const int ngroups = (a.nslots + 31) / 32;
  const int GK = G * kTopK;
  const int pcap = a.pick_cap;
  const int rows_mine = k < nr ? (nr - k + G - 1) / G : 0;  // coverage rows this CTA owns
  for (int d = tid; d <= kSmallRecip; d += blockDim.x) s_rsmall[d] = div_recip(max(d, 1));
  if (tid == 0) {
    s_rG = div_recip(G);
    s_rnr = div_recip(nr);
    s_rpcap = div_recip(pcap);
    s_rrows = div_recip(max(rows_mine, 1));
    s_rnb2 = div_recip(nb2);
  }

  // shared-memory carve-up (sizes mirrored by site_smem_bytes)
  unsigned char *p = sm;
  auto take = [&](size_t bytes) {
    unsigned char *q = p;
    p += (bytes + 15) & ~(size_t)15;
    return q;
  };
  unsigned long long *s_gtop = reinterpret_cast<unsigned long long *>(take((size_t)ngroups * kTopK * 8));
  unsigned long long *s_mkey = reinterpret_cast<unsigned long long *>(take((size_t)GK * 8));
  unsigned long long *s_pkey = reinterpret_cast<unsigned long long *>(take(kMaxPicks * 8));
  int *s_gain = reinterpret_cast<int *>(take((size_t)a.nslots * 4));
  int *s_area = reinterpret_cast<int *>(take((size_t)a.nslots * 4));
  int *s_pos = reinterpret_cast<int *>(take((size_t)a.nslots * 4));
  int *s_dacc = reinterpret_cast<int *>(take((size_t)a.nslots * 4));
  int *s_mpos = reinterpret_cast<int *>(take((size_t)GK * 4));
  int *s_valid = reinterpret_cast<int *>(take((size_t)GK * 4));
  unsigned long long *s_vkey = reinterpret_cast<unsigned long long *>(take((size_t)GK * 8));
  int *s_vrank = reinterpret_cast<int *>(take((size_t)GK * 4));
  int *s_pk = reinterpret_cast<int *>(take(kMaxPicks * 4));    // pick: candidate index
  int *s_ppos = reinterpret_cast<int *>(take(kMaxPicks * 4));  // pick: cell
  int *s_pcnt = reinterpret_cast<int *>(take(kMaxPicks * 4));  // own candidates near the pick
  int *s_pairslot = reinterpret_cast<int *>(take((size_t)a.pair_cap * 4));  // [pick][pcap]
  int *s_plist = reinterpret_cast<int *>(take((size_t)a.pair_cap * 4));  // dense pair indices
  int *s_pairdelta = reinterpret_cast<int *>(take((size_t)a.pair_cap * 4));
  unsigned char *s_paircov = take((size_t)a.pair_cap);  // bit0 pick covers c, bit1 c covered before
  unsigned char *s_flag = take((size_t)a.nslots);
  unsigned char *s_tag = take((size_t)a.nslots);  // bit0 touched, bit1 covered (this round)
  unsigned char *s_dirty = take((size_t)ngroups);
  uint64_t *s_N = reinterpret_cast<uint64_t *>(take((size_t)a.ncap_words * 8));
  unsigned char *s_nmask = take(kMaskCap);

  GroupBarrier gb{a.bar, (unsigned)G, 0u};
  // tracing: device cycles per phase, accumulated by CTA 0's thread 0 in
  // shared memory (a register array would take registers in every thread)
  __shared__ long long s_ph[kSitePhases], s_tmark;
  if (tid == 0) {
    for (int i = 0; i < kSitePhases; i++) s_ph[i] = 0;
    s_tmark = clock64();
  }
  auto mark = [&](int i) {
    if (k == 0 && tid == 0) {
      const long long now = clock64();
      s_ph[i] += now - s_tmark;
      s_tmark = now;
    }
  };

  // ---- own candidates: round-1 gains from the scoring kernel ----------------
  for (int s = tid; s < a.nslots; s += blockDim.x) {
    const bool mine = s < my_slots;
    const int c = s * G + k;
    const int g = mine ? __ldcg(a.gains + c) : 0;
    s_gain[s] = g;
    s_area[s] = g;
    // cells as (row << 16 | column): rows and columns are below 2^16 (n^2 fits an int)
    const int cell = mine ? __ldg(a.obs + c) : 0;
    s_pos[s] = ((cell / n) << 16) | (cell % n);
    s_flag[s] = mine ? 0 : kUsed;
    s_dacc[s] = 0;
    s_tag[s] = 0;
  }
  for (int g = tid; g < ngroups; g += blockDim.x) s_dirty[g] = 1;
  if (tid == 0) {
    s_cum = 0;
    s_done = 0;
  }
  __syncthreads();
  mark(0);

  uint64_t *cum = a.cum0;
  int npicks = 0, rounds = 0, nprev = 0;
  const int lim2 = 4 * roi * roi;

  for (;;) {
    const int par = rounds & 1;
    // ---- A. per-group top-K of dirty groups; this CTA's top-K ----------------
    for (int g = warp; g < ngroups; g += nwarps) {
      if (!s_dirty[g]) continue;
      const int s = g * 32 + lane;
      unsigned long long key = 0;
      if (s < my_slots && !(s_flag[s] & kUsed)) key = make_key(s_area[s], s * G + k);
      for (int e = 0; e < kTopK; e++) {
        const unsigned long long mx = warp_max_key(key);
        if (lane == 0) s_gtop[g * kTopK + e] = mx;
        if (key == mx) key = 0;  // keys are unique (the index is part of them)
      }
      if (lane == 0) s_dirty[g] = 0;
    }
    __syncthreads();
    if (warp == 0) {
      unsigned long long *out = a.topk + ((size_t)par * G + k) * kTopK * 2;
      int h0 = 0, h1 = 0, h2 = 0, h3 = 0;  // heads of groups lane, lane+32, lane+64, lane+96
      for (int e = 0; e < kTopK; e++) {
        unsigned long long key = 0;
        int gi = -1;
#pragma unroll
        for (int q = 0; q < 4; q++) {
          const int g = lane + 32 * q;
          const int h = q == 0 ? h0 : q == 1 ? h1 : q == 2 ? h2 : h3;
          if (g < ngroups && h < kTopK) {
            const unsigned long long v = s_gtop[g * kTopK + h];
            if (v > key) {
              key = v;
              gi = g;
            }
          }
        }
        // keys are unique: the lane holding the largest advances that head
        const unsigned long long mine = key;
        key = warp_max_key(mine);
        if (key && mine == key) {
          const int q = gi >> 5;
          h0 += q == 0;
          h1 += q == 1;
          h2 += q == 2;
          h3 += q == 3;
        }
        if (lane == 0) {
          const int pos = key ? s_pos[key_index(key) / G] : 0;
          __stcg(out + 2 * e, key);
          __stcg(out + 2 * e + 1, (unsigned long long)pos);
        }
      }
    }
    mark(1);
    if (!group_sync(gb, a.err, &s_flagv)) return;
    mark(2);
    // ---- B. merge the published lists; accept the exact prefix --------------
#pragma unroll 2
    for (int i = tid; i < GK; i += blockDim.x) {
      const unsigned long long *src = a.topk + ((size_t)par * GK + i) * 2;
      s_mkey[i] = __ldcg(src);
      s_mpos[i] = (int)__ldcg(src + 1);
    }
    if (tid < kMaxPicks) s_pcnt[tid] = 0;
    if (tid == 0) s_nvalid = 0;
    __syncthreads();
    {  // exactness threshold: unpublished keys are below each full list's last key
      unsigned long long T = 0;
      if (tid < G) T = s_mkey[tid * kTopK + kTopK - 1];
      T = warp_max_key(T);
      if (lane == 0 && warp * 32 < G) s_red[warp] = T;
    }
    __syncthreads();
    {
      unsigned long long T = 0;
      for (int w = 0; w * 32 < G; w++) T = s_red[w] > T ? s_red[w] : T;
      // exactly ordered entries: keys >= T with a positive area
      auto valid_key = [&](unsigned long long key) {
        return key != 0 && (key >> 32) != 0 && key >= T;
      };
      for (int e0 = warp * 32; e0 < GK; e0 += blockDim.x) {  // one shared atomic a warp
        const int e = e0 + lane;
        const unsigned long long key = e < GK ? s_mkey[e] : 0ull;
        const bool ok = key != 0 && (key >> 32) != 0 && key >= T;
        const unsigned bal = __ballot_sync(0xffffffffu, ok);
        if (!bal) continue;
        int v0 = 0;
        if (lane == 0) v0 = atomicAdd(&s_nvalid, __popc(bal));
        v0 = __shfl_sync(0xffffffffu, v0, 0);
        if (ok) {
          const int v = v0 + __popc(bal & ((1u << lane) - 1u));
          s_valid[v] = e;  // GK entries fit
          s_vkey[v] = key;
          s_vrank[v] = 0;
        }
      }
    }
    __syncthreads();
    mark(9);
    const int nvalid = s_nvalid;
    {  // rank of each valid key: count larger valid keys, 32 at a time
      // lanes take consecutive keys against one chunk: the chunk's reads are
      // broadcasts, free of bank conflicts
      const int nch = (nvalid + 31) / 32;
      for (int i = tid; i < nvalid * nch; i += blockDim.x) {
        const int ch = i / nvalid, v = i - ch * nvalid, c0 = ch * 32;
        const unsigned long long key = s_vkey[v];
        const int c1 = min(c0 + 32, nvalid);
        int cnt = 0;
#pragma unroll 8
        for (int j = c0; j < c1; j++) cnt += s_vkey[j] > key;
        if (cnt) atomicAdd(&s_vrank[v], cnt);
      }
    }
    __syncthreads();
    for (int v = tid; v < nvalid; v += blockDim.x)
      if (s_vrank[v] < kMaxPicks) {
        s_rank[s_vrank[v]] = s_valid[v];
        s_rpos[s_vrank[v]] = s_mpos[s_valid[v]];
      }
    __syncthreads();
    mark(10);
    const int nrank = min(nvalid, kMaxPicks);
    if (warp == 0) {
      // prefix: leading ranks that are each > 2roi from every better-ranked
      // one, capped, up to the 95% stop.  Lane l holds ranks l and l+32.
      const int max_m = min(kMaxPicks, a.pair_cap / max(pcap, 1));
      const int lim = min(nrank, max_m);
      const int q0 = lane < lim ? s_rpos[lane] : 0;
      const int q1 = lane + 32 < lim ? s_rpos[lane + 32] : 0;
      const int a0 = lane < lim ? (int)(s_mkey[s_rank[lane]] >> 32) : 0;
      const int a1 = lane + 32 < lim ? (int)(s_mkey[s_rank[lane + 32]] >> 32) : 0;
      long long cumv = s_cum;
      int m = 0, stop_at = -1;
      for (int r = 0; r < lim; r++) {
        const int p1 = __shfl_sync(0xffffffffu, r < 32 ? q0 : q1, r & 31);
        const int area = __shfl_sync(0xffffffffu, r < 32 ? a0 : a1, r & 31);
        const int x1 = p1 >> 16, y1 = p1 & 0xffff;
        const int dx0 = (q0 >> 16) - x1, dy0 = (q0 & 0xffff) - y1;
        const int dx1 = (q1 >> 16) - x1, dy1 = (q1 & 0xffff) - y1;
        const bool near = (lane < r && dx0 * dx0 + dy0 * dy0 <= lim2) ||
                          (lane + 32 < r && dx1 * dx1 + dy1 * dy1 <= lim2);
        if (__any_sync(0xffffffffu, near)) break;
        cumv += area;
        m = r + 1;
        if (cumv >= a.stop_area) {
          stop_at = m;
          break;
        }
      }
      for (int j = lane; j < m; j += 32) {
        const int e = s_rank[j];
        const int c = key_index(s_mkey[e]);
        s_pk[j] = c;
        s_ppos[j] = s_mpos[e];
        s_pkey[j] = s_mkey[e];
        prefetch_l2(a.sheds + (size_t)c * per, per * 8);  // the pick's shed, for D1
        {  // the block rectangle of the neighbour search (FINDMAX geometry, +-2 blocks)
          const float r2f = (float)(2 * roi);
          const int pos = s_mpos[e];
          const int px = pos >> 16, py = pos & 0xffff;
          const int bxl = max(0, (int)floorf(((float)px - r2f) / a.bs) - 2);
          const int bxh = min(a.nb - 1, (int)floorf(((float)px + r2f) / a.bs) + 2);
          const int byl = max(0, (int)floorf(((float)py - r2f) / a.bs) - 2);
          const int byh = min(a.nb - 1, (int)floorf(((float)py + r2f) / a.bs) + 2);
          const int run = (byh - byl + 1) * a.npb;
          const int per_run = run / G + 2;
          s_pbox[j] = make_int4((bxl * a.nb + byl) * a.npb, run, per_run, (bxh - bxl + 1) * per_run);
          s_rrun[j] = per_run <= kSmallRecip ? s_rsmall[per_run] : div_recip(per_run);
        }
      }
      if (lane == 0) {
        s_m = m;
        s_stop_at = stop_at;
        s_rm = s_rsmall[max(m, 1)];  // m <= kMaxPicks <= kSmallRecip
      }
    }
    __syncthreads();
    mark(3);
    const int m = s_m;
    if (m == 0) break;  // the largest area is 0

    // Two ways to the picks' new bits N_p = placed(p) & ~cum.  Small rounds
    // (every pick row one thread's item) compute all rows of every pick in
    // shared memory in each CTA; larger rounds spread the rows over the CTAs
    // (rows k, k+G, ... of each pick), write them to a global buffer and read
    // them after one more barrier, so each row is computed once.  The choice
    // depends on m only, so all CTAs make it alike.
    const bool dist = m * nr > (int)blockDim.x || nwpr > 7 ||
                      m * nr * nb2 > a.ncap_words;
    // A large round also keeps this CTA's own new-bit rows in the (otherwise
    // unused) shared buffer, item i of the spread rows at words i*nb2..: the
    // coverage update ORs them (cum | placed = cum | (placed & ~cum)).
    const bool own_n = dist && m * rows_mine * nb2 <= a.ncap_words;
    // ---- D1 (spread): this CTA's rows of every pick, popcounts for the
    // self-check
    if (dist) {
      const unsigned long long rr = s_rrows;
      // taken from the last thread down, so that these rows overlap the
      // neighbour search below, whose items start at thread 0
      for (int i = blockDim.x - 1 - tid; i < m * rows_mine; i += blockDim.x) {
        const int pi = div_by(i, rr), prow = k + G * (i - pi * rows_mine);
        const int pp = s_ppos[pi];
        const int px = pp >> 16, py = pp & 0xffff;
        int fwp, fbp;
        shed_align(py - roi, fwp, fbp);
        const int gr = px - roi + prow;
        const bool row_in = gr >= 0 && gr < n;
        uint64_t *nrow = a.nbits + (size_t)(pi * nr + prow) * nb2;
        const uint64_t *prw = a.sheds + (size_t)s_pk[pi] * per + (size_t)prow * nwpr;
        int cnt = 0;
        if (nwpr <= 7) {  // all of the row's loads issued together
          const uint64_t *xr = cum + (size_t)(row_in ? gr : 0) * cw;
          uint64_t w[8], x[8];
#pragma unroll
          for (int q = 0; q < 8; q++) {
            w[q] = q < nwpr ? __ldg(prw + q) : 0ull;
            const int W = fwp + q;
            x[q] = (row_in && q < nb2 && W >= 0 && W < cw) ? __ldcg(xr + W) : ~0ull;
          }
          unsigned msk = 0;
#pragma unroll
          for (int q = 0; q < 8; q++) {
            if (q >= nb2) break;
            const uint64_t v =
                ((w[q] >> fbp) | ((q > 0 && fbp) ? w[q - 1] << (64 - fbp) : 0ull)) & ~x[q];
            __stcg(nrow + q, v);
            if (own_n) s_N[(size_t)i * nb2 + q] = v;
            cnt += __popcll(v);
            msk |= (v != 0ull) << q;
          }
          __stcg(a.nmask + pi * nr + prow, (unsigned char)msk);
        } else {
          for (int j = 0; j < nb2; j++) {
            const int W = fwp + j;
            uint64_t v = 0ull;
            if (row_in && W >= 0 && W < cw)
              v = placed_word(prw, j, nwpr, fbp) & ~__ldcg(cum + (size_t)gr * cw + W);
            __stcg(nrow + j, v);
            if (own_n) s_N[(size_t)i * nb2 + j] = v;
            cnt += __popcll(v);
          }
        }
        if (cnt) atomicAdd(a.ncount + par * kMaxPicks + pi, cnt);
      }
    }

    // ---- C. own unused candidates within 2*roi of each pick ------------------
    {
      const unsigned long long rm = s_rm, rG = s_rG;
      for (int i = tid; i < m * a.pick_items; i += blockDim.x) {
        const int it = div_by(i, rm), pi = i - it * m;
        const int4 box = s_pbox[pi];  // first start, run, per_run, items
        if (it >= box.w) continue;
        const int pos = s_ppos[pi];
        const int px = pos >> 16, py = pos & 0xffff;
        const int r = div_by(it, s_rrun[pi]), mm = it - r * box.z;
        const int start = box.x + r * a.nb * a.npb;
        int off = k - (start - div_by(start, rG) * G);  // first index owned by this CTA
        if (off < 0) off += G;
        const int c = start + off + mm * G;
        if (c >= start + box.y || c >= a.nsheds || c == s_pk[pi]) continue;
        const int s = div_by(c, rG);
        if (s_flag[s] & kUsed) continue;
        const int cp = s_pos[s];
        const int cx = cp >> 16, cy = cp & 0xffff;
        const int dx = cx - px, dy = cy - py;
        if (dx * dx + dy * dy > lim2) continue;
        const int idx = atomicAdd(&s_pcnt[pi], 1);
        if (idx < pcap) {
          const int pr = pi * pcap + idx;
          {  // rows of c's shed that overlap the pick's window, for the deltas
            const int r0 = max(0, px - cx), r1 = min(nr - 1, px - cx + 2 * roi);
            if (r1 >= r0)
              prefetch_l2(a.sheds + (size_t)c * per + (size_t)r0 * nwpr,
                          (size_t)(r1 - r0 + 1) * nwpr * 8);
          }
          s_pairslot[pr] = s;
          s_pairdelta[pr] = 0;
          unsigned char cv = 0;
          if (a.intervis)  // own cell already covered?
            cv = (unsigned char)(((__ldcg(cum + (size_t)cx * cw + (cy >> 6)) >> (63 - (cy & 63))) & 1ull)
                                 << 1);
          s_paircov[pr] = cv;
        } else {
          atomicOr(a.err, kErrCapacity);
        }
      }
    }
    __syncthreads();
    mark(4);

    // compact the pairs: offsets of each pick's pairs, then a dense index list
    if (warp == 0) {
      int run = 0;
      for (int base = 0; base < m; base += 32) {
        const int j = base + lane;
        int v = j < m ? min(s_pcnt[j], pcap) : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int w = __shfl_up_sync(0xffffffffu, v, o);
          if (lane >= o) v += w;
        }
        if (j < m) s_poff[j + 1] = run + v;
        run += __shfl_sync(0xffffffffu, v, 31);
      }
      if (lane == 0) {
        s_poff[0] = 0;
        s_npair = run;
      }
    }
    __syncthreads();
    for (int i = tid; i < m * pcap; i += blockDim.x) {
      const int j = div_by(i, s_rpcap), q = i - j * pcap;
      if (q < min(s_pcnt[j], pcap)) s_plist[s_poff[j] + q] = i;
    }
    __syncthreads();
    const int npair = s_npair;
    mark(5);

    if (!dist) {
      // ---- D1. new bits N = placed(p) & ~cum of each pick row, in shared
      // memory (picks with own candidates nearby, or rows of this CTA's
      // self-check); one item per row, all of its loads issued together
      for (int it = tid; it < m * nr; it += blockDim.x) {
        const int pi = it / nr, prow = it - pi * nr;
        const bool own_row = (prow % G) == k;
        if (s_pcnt[pi] == 0 && !own_row) continue;
        const int pp = s_ppos[pi];
        const int px = pp >> 16, py = pp & 0xffff;
        int fwp, fbp;
        shed_align(py - roi, fwp, fbp);
        const int gr = px - roi + prow;
        uint64_t *nrow = s_N + (size_t)it * nb2;
        if (gr < 0 || gr >= n) {
          for (int j = 0; j < nb2; j++) nrow[j] = 0ull;
          continue;
        }
        const uint64_t *prw = a.sheds + (size_t)s_pk[pi] * per + (size_t)prow * nwpr;
        const uint64_t *xr = cum + (size_t)gr * cw;
        uint64_t w[8], x[8];
#pragma unroll
        for (int q = 0; q < 8; q++) {
          w[q] = q < nwpr ? __ldg(prw + q) : 0ull;
          const int W = fwp + q;
          x[q] = (q < nb2 && W >= 0 && W < cw) ? __ldcg(xr + W) : ~0ull;
        }
        int cnt = 0;
#pragma unroll
        for (int q = 0; q < 8; q++) {
          if (q >= nb2) break;
          const uint64_t v = ((w[q] >> fbp) | ((q > 0 && fbp) ? w[q - 1] << (64 - fbp) : 0ull)) & ~x[q];
          nrow[q] = v;
          cnt += __popcll(v);
        }
        if (own_row && cnt) atomicAdd(a.ncount + par * kMaxPicks + pi, cnt);
      }
      __syncthreads();
      // ---- D2. per (pair, row): popcount(placed(c) & N) ----------------------
      for (int it = tid; it < npair * nr; it += blockDim.x) {
        const int u = div_by(it, s_rnr), r = it - u * nr;
        const int pr = s_plist[u];
        const int pi = div_by(pr, s_rpcap);
        const int s = s_pairslot[pr];
        const int cp = s_pos[s], pp = s_ppos[pi];
        const int cx = cp >> 16, cy = cp & 0xffff, px = pp >> 16, py = pp & 0xffff;
        const int gr = cx - roi + r, prow = gr - (px - roi);
        if (prow < 0 || prow >= nr || gr < 0 || gr >= n) continue;
        int fwc, fbc, fwp, fbp;
        shed_align(cy - roi, fwc, fbc);
        shed_align(py - roi, fwp, fbp);
        const uint64_t *nrow = s_N + (size_t)(pi * nr + prow) * nb2;
        if (a.intervis && r == roi) {  // own cell: newly covered by the pick?
          const int j = (cy >> 6) - fwp;
          if (j >= 0 && j < nb2 && ((nrow[j] >> (63 - (cy & 63))) & 1ull))
            atomicOr(reinterpret_cast<unsigned *>(s_paircov + (pr & ~3)), 1u << (8 * (pr & 3)));
        }
        const int lo = max(max(fwc, fwp), 0);
        const int hi = min(min((cy + roi) >> 6, fwp + nwpr), cw - 1);
        if (lo > hi) continue;
        // the pick's new bits under c's columns (shared memory) first: where
        // they are all zero the item loads nothing from c's shed
        uint64_t x[8], any = 0ull;
#pragma unroll
        for (int q = 0; q < 8; q++) {
          const int W = fwc + q;  // c's placed word q lands at column word fwc+q
          x[q] = (q < nb2 && W >= lo && W <= hi) ? nrow[W - fwp] : 0ull;
          any |= x[q];
        }
        if (!any) continue;
        const uint64_t *crow = a.sheds + (size_t)(s * G + k) * per + (size_t)r * nwpr;
        uint64_t w[8];
#pragma unroll
        for (int q = 0; q < 8; q++) w[q] = q < nwpr ? __ldg(crow + q) : 0ull;
        int d = 0;
#pragma unroll
        for (int q = 0; q < 8; q++) {
          if (q >= nb2) break;
          const uint64_t vc = (w[q] >> fbc) | ((q > 0 && fbc) ? w[q - 1] << (64 - fbc) : 0ull);
          d += __popcll(vc & x[q]);
        }
        if (d) atomicAdd(&s_pairdelta[pr], d);
      }
    } else {
    // every CTA's rows of N are written
    if (!group_sync(gb, a.err, &s_flagv)) return;
    mark(11);
    // the rows' nonzero-word masks into shared memory (a few hundred bytes):
    // an item whose candidate's columns meet only zero words of the pick's
    // new bits loads nothing (a third of the items at 4096²)
    const bool masked = nwpr <= 7 && m * nr <= kMaskCap;
    if (masked) {
      const int n16 = (m * nr + 15) / 16;
      const uint4 *src = reinterpret_cast<const uint4 *>(a.nmask);
      for (int i = tid; i < n16; i += blockDim.x)
        reinterpret_cast<uint4 *>(s_nmask)[i] = __ldcg(src + i);
      __syncthreads();
    }
    // bits j of the N words an item reads: columns lo..hi of the row
    auto need = [&](int pi, int prow, int lo, int hi, int fwp) -> unsigned {
      const unsigned span = ((1u << (hi - lo + 1)) - 1u) << (lo - fwp);
      return masked ? span & s_nmask[pi * nr + prow] : span;
    };
    if (kThreads == 512 && nwpr <= 4) {
      // ---- D2 for narrow sheds: two (pair, row) items a thread in flight
      // (512-thread CTAs only: the 1024-thread build has no registers for it).
      // Items past the end load nothing (pr < 0).
      // An item's loads: c's row (w) and the pick's new bits under it (x);
      // pr < 0 marks an item with nothing to count.
      auto load_item = [&](int it, uint64_t(&w)[4], uint64_t(&x)[5], int &pr, int &fbc) {
        pr = -1;
        if (it >= npair * nr) return;
        const int u = div_by(it, s_rnr), r = it - u * nr;
        const int pq = s_plist[u];
        const int pi = div_by(pq, s_rpcap);
        const int s = s_pairslot[pq];
        const int cp = s_pos[s], pp = s_ppos[pi];
        const int cx = cp >> 16, cy = cp & 0xffff, px = pp >> 16, py = pp & 0xffff;
        const int gr = cx - roi + r, prow = gr - (px - roi);
        if (prow < 0 || prow >= nr || gr < 0 || gr >= n) return;
        int fwc, fwp, fbp;
        shed_align(cy - roi, fwc, fbc);
        shed_align(py - roi, fwp, fbp);
        const uint64_t *nrow = a.nbits + (size_t)(pi * nr + prow) * nb2;
        const unsigned rowm = masked ? s_nmask[pi * nr + prow] : 0xffu;
        if (a.intervis && r == roi) {  // own cell: newly covered by the pick?
          const int j = (cy >> 6) - fwp;
          if (j >= 0 && j < nb2 && ((rowm >> j) & 1u) &&
              ((__ldcg(nrow + j) >> (63 - (cy & 63))) & 1ull))
            atomicOr(reinterpret_cast<unsigned *>(s_paircov + (pq & ~3)), 1u << (8 * (pq & 3)));
        }
        const int lo = max(max(fwc, fwp), 0);
        const int hi = min(min((cy + roi) >> 6, fwp + nwpr), cw - 1);
        if (lo > hi) return;
        const unsigned nm = need(pi, prow, lo, hi, fwp);
        if (!nm) return;  // the pick adds nothing under c's columns of this row
        const uint64_t *crow = a.sheds + (size_t)(s * G + k) * per + (size_t)r * nwpr;
#pragma unroll
        for (int q = 0; q < 4; q++) w[q] = q < nwpr ? __ldg(crow + q) : 0ull;
#pragma unroll
        for (int q = 0; q < 5; q++) {
          const int W = fwc + q;  // c's placed word q lands at column word fwc+q
          x[q] = (q < nb2 && W >= lo && W <= hi && ((nm >> (W - fwp)) & 1u))
                     ? __ldcg(nrow + (W - fwp)) : 0ull;
        }
        pr = pq;
      };
      auto count_item = [&](const uint64_t(&w)[4], const uint64_t(&x)[5], int pr, int fbc) {
        int d = 0;
#pragma unroll
        for (int q = 0; q < 5; q++) {
          const uint64_t cur = q < 4 ? w[q] : 0ull;
          const uint64_t vc = (cur >> fbc) | ((q > 0 && fbc) ? w[q - 1] << (64 - fbc) : 0ull);
          d += __popcll(vc & x[q]);
        }
        if (d) atomicAdd(&s_pairdelta[pr], d);
      };
      for (int it = tid; it < npair * nr; it += 2 * blockDim.x) {
        uint64_t w0[4], x0[5], w1[4], x1[5];
        int pr0, pr1, fb0 = 0, fb1 = 0;
        load_item(it, w0, x0, pr0, fb0);
        load_item(it + blockDim.x, w1, x1, pr1, fb1);
        if (pr0 >= 0) count_item(w0, x0, pr0, fb0);
        if (pr1 >= 0) count_item(w1, x1, pr1, fb1);
      }
    } else if (nwpr <= 7) {
      // ---- D2. per (pair, row): popcount(placed(c) & N), loads issued together
      for (int it = tid; it < npair * nr; it += blockDim.x) {
        const int u = div_by(it, s_rnr), r = it - u * nr;
        const int pr = s_plist[u];
        const int pi = div_by(pr, s_rpcap);
        const int s = s_pairslot[pr];
        const int cp = s_pos[s], pp = s_ppos[pi];
        const int cx = cp >> 16, cy = cp & 0xffff, px = pp >> 16, py = pp & 0xffff;
        const int gr = cx - roi + r, prow = gr - (px - roi);
        if (prow < 0 || prow >= nr || gr < 0 || gr >= n) continue;
        int fwc, fbc, fwp, fbp;
        shed_align(cy - roi, fwc, fbc);
        shed_align(py - roi, fwp, fbp);
        const uint64_t *nrow = a.nbits + (size_t)(pi * nr + prow) * nb2;
        const unsigned rowm = masked ? s_nmask[pi * nr + prow] : 0xffu;
        if (a.intervis && r == roi) {  // own cell: newly covered by the pick?
          const int j = (cy >> 6) - fwp;
          if (j >= 0 && j < nb2 && ((rowm >> j) & 1u) &&
              ((__ldcg(nrow + j) >> (63 - (cy & 63))) & 1ull))
            atomicOr(reinterpret_cast<unsigned *>(s_paircov + (pr & ~3)), 1u << (8 * (pr & 3)));
        }
        const int lo = max(max(fwc, fwp), 0);
        const int hi = min(min((cy + roi) >> 6, fwp + nwpr), cw - 1);
        if (lo > hi) continue;
        const unsigned nm = need(pi, prow, lo, hi, fwp);
        if (!nm) continue;  // the pick adds nothing under c's columns of this row
        const uint64_t *crow = a.sheds + (size_t)(s * G + k) * per + (size_t)r * nwpr;
        uint64_t w[8], x[8];
#pragma unroll
        for (int q = 0; q < 8; q++) {
          w[q] = q < nwpr ? __ldg(crow + q) : 0ull;
          const int W = fwc + q;  // c's placed word q lands at column word fwc+q
          x[q] = (q < nb2 && W >= lo && W <= hi && ((nm >> (W - fwp)) & 1u))
                     ? __ldcg(nrow + (W - fwp)) : 0ull;
        }
        int d = 0;
#pragma unroll
        for (int q = 0; q < 8; q++) {
          if (q >= nb2) break;
          const uint64_t vc = (w[q] >> fbc) | ((q > 0 && fbc) ? w[q - 1] << (64 - fbc) : 0ull);
          d += __popcll(vc & x[q]);
        }
        if (d) atomicAdd(&s_pairdelta[pr], d);
      }
    } else {
      // ---- D2 for wide sheds: per (pair, row, 4-word chunk)
      for (int i = tid; i < npair * nr * nch; i += blockDim.x) {
        const int u = i / (nr * nch), rem = i - u * nr * nch;
        const int pr = s_plist[u];
        const int pi = pr / pcap;
        const int r = rem / nch, ch = rem - r * nch;
        const int s = s_pairslot[pr];
        const int cp = s_pos[s], pp = s_ppos[pi];
        const int cx = cp >> 16, cy = cp & 0xffff, px = pp >> 16, py = pp & 0xffff;
        const int gr = cx - roi + r, prow = gr - (px - roi);
        if (prow < 0 || prow >= nr || gr < 0 || gr >= n) continue;
        int fwc, fbc, fwp, fbp;
        shed_align(cy - roi, fwc, fbc);
        shed_align(py - roi, fwp, fbp);
        const uint64_t *nrow = a.nbits + (size_t)(pi * nr + prow) * nb2;
        if (a.intervis && r == roi && ch == 0) {  // own cell: newly covered by the pick?
          const int j = (cy >> 6) - fwp;
          if (j >= 0 && j < nb2 && ((__ldcg(nrow + j) >> (63 - (cy & 63))) & 1ull))
            atomicOr(reinterpret_cast<unsigned *>(s_paircov + (pr & ~3)), 1u << (8 * (pr & 3)));
        }
        const int lwc = (cy + roi) >> 6;
        const int lo = max(max(fwc, fwp), 0), hi = min(min(lwc, fwp + nwpr), cw - 1);
        const int W0 = lo + 4 * ch;
        if (W0 > hi) continue;
        const uint64_t *crow = a.sheds + (size_t)(s * G + k) * per + (size_t)r * nwpr;
        uint64_t cwd[5], xw[4];
#pragma unroll
        for (int t = 0; t < 5; t++) {
          const int jc = W0 - fwc - 1 + t;
          cwd[t] = (jc >= 0 && jc < nwpr) ? __ldg(crow + jc) : 0ull;
        }
#pragma unroll
        for (int t = 0; t < 4; t++) xw[t] = (W0 + t <= hi) ? __ldcg(nrow + (W0 + t - fwp)) : 0ull;
        int d = 0;
#pragma unroll
        for (int t = 0; t < 4; t++) {
          const uint64_t vc = (cwd[t + 1] >> fbc) | (fbc ? cwd[t] << (64 - fbc) : 0ull);
          d += __popcll(vc & xw[t]);
        }
        if (d) atomicAdd(&s_pairdelta[pr], d);
      }
    }
    }
    __syncthreads();
    mark(6);

    // ---- E. intervis: where would a newly covered candidate overtake? --------
    if (tid == 0) s_roundcut = m;
    __syncthreads();
    if (a.intervis) {
      for (int u = tid; u < npair; u += blockDim.x) {
        const int i = s_plist[u];
        const int j = div_by(i, s_rpcap);
        const int s = s_pairslot[i];
        if (!(s_flag[s] & kInel) || !(s_paircov[i] & 1)) continue;
        const int c = s * G + k;
        // this candidate's deltas by pick: it is within 2roi of few picks, which
        // are > 2roi apart; more than 8 falls back to cutting at the first
        // position it could matter, which is always safe
        int dpick0 = -1, dpick1 = -1, dpick2 = -1, dpick3 = -1, dpick4 = -1, dpick5 = -1;
        int dval0 = 0, dval1 = 0, dval2 = 0, dval3 = 0, dval4 = 0, dval5 = 0, nd = 0;
        bool many = false;
        for (int j2 = 0; j2 < m; j2++) {
          const int cnt2 = min(s_pcnt[j2], pcap);
          for (int q2 = 0; q2 < cnt2; q2++)
            if (s_pairslot[j2 * pcap + q2] == s) {
              const int dv = s_pairdelta[j2 * pcap + q2];
              switch (nd) {
                case 0: dpick0 = j2; dval0 = dv; break;
                case 1: dpick1 = j2; dval1 = dv; break;
                case 2: dpick2 = j2; dval2 = dv; break;
                case 3: dpick3 = j2; dval3 = dv; break;
                case 4: dpick4 = j2; dval4 = dv; break;
                case 5: dpick5 = j2; dval5 = dv; break;
                default: many = true;
              }
              nd++;
            }
        }
        int cut = m;
        if (many) {
          cut = j + 1;
        } else {
          for (int qq = j + 1; qq < m; qq++) {  // gain after picks 0..qq-1
            int g = s_gain[s];
            g -= (dpick0 >= 0 && dpick0 < qq) ? dval0 : 0;
            g -= (dpick1 >= 0 && dpick1 < qq) ? dval1 : 0;
            g -= (dpick2 >= 0 && dpick2 < qq) ? dval2 : 0;
            g -= (dpick3 >= 0 && dpick3 < qq) ? dval3 : 0;
            g -= (dpick4 >= 0 && dpick4 < qq) ? dval4 : 0;
            g -= (dpick5 >= 0 && dpick5 < qq) ? dval5 : 0;
            if (make_key(g, c) > s_pkey[qq]) {
              cut = qq;
              break;
            }
          }
        }
        if (cut < m) atomicMin(&s_roundcut, cut);
      }
      __syncthreads();
      if (tid == 0) __stcg(a.cuts + par * G + k, s_roundcut);
    }
    mark(12);
    // every read of the coverage this round is done once all CTAs pass here.
    // Without intervis there is no cut to agree on, and in a spread round the
    // coverage is read only before the spread barrier: the coverage update
    // may start at once.  (The buffers reused by the next round are written
    // only after its first barrier, which every CTA reaches after this one.)
    if ((a.intervis || !dist) && !group_sync(gb, a.err, &s_flagv)) return;
    if (tid == 0) s_mcut = m;
    __syncthreads();
    if (a.intervis) {  // the smallest cut of any CTA: one load per thread
      int c = tid < G ? __ldcg(a.cuts + par * G + tid) : m;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) c = min(c, __shfl_xor_sync(0xffffffffu, c, o));
      if (lane == 0 && c < m) atomicMin(&s_mcut, c);
    }
    __syncthreads();
    const int mcut = s_mcut;
    mark(7);

    // ---- F. apply picks 0..mcut-1 -------------------------------------------
    if (k == 0 && tid >= blockDim.x - kMaxPicks) {  // self-check this round, then reset
      const int i = tid - (blockDim.x - kMaxPicks);
      int *nc = a.ncount + par * kMaxPicks;
      if (i < mcut && __ldcg(nc + i) != (int)(s_pkey[i] >> 32)) atomicOr(a.err, kErrSiteMismatch);
      if (i < m) __stcg(nc + i, 0);
    }
    for (int i = tid; i < mcut; i += blockDim.x) {
      const int c = s_pk[i];
      const int cs = div_by(c, s_rG);
      if (c - cs * G == k) {
        const int s = cs;
        s_flag[s] |= kUsed;
        s_dirty[s >> 5] = 1;
        a.selected[c] = 1;
      }
      if (k == 0) a.order[npicks + i] = c;
    }
    for (int u = tid; u < npair; u += blockDim.x) {
      const int i = s_plist[u];
      if (div_by(i, s_rpcap) >= mcut) continue;
      const int s = s_pairslot[i];
      atomicAdd(&s_dacc[s], s_pairdelta[i]);
      const unsigned char cv = s_paircov[i];
      atomicOr(reinterpret_cast<unsigned *>(s_tag + (s & ~3)),
               (1u | ((cv & 1) ? 2u : 0u) | ((cv & 2) ? 4u : 0u)) << (8 * (s & 3)));
    }
    // coverage: OR this CTA's rows of the accepted picks' placed sheds
    {
      const unsigned long long rrb = s_rrows, rnb = s_rnb2;
      for (int i = tid; i < mcut * rows_mine * nb2; i += blockDim.x) {
        const int q = div_by(i, rnb), j = i - q * nb2;  // q = pick*rows_mine + own row
        const int pi = div_by(q, rrb), prow = k + G * (q - pi * rows_mine);
        const int pos = s_ppos[pi];
        const int px = pos >> 16, py = pos & 0xffff;
        int fwp, fbp;
        shed_align(py - roi, fwp, fbp);
        const int gr = px - roi + prow, W = fwp + j;
        if (gr < 0 || gr >= n || W < 0 || W >= cw) continue;
        // the pick's new bits where this CTA holds them, else its placed shed
        const uint64_t v =
            own_n ? s_N[i]
            : !dist ? s_N[(size_t)(pi * nr + prow) * nb2 + j]
                    : placed_word(a.sheds + (size_t)s_pk[pi] * per + (size_t)prow * nwpr, j, nwpr, fbp);
        if (v) atomicOr(reinterpret_cast<unsigned long long *>(cum + (size_t)gr * cw + W), v);
      }
    }
    __syncthreads();
    for (int u = tid; u < npair; u += blockDim.x) {
      const int i = s_plist[u];
      if (div_by(i, s_rpcap) >= mcut) continue;
      const int s = s_pairslot[i];
      const unsigned char tag = s_tag[s];
      if (!(tag & 1)) continue;  // already applied through another pair
      if (atomicAnd(reinterpret_cast<unsigned *>(s_tag + (s & ~3)), ~(0xFFu << (8 * (s & 3)))) &
          (1u << (8 * (s & 3)))) {
        // first pair of this candidate: apply its summed delta once
        const int g = s_gain[s] - s_dacc[s];
        s_gain[s] = g;
        s_dacc[s] = 0;
        const bool inel = a.intervis && !(tag & 6);
        s_area[s] = inel ? 0 : g;
        s_flag[s] = (unsigned char)((s_flag[s] & ~kInel) | (inel ? kInel : 0));
        s_dirty[s >> 5] = 1;
      }
    }
    if (tid == 0) {
      long long cadd = 0;
      for (int i = 0; i < mcut; i++) cadd += (long long)(s_pkey[i] >> 32);
      s_cum += cadd;
      s_done = (s_stop_at > 0 && s_stop_at <= mcut) ? 1 : 0;
    }
    __syncthreads();
    mark(8);
    npicks += mcut;
    nprev = mcut;
    rounds++;
    if (s_done) break;
  }

  if (k == 0 && tid == 0) {
    a.out[0] = npicks;
    a.out[1] = s_cum;
    a.out[2] = rounds;
    for (int i = 0; i < kSitePhases; i++) a.out[3 + i] = s_ph[i];
  }
}

// Bounds of the neighbour search around one pick: the block rectangle
// spans at most ceil((4roi+1)/bs)+6 block rows and columns (the kernel's +-2
// margins), and a CTA owns every G-th index of each contiguous block-row run.
struct PickBounds {
  int items;  // enumeration items per pick
  int cap;    // own candidates near one pick
};

PickBounds site_pick_bounds(int roi, int nsheds, int G, int nb, int npb, float bs) {
  const int span = (int)std::ceil((4.0 * roi + 1.0) / bs) + 6;
  const int nbx = std::min(nb, span);
  const long long run = (long long)std::min(nb, span) * npb;
  const long long items = (long long)nbx * (run / G + 2);
  PickBounds b;
  b.items = (int)std::min<long long>(items, 1 << 30);
  b.cap = (int)std::max<long long>(1, std::min<long long>(items, (nsheds + G - 1) / G));
  return b;
}

int site_pair_cap(const PickBounds &b) {
  return (int)std::min<long long>(kMaxPairs, (long long)b.cap * kMaxPicks);
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

namespace {

size_t scratch_layout(int nrows, int nsheds, int nctas, int roi, unsigned char *base,
                      SiteScratch *s) {
  const size_t cw = (size_t)(nrows + 63) / 64;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    unsigned char *q = base ? base + off : nullptr;
    off += (bytes + 255) & ~(size_t)255;
    return q;
  };
  // zeroed before a launch: everything up to `order`
  unsigned char *c0 = take((size_t)nrows * cw * 8);
  unsigned char *tk = take((size_t)2 * nctas * kTopK * 2 * 8);
  unsigned char *cu = take((size_t)2 * nctas * 4);
  unsigned char *nc = take((size_t)2 * kMaxPicks * 4);
  unsigned char *br = take(64);
  unsigned char *ou = take(128);
  unsigned char *od = take((size_t)nsheds * 4);
  unsigned char *gn = take((size_t)nsheds * 4);
  const size_t nr = 2 * (size_t)roi + 1;  // every row is written before it is read
  unsigned char *nb = take((size_t)kMaxPicks * nr * ((nr + 63) / 64 + 1) * 8);
  unsigned char *nm = take((size_t)kMaxPicks * nr + 16);  // + the 16-byte loads' tail
  unsigned char *tb = take(site_job_table_bytes(1, nctas));
  if (s) {
    s->cum = reinterpret_cast<uint64_t *>(c0);
    s->nbits = reinterpret_cast<uint64_t *>(nb);
    s->nmask = nm;
    s->topk = reinterpret_cast<unsigned long long *>(tk);
    s->cuts = reinterpret_cast<int *>(cu);
    s->ncount = reinterpret_cast<int *>(nc);
    s->bar = reinterpret_cast<unsigned *>(br);
    s->out = reinterpret_cast<long long *>(ou);
    s->order = reinterpret_cast<int32_t *>(od);
    s->gains = reinterpret_cast<int32_t *>(gn);
    s->table = tb;
  }
  return off;
}

size_t round16(size_t b) { return (b + 15) & ~(size_t)15; }

}  // namespace

size_t site_scratch_bytes(int nrows, int nsheds, int nctas, int roi) {
  return scratch_layout(nrows, nsheds, nctas, roi, nullptr, nullptr);
}

void site_carve_scratch(void *base, int nrows, int nsheds, int nctas, int roi, SiteScratch *s) {
  scratch_layout(nrows, nsheds, nctas, roi, static_cast<unsigned char *>(base), s);
}

// Up to one CTA per SM, about 100 candidates per CTA but at least 32 CTAs:
// each round's work is spread widely, while mid-size jobs keep fewer CTAs in
// their barriers (1000^2, 10 000 candidates: 1.79 ms at 96-100 CTAs against
// 1.99 ms at 152; 256^2, 512 candidates: 0.34 ms at 32 CTAs, 0.43 ms at 5).
// The merged top-K lists (G * kTopK keys) stay small enough to walk with one
// warp.
int site_default_ctas(int nsheds, int sm_count) {
  int g = std::max(1, std::min(std::max(std::min(32, nsheds), nsheds / 100), sm_count));
  g = std::max(g, (nsheds + kMaxSlots - 1) / kMaxSlots);
  return std::min(g, std::min(sm_count, 160));
}

// Candidate c belongs to CTA c % G, and candidates are numbered block-major
// ((block row * nb + block column) * npb + k), so a pick's neighbour search
// (span block rows of span*npb consecutive indices, the FINDMAX geometry) lands
// on CTAs (r * nb * npb + w) % G.  When nb*npb shares a large factor with G
// the rows fall on the same few CTAs (1000^2, nb = 100: at G = 100 every CTA
// owns one block column, and a round's pairs sit on ~27 of the 100 CTAs).
// Among G within a quarter of the default, take the one whose busiest CTA owns
// the fewest indices of such a rectangle, the nearest to the default on ties.
int site_spread_ctas(int G0, int roi, int nsheds, int nb, int npb, float bs, int sm_count) {
  if (nb <= 1) return G0;  // candidates in one run (no block geometry): nothing to spread
  const int span = std::min(nb, (int)std::ceil((4.0 * roi + 1.0) / bs) + 6);
  const long long stride = (long long)nb * npb, W = (long long)span * npb;
  const int lo = std::max({1, (G0 * 3) / 4, (nsheds + kMaxSlots - 1) / kMaxSlots});
  const int hi = std::min({sm_count, 160, (G0 * 5) / 4});
  auto busiest = [&](int G) {
    std::vector<int> diff(G + 1, 0);
    long long all = 0;
    for (int r = 0; r < span; r++) {  // row r covers W consecutive residues from r*stride
      const int start = (int)((r * stride) % G);
      all += W / G;
      const int rem = (int)(W % G);
      if (rem == 0) continue;
      diff[start]++;
      if (start + rem <= G) {
        diff[start + rem]--;
      } else {
        diff[G]--;
        diff[0]++;
        diff[start + rem - G]--;
      }
    }
    int run = 0, mx = 0;
    for (int g = 0; g < G; g++) mx = std::max(mx, run += diff[g]);
    return all + mx;
  };
  int best = G0;
  long long bw = G0 >= lo && G0 <= hi ? busiest(G0) : (long long)1 << 62;
  for (int G = lo; G <= hi; G++) {
    const long long w = busiest(G);
    if (w < bw || (w == bw && std::abs(G - G0) < std::abs(best - G0))) {
      bw = w;
      best = G;
    }
  }
  return best;
}

namespace {

// Shared memory of everything but the new-bits buffer.
size_t site_smem_base(int roi, int nsheds, int nctas, int nblocks, int npb, float blocksize) {
  const int nslots = (nsheds + nctas - 1) / nctas;
  const int ngroups = (nslots + 31) / 32;
  const int GK = nctas * kTopK;
  const PickBounds pb = site_pick_bounds(roi, nsheds, nctas, nblocks, npb, blocksize);
  const int pair_cap = site_pair_cap(pb);
  size_t b = 0;
  b += round16((size_t)ngroups * kTopK * 8) + round16((size_t)GK * 8) + round16(kMaxPicks * 8);
  b += 4 * round16((size_t)nslots * 4);
  b += 3 * round16((size_t)GK * 4) + round16((size_t)GK * 8) + 3 * round16(kMaxPicks * 4);
  b += 3 * round16((size_t)pair_cap * 4) + round16((size_t)pair_cap);
  b += 2 * round16((size_t)nslots) + round16((size_t)ngroups);
  b += kMaskCap;
  return b;
}

}  // namespace

// Shared words for the new bits of a small round (the spread path takes the
// rest): up to 32 KB, within the 220 KB plan.
constexpr size_t kSiteSmemPlan = 220 * 1024;
constexpr int kMaxNWords = 4096;

int site_ncap_words(size_t base) {
  if (base >= kSiteSmemPlan) return 0;
  return (int)std::min<size_t>(kMaxNWords, (kSiteSmemPlan - base) / 8 / 2 * 2);
}

size_t site_smem_bytes(int roi, int nsheds, int nctas, int nblocks, int npb, float blocksize) {
  const size_t base = site_smem_base(roi, nsheds, nctas, nblocks, npb, blocksize);
  return base + round16((size_t)site_ncap_words(base) * 8);
}

bool site_supported(int roi, int nsheds, int nctas) {
  const int nslots = (nsheds + nctas - 1) / nctas;
  return nslots <= kMaxSlots && nctas <= 160 && roi <= 2000;
}

namespace {

SiteArgs make_site_args(const SiteJob &j, int block0) {
  SiteArgs a{};
  a.n = j.nrows;
  a.roi = j.roi;
  a.intervis = j.intervis;
  a.nsheds = j.nsheds;
  a.G = j.nctas;
  a.obs = j.obs;
  a.sheds = j.sheds;
  a.bs = j.blocksize;
  a.nb = j.nblocks;
  a.npb = j.npb;
  a.cum0 = j.scratch.cum;
  a.nbits = j.scratch.nbits;
  a.nmask = j.scratch.nmask;
  a.ncap_words =
      site_ncap_words(site_smem_base(j.roi, j.nsheds, j.nctas, j.nblocks, j.npb, j.blocksize));
  a.topk = j.scratch.topk;
  a.cuts = j.scratch.cuts;
  a.ncount = j.scratch.ncount;
  a.bar = j.scratch.bar;
  a.out = j.scratch.out;
  a.order = j.scratch.order;
  a.selected = j.selected;
  a.gains = j.scratch.gains;
  a.err = j.err;
  a.nslots = (j.nsheds + j.nctas - 1) / j.nctas;
  const PickBounds pb = site_pick_bounds(j.roi, j.nsheds, j.nctas, j.nblocks, j.npb, j.blocksize);
  a.pick_items = pb.items;
  a.pick_cap = pb.cap;
  a.pair_cap = site_pair_cap(pb);
  a.stop_area = site_stop_area(j.nrows);
  a.block0 = block0;
  return a;
}

}  // namespace

size_t site_job_table_bytes(int njobs, int total_ctas) {
  return (((size_t)njobs * sizeof(SiteArgs) + 255) & ~(size_t)255) + (size_t)total_ctas * 4;
}

cudaError_t launch_site_jobs(const SiteJob *jobs, int njobs, void *d_table, void *h_stage,
                             cudaStream_t st) {
  int total = 0;
  size_t shm = 0;
  std::vector<SiteArgs> args(njobs);
  std::vector<int> block_job;
  for (int i = 0; i < njobs; i++) {
    args[i] = make_site_args(jobs[i], total);
    for (int b = 0; b < jobs[i].nctas; b++) block_job.push_back(i);
    total += jobs[i].nctas;
    shm = std::max(shm, site_smem_bytes(jobs[i].roi, jobs[i].nsheds, jobs[i].nctas,
                                        jobs[i].nblocks, jobs[i].npb, jobs[i].blocksize));
  }
  if (total == 0) return cudaSuccess;
  // job table: arguments, then the CTA -> job map
  const size_t tbytes = site_job_table_bytes(njobs, total);
  std::vector<unsigned char> pageable;
  unsigned char *host = static_cast<unsigned char *>(h_stage);
  if (!host) {
    pageable.resize(tbytes);
    host = pageable.data();
  }
  const size_t off = ((size_t)njobs * sizeof(SiteArgs) + 255) & ~(size_t)255;
  memcpy(host, args.data(), (size_t)njobs * sizeof(SiteArgs));
  memcpy(host + off, block_job.data(), (size_t)total * 4);
  cudaError_t e = cudaMemcpyAsync(d_table, host, tbytes, cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return e;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  // The scoring and the selection run at the device's highest priority,
  // carried by each launch so that a CUDA graph captured from the stream
  // keeps it: the block scheduler then gives them SMs as the CTAs of
  // concurrent stage kernels end.
  int least = 0, greatest = 0;
  e = cudaDeviceGetStreamPriorityRange(&least, &greatest);
  if (e != cudaSuccess) return e;
  cudaLaunchAttribute prio;
  prio.id = cudaLaunchAttributePriority;
  prio.val.priority = greatest;
  for (int i = 0; i < njobs; i++) {  // round-1 gains of every job
    const SiteJob &j = jobs[i];
    if (j.nsheds <= 0) continue;
    const int nr = 2 * j.roi + 1, per = nr * ((nr + 63) / 64);
    const int sgrid = std::max(1, std::min(sms * 8, (j.nsheds + 7) / 8));
    cudaLaunchConfig_t sc = {};
    sc.gridDim = dim3(sgrid);
    sc.blockDim = dim3(256);
    sc.stream = st;
    sc.attrs = &prio;
    sc.numAttrs = 1;
    e = cudaLaunchKernelEx(&sc, site_score_kernel, j.sheds, j.nsheds, per, j.scratch.gains);
    if (e != cudaSuccess) return e;
  }
  int threads = 512;
  for (int i = 0; i < njobs; i++)
    threads = std::max(threads, site_threads_for((jobs[i].nsheds + jobs[i].nctas - 1) /
                                                     std::max(1, jobs[i].nctas),
                                                 jobs[i].roi));
  const void *kern = threads == 1024 ? (const void *)site_kernel<1024> : (const void *)site_kernel<512>;
  e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm);
  if (e != cudaSuccess) return e;
  const SiteArgs *d_args = static_cast<const SiteArgs *>(d_table);
  const int *d_map = reinterpret_cast<const int *>(static_cast<unsigned char *>(d_table) + off);
  void *kargs[] = {&d_args, &d_map};
  // cooperative: its CTAs wait for one another at group barriers, so all
  // must be resident
  cudaLaunchAttribute attr[2];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  attr[1].id = cudaLaunchAttributePriority;
  attr[1].val.priority = greatest;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(total);
  cfg.blockDim = dim3(threads);
  cfg.dynamicSmemBytes = shm;
  cfg.stream = st;
  cfg.attrs = attr;
  cfg.numAttrs = 2;
  return cudaLaunchKernelExC(&cfg, kern, kargs);
}

cudaError_t launch_site(int nrows, int roi, int intervis, int nsheds, const int32_t *obs,
                        const uint64_t *sheds, float blocksize, int nblocks, int npb,
                        uint8_t *selected, const SiteScratch &s, int nctas, int *d_err,
                        cudaStream_t st) {
  SiteJob j{nrows, roi, intervis, nsheds, obs, sheds, blocksize, nblocks, npb, selected, s, nctas,
            d_err};
  return launch_site_jobs(&j, 1, s.table, nullptr, st);
}

}  // namespace siting

// ---- allocation-free SITE entry point --------------------------------------
//
// Some callers cannot allocate device memory on their call path: a serving
// loop that reserves its HBM budget at start-up and allows no allocation
// afterwards, or a host application whose memory pool (for example PyTorch's
// caching allocator) already owns the device's memory.  For them,
// siting_site_it_noalloc runs SITE with its scratch (coverage bitmap, CTA key
// lists, barrier, pick order, round-1 gains, error flag) carved from this
// file-scope device array instead of cudaMalloc'd workspace.  Every GPU that
// loads the library holds the array until the process exits.
//
// The array is shared by every call on a device and keeps the last call's
// contents: each call clears what must start at zero.  Calls whose work
// overlaps on the GPU (different streams, or different host threads) race on
// it and must be serialised by the caller.
namespace {

constexpr size_t kNoAllocScratchBytes = size_t(16) << 20;  // 16 MiB per device

}  // namespace

static __device__ __align__(256) unsigned char g_site_noalloc_scratch[kNoAllocScratchBytes];

namespace {

// Device address of the scratch array on the current device (host code only
// sees a host-side stand-in for the symbol).  Looked up on every call, with
// that device current, so that a context torn down and created again (for
// example after cudaDeviceReset) never leaves a stale address behind; the
// lookup costs microseconds against a SITE run.
int noalloc_scratch(void **out) {
  void *p = nullptr;
  if (cudaGetSymbolAddress(&p, g_site_noalloc_scratch) != cudaSuccess || !p) {
    cudaGetLastError();
    return SITING_ECUDA;
  }
  *out = p;
  return SITING_OK;
}

}  // namespace

extern "C" int siting_site_it_noalloc(int nrows, int roi, int intervis, int nsheds,
                                      const int32_t *d_obs, const uint64_t *d_sheds,
                                      uint8_t *d_selected, void *stream, siting_result *res) {
  using namespace siting;
  if (nrows <= 0 || nrows > 20000 || roi < 1 || (intervis != 0 && intervis != 1) || nsheds < 0 ||
      (nsheds && (!d_obs || !d_sheds || !d_selected)))
    return SITING_EINVAL;
  if (res) {
    res->nusedsheds = 0;
    res->cumarea = 0;
    res->coverage = 0.0;
    res->site_rounds = 0;
  }
  if (nsheds == 0) return SITING_OK;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) return SITING_EDEVICE;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return SITING_EDEVICE;
  const int G = site_default_ctas(nsheds, sms);
  if (!site_supported(roi, nsheds, G)) return SITING_EINVAL;
  // candidates are taken in any order: one block row holding them all
  const float bs = (float)nrows;
  if (site_smem_bytes(roi, nsheds, G, 1, nsheds, bs) > 220 * 1024) return SITING_EINVAL;
  const size_t need = site_scratch_bytes(nrows, nsheds, G, roi) + 256;  // + error flag
  if (need > kNoAllocScratchBytes) return SITING_ENOMEM;  // beyond the 16 MiB array
  void *base = nullptr;
  int rc = noalloc_scratch(&base);
  if (rc) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  SiteScratch s;
  site_carve_scratch(base, nrows, nsheds, G, roi, &s);
  int *d_err = reinterpret_cast<int *>(static_cast<unsigned char *>(base) + need - 256);
  // zero coverage, key lists, cuts, self-check counters, barrier and outputs
  if (cudaMemsetAsync(base, 0, (unsigned char *)s.order - (unsigned char *)base, st) != cudaSuccess ||
      cudaMemsetAsync(d_err, 0, sizeof(int), st) != cudaSuccess ||
      cudaMemsetAsync(d_selected, 0, nsheds, st) != cudaSuccess)
    return SITING_ECUDA;
  // the observer indices are checked before SITE reads any cell through them:
  // a bad index returns SITING_EINVAL with no SITE launch
  int herr = 0;
  if (launch_check_obs(d_obs, nsheds, nrows, d_err, st) != cudaSuccess ||
      cudaMemcpyAsync(&herr, d_err, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return SITING_ECUDA;
  if (herr & kErrBadInput) return SITING_EINVAL;
  if (herr) return SITING_ECUDA;
  if (launch_site(nrows, roi, intervis, nsheds, d_obs, d_sheds, bs, 1, nsheds, d_selected, s, G,
                  d_err, st) != cudaSuccess)
    return SITING_ECUDA;
  long long out[3] = {0, 0, 0};
  if (cudaMemcpyAsync(out, s.out, sizeof(out), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaMemcpyAsync(&herr, d_err, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return SITING_ECUDA;
  if (herr & kErrBadInput) return SITING_EINVAL;
  if (herr & (kErrTmaTimeout | kErrBarrierTimeout)) return SITING_ETIMEOUT;
  if (herr) return SITING_ECUDA;
  if (res) {
    res->nusedsheds = (int)out[0];
    res->cumarea = out[1];
    res->coverage = 100.0 * out[1] / ((double)nrows * nrows);
    res->site_rounds = (int)out[2];
  }
  return SITING_OK;
}
