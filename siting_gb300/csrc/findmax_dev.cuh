// FINDMAX of one block by one warp (siting.cpp:204-241), shared by the
// one-job FINDMAX kernel and the multi-job one of the batched form.
//
// Block (bx,by) spans rows [(int)(bs*bx), min((int)(bs*(bx+1)), n)) and the
// same for columns.  Each round picks the block cell with the largest
// (vix, h), h = x*(x+y)*010101010101 wrapping in int32; among equal (vix, h)
// the first cell of the row-major scan wins.  The winner goes to
// obs[block*npb + round] and its vix is cleared, so a later round can pick a
// cleared cell again once every cell is zero.  Each lane folds its strided
// subset of the block into one 64-bit key (vix:8 | h^0x80000000:32 |
// 0xFFFFFF-j:24, j < 3000^2 < 2^24 is the row-major position), so an unsigned
// max over the warp (shuffles) gives exactly the reference's winner and
// tie-break.
#pragma once

#include "common.cuh"

namespace siting {

__device__ __forceinline__ unsigned long long warp_max_u64(unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
    v = w > v ? w : v;
  }
  return v;
}

// Row (or column) range [x0, x1) of block index bx.
__device__ __forceinline__ void block_range(float bs, int bx, int n, int *x0, int *x1) {
  *x0 = f2i(fmul(bs, i2f(bx)));
  *x1 = min(f2i(fmul(bs, i2f(bx + 1))), n);
}

__device__ __forceinline__ void findmax_block(uint8_t *vix, int n, float bs, int nb, int npb,
                                              int32_t *obs, int b, int lane) {
  const int bx = b / nb, by = b - (b / nb) * nb;
  int x0, x1, y0, y1;
  block_range(bs, bx, n, &x0, &x1);
  block_range(bs, by, n, &y0, &y1);
  const int w = y1 - y0, npts = (x1 - x0) * w;
  for (int k = 0; k < npb; k++) {
    unsigned long long best = 0;
    // walk j = lane, lane+32, ... keeping (row, col) incrementally
    int r = lane / max(w, 1), c = lane - r * w;
    for (int j = lane; j < npts; j += 32) {
      const int x = x0 + r, y = y0 + c;
      const unsigned v = vix[x * n + y];
      const unsigned h = (unsigned)x * (unsigned)(x + y) * 0x41041041u;
      const unsigned long long key = ((unsigned long long)v << 56) |
                                     ((unsigned long long)(h ^ 0x80000000u) << 24) |
                                     (unsigned long long)(0xFFFFFF - j);
      best = key > best ? key : best;
      c += 32;
      while (c >= w) {
        c -= w;
        r++;
      }
    }
    best = warp_max_u64(best);
    // an empty block keeps the scan's starting cell (xmin, ymin), as the
    // reference's loop does when it never runs
    const int j = npts > 0 ? 0xFFFFFF - (int)(best & 0xFFFFFFull) : 0;
    const int x = npts > 0 ? x0 + j / w : x0, y = npts > 0 ? y0 + j % w : y0;
    if (lane == 0) {
      obs[(size_t)b * npb + k] = x * n + y;
      if (x < n && y < n) vix[x * n + y] = 0;
    }
    __syncwarp();
  }
}

}  // namespace siting
