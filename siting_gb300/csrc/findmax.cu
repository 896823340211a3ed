// FINDMAX: tentative observers, nwantedperblock per block
// (siting.cpp:204-241).
//
// Block (bx,by) spans rows [(int)(bs*bx), min((int)(bs*(bx+1)), n)) and the
// same for columns.  Each round picks the block cell with the largest
// (vix, h), h = x*(x+y)*010101010101 wrapping in int32; among equal (vix, h)
// the first cell of the row-major scan wins.  The winner goes to
// obs[block*npb + round] and its vix is cleared, so a later round can pick a
// cleared cell again once every cell is zero.
//
// GB300 mapping: one warp per block.  Each lane folds its strided subset of
// the block into one 64-bit key (vix:8 | h^0x80000000:32 | 0xFFFFFF-j:24,
// j < 3000^2 < 2^24 is the row-major position), so an unsigned max over the
// warp (shuffles) gives exactly the reference's winner and tie-break.
#include "common.cuh"
#include "kernels.h"

namespace siting {
namespace {

__device__ __forceinline__ unsigned long long warp_max_u64(unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
    v = w > v ? w : v;
  }
  return v;
}

__global__ void __launch_bounds__(256) findmax_kernel(uint8_t *vix, int n, float bs, int nb,
                                                      int npb, int32_t *obs) {
  const int b = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (b >= nb * nb) return;
  const int bx = b / nb, by = b - (b / nb) * nb;
  const int x0 = f2i(fmul(bs, i2f(bx))), y0 = f2i(fmul(bs, i2f(by)));
  const int x1 = min(f2i(fmul(bs, i2f(bx + 1))), n);
  const int y1 = min(f2i(fmul(bs, i2f(by + 1))), n);
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

// Flags observer indices outside [0, n*n).
__global__ void check_obs_kernel(const int32_t *obs, int nsheds, long long ncell, int *err) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nsheds; i += gridDim.x * blockDim.x)
    if (obs[i] < 0 || obs[i] >= ncell) atomicOr(err, kErrBadInput);
}

}  // namespace

cudaError_t launch_check_obs(const int32_t *obs, int nsheds, int nrows, int *d_err,
                             cudaStream_t st) {
  if (nsheds <= 0) return cudaSuccess;
  const int grid = (nsheds + 255) / 256 < 1024 ? (nsheds + 255) / 256 : 1024;
  check_obs_kernel<<<grid, 256, 0, st>>>(obs, nsheds, (long long)nrows * nrows, d_err);
  return cudaGetLastError();
}

cudaError_t launch_findmax(uint8_t *vix, int nrows, float blocksize, int nblocks, int npb,
                           int32_t *obs, cudaStream_t st) {
  const long long warps = (long long)nblocks * nblocks;
  const int threads = 256;
  const long long grid = (warps * 32 + threads - 1) / threads;
  findmax_kernel<<<(unsigned)grid, threads, 0, st>>>(vix, nrows, blocksize, nblocks, npb, obs);
  return cudaGetLastError();
}

}  // namespace siting
