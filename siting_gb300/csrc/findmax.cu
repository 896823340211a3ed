// FINDMAX: tentative observers, nwantedperblock per block
// (siting.cpp:204-241), one warp per block (findmax_dev.cuh).
#include "common.cuh"
#include "findmax_dev.cuh"
#include "kernels.h"

namespace siting {
namespace {

__global__ void __launch_bounds__(256) findmax_kernel(uint8_t *vix, int n, float bs, int nb,
                                                      int npb, int32_t *obs) {
  const int b = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (b >= nb * nb) return;
  findmax_block(vix, n, bs, nb, npb, obs, b, threadIdx.x & 31);
}

// FINDMAX of many jobs in one grid (batched form): one warp per (job, block)
// item; the job table is the kernel's parameters and a warp finds its job
// from its index.
struct FindmaxQJob {
  uint8_t *vix;
  int32_t *obs;
  int n, nb, npb;
  float bs;
  unsigned first;  // warp index of the job's first block
};
struct FindmaxQTable {
  FindmaxQJob jobs[kStageQueueMaxJobs];
  int njobs;
  unsigned total;
};

__global__ void __launch_bounds__(256) findmaxq_kernel(const __grid_constant__ FindmaxQTable tab) {
  const unsigned it = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (it >= tab.total) return;
  int lo = 0, hi = tab.njobs - 1;  // the last job whose first block is at or before `it`
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (tab.jobs[mid].first <= it)
      lo = mid;
    else
      hi = mid - 1;
  }
  const FindmaxQJob &J = tab.jobs[lo];
  findmax_block(J.vix, J.n, J.bs, J.nb, J.npb, J.obs, (int)(it - J.first),
                       threadIdx.x & 31);
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

cudaError_t launch_findmax_queue(const StageJob *jobs, int njobs, cudaStream_t st) {
  static thread_local FindmaxQTable tab;
  int j = 0;
  while (j < njobs) {
    tab.njobs = 0;
    tab.total = 0;
    for (; j < njobs && tab.njobs < kStageQueueMaxJobs; j++) {
      const StageJob &J = jobs[j];
      tab.jobs[tab.njobs++] =
          FindmaxQJob{J.vix, J.obs, J.dem.nrows, J.nb, J.npb, J.bs, tab.total};
      tab.total += (unsigned)(J.nb * J.nb);
    }
    const long long grid = ((long long)tab.total * 32 + 255) / 256;
    findmaxq_kernel<<<(unsigned)grid, 256, 0, st>>>(tab);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
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
