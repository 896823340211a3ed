// Self-test of the bounded device waits: each wait is run against a condition
// that nothing ever satisfies, with a short limit, and must give up, set the
// error flag and return (the context stays usable).  This is how failure
// detection is exercised without faulting or hanging a GPU.
#include "common.cuh"
#include "ctx.h"
#include "kernels.h"
#include "siting.h"

namespace siting {
namespace {

// which 0: the SITE group barrier, for a group of two CTAs of which only one
// is launched (the other never arrives); which 1: the TMA mbarrier, armed for
// 16 bytes that no copy delivers.
__global__ void wait_selftest_kernel(unsigned *bar, int *err, long long limit, int which) {
  __shared__ int s_flag;
  __shared__ __align__(8) uint64_t mbar;
  if (which == 0) {
    GroupBarrier gb{bar, 2u, 0u};
    group_sync(gb, err, &s_flag, limit);
  } else if (threadIdx.x == 0) {
    mbar_init(&mbar, 1);
    mbar_expect_tx(&mbar, 16);
    if (!mbar_wait(&mbar, 0, limit)) atomicOr(err, kErrTmaTimeout);
  }
}

}  // namespace
}  // namespace siting

using namespace siting;

extern "C" int siting_selftest_wait(siting_ctx *ctx, int which, long long max_cycles) {
  if (!ctx || (which != 0 && which != 1) || max_cycles <= 0 || max_cycles > kWaitCycles)
    return fail(ctx, SITING_EINVAL, "selftest_wait: invalid arguments");
  cudaSetDevice(ctx->device);
  void *p;
  int rc = ws_get(ctx, kErr, 256, &p);
  if (rc) return rc;
  int *err = static_cast<int *>(p);
  unsigned *bar = reinterpret_cast<unsigned *>(static_cast<unsigned char *>(p) + 128);
  CK(cudaMemsetAsync(p, 0, 256, ctx->stream));
  wait_selftest_kernel<<<1, 32, 0, ctx->stream>>>(bar, err, max_cycles, which);
  CK(cudaGetLastError());
  int h = 0;
  CK(cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return check_err_flags(ctx, &h, 1);
}
