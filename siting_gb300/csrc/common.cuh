// Device helpers shared by the siting kernels (sm_103a).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "kernels.h"

namespace siting {

// Bounded waits: ~2^31 cycles (about a second at GB300 clocks).
constexpr long long kWaitCycles = 1ll << 31;

// ---- reference arithmetic --------------------------------------------------
// glibc LCG step on 31 bits (siting.cpp:29-33).
__host__ __device__ __forceinline__ uint32_t lcg_step(uint32_t s) {
  return (1103515245u * (s & 0x7fffffffu) + 12345u) & 0x7fffffffu;
}

// FP32 operations with explicit round-to-nearest so that nvcc never contracts
// a multiply and an add into an FMA (the reference's results are those of
// separately rounded operations).
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float i2f(int v) { return __int2float_rn(v); }
__device__ __forceinline__ int f2i(float v) { return __float2int_rz(v); }
// (int)roundf(v), half away from zero, for |v| < 2^31: truncation of
// v + copysign(pred(0.5), v), with pred(0.5) = 0.5 - 2^-25 the float just
// below one half (the usual trunc-based round: adding 0.5 itself would round
// 0.5 - 2^-25 up to 1).  Checked against roundf over every float in range.
__device__ __forceinline__ int round_i(float v) {
  const float h = __uint_as_float((__float_as_uint(v) & 0x80000000u) | 0x3effffffu);
  return __float2int_rz(__fadd_rn(v, h));
}

// Packed FP32 pairs (low half, high half) for the f32x2 instructions of
// sm_100 and later: each half is an IEEE round-to-nearest operation of its
// own, so a packed add or multiply equals two scalar ones bit for bit.
__device__ __forceinline__ unsigned long long f2_pack(float lo, float hi) {
  unsigned long long v;
  asm("mov.b64 %0, {%1, %2};" : "=l"(v) : "f"(lo), "f"(hi));
  return v;
}
__device__ __forceinline__ float f2_lo(unsigned long long v) {
  float lo;
  asm("{\n\t.reg .f32 t;\n\tmov.b64 {%0, t}, %1;\n\t}" : "=f"(lo) : "l"(v));
  return lo;
}
__device__ __forceinline__ float f2_hi(unsigned long long v) {
  float hi;
  asm("{\n\t.reg .f32 t;\n\tmov.b64 {t, %0}, %1;\n\t}" : "=f"(hi) : "l"(v));
  return hi;
}
__device__ __forceinline__ unsigned long long f2_add(unsigned long long a, unsigned long long b) {
  unsigned long long d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ unsigned long long f2_mul(unsigned long long a, unsigned long long b) {
  unsigned long long d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
// copysign(pred(0.5), v): the addend of round_i for v's sign
__device__ __forceinline__ float round_addend(float v) {
  return __uint_as_float((__float_as_uint(v) & 0x80000000u) | 0x3effffffu);
}

// ---- memory-order helpers --------------------------------------------------
__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned *p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_u32(unsigned *p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// ---- mbarrier + TMA (cp.async.bulk.tensor) ---------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

// Waits for phase `parity` of the mbarrier; false if the bounded wait expired.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity,
                                          long long limit = kWaitCycles) {
  const uint32_t addr = smem_u32(bar);
  const long long t0 = clock64();
  for (;;) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(addr), "r"(parity)
        : "memory");
    if (done) return true;
    if (clock64() - t0 > limit) return false;
  }
}

// TMA load of a DEM window (3-D map of make_dem_tensor_map): columns from
// y0 (a multiple of 8) and rows from x0, into dense row-major shared memory.
// Out-of-DEM rows and columns are filled with zeros.
__device__ __forceinline__ void tma_load_window(void *dst, const CUtensorMap *map, int y0, int x0,
                                                uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(0), "r"(y0 >> 3), "r"(x0), "r"(smem_u32(bar))
      : "memory");
}

// Bulk prefetch of [p, p+bytes) into L2 (p and bytes rounded out to 16 bytes).
__device__ __forceinline__ void prefetch_l2(const void *p, size_t bytes) {
  const uintptr_t a = reinterpret_cast<uintptr_t>(p) & ~uintptr_t(15);
  const uintptr_t e = (reinterpret_cast<uintptr_t>(p) + bytes + 15) & ~uintptr_t(15);
  if (e > a)
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(a), "r"((unsigned)(e - a))
                 : "memory");
}

// ---- bounded barrier over a group of co-resident CTAs ------------------------
// bar[0] counts arrivals and is never reset: the g-th barrier completes when
// it reaches g * nctas.  One release-add per CTA, then acquire-polls.  Must be
// reached by all threads of every CTA of the group.  Returns false (and sets
// err) when the wait expired; the group then abandons its work.
struct GroupBarrier {
  unsigned *bar;
  unsigned nctas;
  unsigned gen;
};

__device__ __forceinline__ void red_release_add(unsigned *p, unsigned v) {
  asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ bool group_sync(GroupBarrier &b, int *err, int *s_flag,
                                          long long limit = kWaitCycles) {
  __syncthreads();
  b.gen++;
  if (threadIdx.x == 0) {
    int ok = 1;
    red_release_add(&b.bar[0], 1u);
    const unsigned target = b.gen * b.nctas;
    const long long t0 = clock64();
    while ((int)(ld_acquire_u32(&b.bar[0]) - target) < 0) {
      if (clock64() - t0 > limit) {
        atomicOr(err, kErrBarrierTimeout);
        ok = 0;
        break;
      }
    }
    *s_flag = ok;
  }
  __syncthreads();
  const bool ok = *s_flag != 0;
  __syncthreads();
  return ok;
}

__host__ __device__ __forceinline__ int ceil_div(int a, int b) { return (a + b - 1) / b; }

}  // namespace siting
