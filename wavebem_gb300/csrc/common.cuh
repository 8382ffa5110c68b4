// Shared device helpers: error reporting, bounded mbarrier waits, bulk copies
// (TMA, cp.async.bulk) and double-float arithmetic on FP32 units.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace wbem {

// Device-side error word (first error wins). Codes match wbem.h.
struct DevErr {
  int code;
  int where;
  int a, b;
};

__device__ __forceinline__ void dev_fail(DevErr* e, int code, int where, int a = 0, int b = 0) {
  if (atomicCAS(&e->code, 0, code) == 0) {
    e->where = where;
    e->a = a;
    e->b = b;
  }
}

// ------------------------------------------------------------- mbarrier / TMA
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, "
      "p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait on an mbarrier phase. Returns false after `limit` polls.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity,
                                                  uint32_t limit = (1u << 24)) {
  for (uint32_t it = 0; it < limit; ++it)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// 1-D bulk copy global -> shared (TMA engine), completion counted on `bar`.
// dst, src 16-byte aligned; bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes,
                                         uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cta.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

// ---------------------------------------------------------- double-float math
// A value is hi + lo with |lo| <= ulp(hi)/2 (about 48 significant bits).
struct df {
  float hi, lo;
};

__device__ __forceinline__ df two_sum(float a, float b) {
  float s = a + b;
  float bb = s - a;
  float e = (a - (s - bb)) + (b - bb);
  return {s, e};
}
__device__ __forceinline__ df fast_two_sum(float a, float b) {
  float s = a + b;
  float e = b - (s - a);
  return {s, e};
}
__device__ __forceinline__ df two_prod(float a, float b) {
  float p = a * b;
  float e = __fmaf_rn(a, b, -p);
  return {p, e};
}
__device__ __forceinline__ df df_add(df a, df b) {
  df s = two_sum(a.hi, b.hi);
  df t = two_sum(a.lo, b.lo);
  s.lo += t.hi;
  s = fast_two_sum(s.hi, s.lo);
  s.lo += t.lo;
  return fast_two_sum(s.hi, s.lo);
}
// cheaper add (sloppy in the lo parts, fine for sums of like-signed terms and
// for accumulating small corrections)
__device__ __forceinline__ df df_add_fast(df a, df b) {
  df s = two_sum(a.hi, b.hi);
  s.lo += a.lo + b.lo;
  return fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ df df_add_f(df a, float b) {
  df s = two_sum(a.hi, b);
  s.lo += a.lo;
  return fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ df df_mul(df a, df b) {
  df p = two_prod(a.hi, b.hi);
  p.lo = __fmaf_rn(a.hi, b.lo, p.lo);
  p.lo = __fmaf_rn(a.lo, b.hi, p.lo);
  return fast_two_sum(p.hi, p.lo);
}
__device__ __forceinline__ df df_mul_f(df a, float b) {
  df p = two_prod(a.hi, b);
  p.lo = __fmaf_rn(a.lo, b, p.lo);
  return fast_two_sum(p.hi, p.lo);
}
__device__ __forceinline__ df df_from_double(double x) {
  float h = __double2float_rn(x);
  float l = __double2float_rn(x - (double)h);
  return {h, l};
}
__device__ __forceinline__ double df_to_double(df a) { return (double)a.hi + (double)a.lo; }

}  // namespace wbem
