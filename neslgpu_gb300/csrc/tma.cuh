// tma.cuh -- inline-PTX helpers for TMA tensor copies and mbarriers, and
// the integer arithmetic that keeps float64 folds off the FP64 pipe.
#pragma once

#include <cuda.h>

#include "gcvl.cuh"

namespace gcvl {

// ------------------------------------------------------------ TMA / mbarrier
__device__ __forceinline__ unsigned smem_addr(const void *p) {
  return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long *bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long *bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// 2-D tiled TMA load of box {inner, rows} at coordinates (x, y) into smem.
__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, unsigned long long *bar,
                                            int x, int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];"
      ::"r"(smem_addr(dst)), "l"(map), "r"(smem_addr(bar)), "r"(x), "r"(y)
      : "memory");
}
__device__ __forceinline__ void tma_store_2d(const CUtensorMap *map, const void *src, int x, int y) {
  asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%2, %3}], [%1];"
               ::"l"(map), "r"(smem_addr(src)), "r"(x), "r"(y)
               : "memory");
}
// 1-D bulk copy global -> shared (16-byte aligned addresses, size % 16 == 0).
__device__ __forceinline__ void bulk_load_1d(void *dst, const void *src, unsigned bytes,
                                             unsigned long long *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
      ::"r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}
__device__ __forceinline__ void mbar_arrive(unsigned long long *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}
// Bounded wait for the completion of phase `parity`; false on timeout.
__device__ __forceinline__ bool mbar_wait(unsigned long long *bar, unsigned parity, int limit) {
  int it = 0;
  while (!mbar_try_wait(bar, parity)) {
    if (++it >= limit) return false;
  }
  return true;
}
__device__ __forceinline__ void bulk_wait_read_1() {
  asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory");
}
// Barrier among the first `n` threads of the CTA (the consumer warps).
__device__ __forceinline__ void named_sync(int id, int n) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_read_all() {
  asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
// Byte offset of the 16-byte unit `c` of 128-byte row `r` in a tile that
// TMA wrote with 128-byte swizzling (buffer 1024-byte aligned).
__device__ __forceinline__ int swz(int r, int c) { return r * 128 + (((c ^ r) & 7) << 4); }

// ------------------------------------------- float64 sums in integers ---
// A group of doubles is summed exactly in a signed 128-bit fixed-point
// accumulator whose scale follows the largest exponent `emax` of the group:
// a value m * 2^(E-1075) becomes m << (E - emax + 70).  Sixteen 53-bit
// mantissas shifted by at most 70 stay below 2^127; addends smaller than
// 2^-70 of the largest one are truncated (far below the float64 rounding
// of the result).  The total is rounded to double once, to nearest even.
constexpr int FX_GUARD = 70;

struct Fx128 { unsigned long long lo, hi; };

__device__ __forceinline__ int fx_exp(unsigned long long b) {
  int e = (int)((b >> 52) & 0x7FF);
  return e ? e : 1;
}
__device__ __forceinline__ void fx_add(Fx128 &a, unsigned long long b, int emax) {
  int e = (int)((b >> 52) & 0x7FF);
  unsigned long long m = b & 0xFFFFFFFFFFFFFULL;
  if (e) m |= 1ULL << 52; else e = 1;
  int sh = e - emax + FX_GUARD;
  unsigned long long lo, hi;
  if (sh >= 64) { lo = 0; hi = m << (sh - 64); }
  else if (sh > 0) { lo = m << sh; hi = m >> (64 - sh); }
  else if (sh > -64) { lo = m >> (-sh); hi = 0; }
  else { lo = 0; hi = 0; }
  if (b >> 63) {
    lo = ~lo + 1ULL;
    hi = ~hi + (lo == 0ULL ? 1ULL : 0ULL);
  }
  asm("add.cc.u64 %0, %0, %2;\n\taddc.u64 %1, %1, %3;" : "+l"(a.lo), "+l"(a.hi) : "l"(lo), "l"(hi));
}
// The accumulated value, rounded to the nearest double (ties to even).
__device__ __forceinline__ double fx_to_double(Fx128 a, int emax) {
  unsigned long long lo = a.lo, hi = a.hi;
  const bool neg = (long long)hi < 0;
  if (neg) { lo = ~lo + 1ULL; hi = ~hi + (lo == 0ULL ? 1ULL : 0ULL); }
  if ((hi | lo) == 0ULL) return 0.0;
  const int lz = hi ? __clzll((long long)hi) : 64 + __clzll((long long)lo);
  const int p = 127 - lz;
  int eb = p + emax - (FX_GUARD + 52);
  unsigned long long mant;
  if (eb <= 0 || eb >= 2047) {
    // subnormal or overflowing result: let the FP64 unit round it
    double r = __ull2double_rn(hi) * 0x1.0p64 + __ull2double_rn(lo);
    r = scalbn(r, emax - 1075 - FX_GUARD);
    return neg ? -r : r;
  }
  if (p <= 52) {
    mant = lo << (52 - p);
  } else {
    const int s = p - 52;  // 1 .. 75
    unsigned long long rem_hi, rem_lo, half_hi, half_lo;
    if (s >= 64) {
      mant = hi >> (s - 64);
      rem_hi = (s == 64) ? 0ULL : (hi & ((1ULL << (s - 64)) - 1ULL));
      rem_lo = lo;
      half_hi = (s == 64) ? 0ULL : (1ULL << (s - 65));
      half_lo = (s == 64) ? (1ULL << 63) : 0ULL;
    } else {
      mant = (lo >> s) | (hi << (64 - s));
      rem_hi = 0ULL;
      rem_lo = lo & ((1ULL << s) - 1ULL);
      half_hi = 0ULL;
      half_lo = 1ULL << (s - 1);
    }
    const bool above = rem_hi > half_hi || (rem_hi == half_hi && rem_lo > half_lo);
    const bool tie = rem_hi == half_hi && rem_lo == half_lo;
    if (above || (tie && (mant & 1ULL))) {
      ++mant;
      if (mant == (1ULL << 53)) { mant >>= 1; ++eb; if (eb >= 2047) return neg ? -INFINITY : INFINITY; }
    }
  }
  const unsigned long long bits =
      ((unsigned long long)neg << 63) | ((unsigned long long)eb << 52) | (mant & 0xFFFFFFFFFFFFFULL);
  return __longlong_as_double((long long)bits);
}

}  // namespace gcvl
