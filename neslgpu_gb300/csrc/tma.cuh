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
// Iteration limit of the waits that let a CTA's own bulk copies land before
// it reads or leaves their shared memory, after a shorter wait gave up.
constexpr int kDrainLimit = 1 << 20;
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
// Arrive at a named barrier without waiting (the producer side of bar.sync).
__device__ __forceinline__ void named_arrive(int id, int n) {
  asm volatile("bar.arrive %0, %1;" ::"r"(id), "r"(n) : "memory");
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
// A thread's group of at most 16 doubles is summed in 64-bit fixed point at
// the scale of its largest exponent `emax`: each value's magnitude is
// truncated to a multiple of 2^(emax-1075) -- the unit in the last place of
// the largest value -- and the integers are added exactly (sixteen 53-bit
// mantissas fit in 57 bits); the total is converted to double once.  The
// error is under 16 ulp of the group's largest value, so over a segment
// under 2^-48 of the sum of the magnitudes, and the work runs on the integer
// pipes instead of GB300's narrow FP64 pipe (2 FP64 operations per clock per
// SM).  Truncating instead of rounding each addend measured 6 % faster on
// the float64 reduction.
__device__ __forceinline__ int fx_exp(unsigned long long b) {
  int e = (int)((b >> 52) & 0x7FF);
  return e ? e : 1;
}
__device__ __forceinline__ void fx_add(long long &acc, unsigned long long b, int emax) {
  int e = (int)((b >> 52) & 0x7FF);
  unsigned long long m = b & 0xFFFFFFFFFFFFFULL;
  if (e) m |= 1ULL << 52; else e = 1;
  const int d = min(emax - e, 63);
  const unsigned long long v = m >> d;  // magnitude truncated to the common scale
  const long long sgn = (long long)b >> 63;  // 0 or -1
  acc += ((long long)v ^ sgn) - sgn;
}
// acc * 2^(emax - 1075), rounded once to the nearest double (ties to even),
// by integer bit assembly: no FP64 pipe work.  The scans use it (their FP64
// pipe carries the outputs' add chain: 1.228 -> 1.212 ms for the float64
// scan at 2^28); the reductions keep the FP64 conversion below (their ALU is
// the busier pipe: the integer form cost them 3 %).
__device__ __forceinline__ double fx_to_double_alu(long long acc, int emax) {
  if (acc == 0) return 0.0;
  const unsigned long long sgn = acc < 0 ? 0x8000000000000000ULL : 0ULL;
  unsigned long long a = acc < 0 ? 0ULL - (unsigned long long)acc : (unsigned long long)acc;
  const int p = 63 - __clzll((long long)a);  // top bit
  int be = p + emax - 52;                   // biased exponent of the result
  if (be <= 0)  // subnormal: a * 2^(emax-1) units of 2^-1074, exact (below 2^52)
    return __longlong_as_double((long long)(sgn | (a << (emax - 1))));
  if (p > 52) {
    const int sh = p - 52;
    const unsigned long long rem = a & ((1ULL << sh) - 1ULL), half = 1ULL << (sh - 1);
    a >>= sh;
    if (rem > half || (rem == half && (a & 1ULL))) {
      ++a;
      if (a >> 53) { a >>= 1; ++be; }
    }
  } else {
    a <<= (52 - p);
  }
  if (be >= 2047) return __longlong_as_double((long long)(sgn | 0x7FF0000000000000ULL));
  return __longlong_as_double((long long)(sgn | ((unsigned long long)be << 52) | (a & 0xFFFFFFFFFFFFFULL)));
}
// the same, by the int64 -> float64 conversion and one multiply
__device__ __forceinline__ double fx_to_double(long long acc, int emax) {
  const double v = __ll2double_rn(acc);
  if (emax >= 53) return v * __longlong_as_double((long long)(emax - 52) << 52);
  return scalbn(v, emax - 1075);
}

// The fixed-point sum of the items of x[LO..HI) that lie in [from, to).
template <int ITEMS, int LO, int HI>
__device__ __forceinline__ double fx_range_part(const double (&x)[ITEMS], int from, int to) {
  int emax = 1;
#pragma unroll
  for (int i = LO; i < HI; i++)
    if (i >= from && i < to) emax = max(emax, fx_exp((unsigned long long)__double_as_longlong(x[i])));
  if (emax == 2047) {
    double v = -0.0;
#pragma unroll
    for (int i = LO; i < HI; i++)
      if (i >= from && i < to) v = __dadd_rn(v, x[i]);
    return v;
  }
  long long acc = 0;
#pragma unroll
  for (int i = LO; i < HI; i++)
    if (i >= from && i < to) fx_add(acc, (unsigned long long)__double_as_longlong(x[i]), emax);
  return fx_to_double(acc, emax);
}

// Sum of x[from..to) by the fixed-point path (FP64 when inf/NaN present).
template <int ITEMS>
__device__ __forceinline__ double fx_range(const double (&x)[ITEMS], int from, int to) {
  int emax = 1;
#pragma unroll
  for (int i = 0; i < ITEMS; i++)
    if (i >= from && i < to) emax = max(emax, fx_exp((unsigned long long)__double_as_longlong(x[i])));
  if (emax == 2047) {
    double v = -0.0;
#pragma unroll
    for (int i = 0; i < ITEMS; i++)
      if (i >= from && i < to) v = __dadd_rn(v, x[i]);
    return v;
  }
  long long acc = 0;
#pragma unroll
  for (int i = 0; i < ITEMS; i++)
    if (i >= from && i < to) fx_add(acc, (unsigned long long)__double_as_longlong(x[i]), emax);
  return fx_to_double(acc, emax);
}

}  // namespace gcvl
