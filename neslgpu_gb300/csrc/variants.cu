// variants.cu -- other mappings of the segmented scans, reductions and ranks
// onto the GPU, for the dispatcher (dispatch.cu) to choose between.
//
// The library's default kernels are "flat": tiles of a fixed number of
// elements regardless of segment boundaries, joined by a decoupled
// look-back (scan.cu, rank.cu).  That is the right shape for long segments
// and for very short ones.  In between, a segment can be handed whole to one
// CTA or one warp, which then walks it chunk by chunk with the carry in
// registers: no look-back round trips, no cross-CTA traffic, but a segment
// much longer than a chunk serialises on its owner.  Which one wins depends
// on the length distribution, which is what the dispatcher learns.
//
// Every variant computes the same CVL function as the default kernel
// (nesl/cvl/serial/vprims.c:62-201 for scans and reductions, rank.c:49-362
// for ranks): integer, boolean, min/max and rank results are bit-identical
// whichever variant runs; float64 sums differ only by association, within
// the same tolerance as the default (the default's own association already
// varies with the look-back's timing).
#include "gcvl.cuh"
#include "tma.cuh"

#include <string.h>

#include <type_traits>

namespace gcvl {

// fold of a thread's first cnt items (ident when none)
template <class Op, int ITEMS>
__device__ __forceinline__ typename Op::T thread_fold(const typename Op::T (&x)[ITEMS], int cnt) {
  if constexpr (std::is_same<Op, AddD>::value) {
    return cnt > 0 ? fx_range<ITEMS>(x, 0, cnt) : AddD::ident();
  } else {
    typename Op::T v = Op::ident();
#pragma unroll
    for (int i = 0; i < ITEMS; i++)
      if (i < cnt) v = Op::apply(v, x[i]);
    return v;
  }
}
template <class Op> __device__ __forceinline__ typename Op::T warp_incl(typename Op::T v, int lane) {
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    typename Op::T u = shfl_up(v, d);
    if (lane >= d) v = Op::apply(u, v);
  }
  return v;
}

// ---------------------------------------------------- one CTA per segment
// Segments are taken one at a time from a counter.  Each chunk of NT*ITEMS
// elements is staged through shared memory (coalesced global accesses; each
// thread then owns ITEMS consecutive elements, rows padded by one element
// against bank conflicts).
template <class Op, int MODE, int NT, int ITEMS>
__global__ void __launch_bounds__(NT) k_seg_block(typename Op::T *__restrict__ out,
                                                  const typename Op::T *__restrict__ in,
                                                  const int *__restrict__ off, int m, unsigned *counter) {
  typedef typename Op::T T;
  constexpr int CH = NT * ITEMS, NW = NT / 32;
  __shared__ T s_buf[CH + NT];
  __shared__ T s_w[NW], s_wx[NW], s_tot;
  __shared__ int s_seg;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (;;) {
    if (tid == 0) s_seg = (int)atomicAdd(counter, 1u);
    __syncthreads();
    const int s = s_seg;
    if (s >= m) return;
    const int start = __ldg(off + s), end = __ldg(off + s + 1);
    T carry = Op::init();
    for (int base = start; base < end; base += CH) {
      const int cnt = min(CH, end - base);
#pragma unroll
      for (int c = 0; c < ITEMS; c++) {
        const int e = c * NT + tid;
        if (e < cnt) s_buf[e + e / ITEMS] = __ldcs(in + base + e);
      }
      __syncthreads();
      const int my = tid * ITEMS, mc = max(0, min(ITEMS, cnt - my));
      T x[ITEMS];
#pragma unroll
      for (int i = 0; i < ITEMS; i++) x[i] = i < mc ? s_buf[my + tid + i] : Op::ident();
      const T incl = warp_incl<Op>(thread_fold<Op, ITEMS>(x, mc), lane);
      if (lane == 31) s_w[warp] = incl;
      __syncthreads();
      if (warp == 0) {
        const T w = lane < NW ? s_w[lane] : Op::ident();
        const T wi = warp_incl<Op>(w, lane);
        const T wx = shfl_up(wi, 1);
        if (lane < NW) s_wx[lane] = lane ? wx : Op::ident();
        if (lane == NW - 1) s_tot = wi;
      }
      __syncthreads();
      if (MODE == M_SCAN) {
        T ex = shfl_up(incl, 1);
        if (lane == 0) ex = Op::ident();
        T run = Op::apply(Op::apply(carry, s_wx[warp]), ex);
#pragma unroll
        for (int i = 0; i < ITEMS; i++)
          if (i < mc) {
            const T y = run;
            run = Op::apply(run, x[i]);
            s_buf[my + tid + i] = y;
          }
        __syncthreads();
#pragma unroll
        for (int c = 0; c < ITEMS; c++) {
          const int e = c * NT + tid;
          if (e < cnt) __stcs(out + base + e, s_buf[e + e / ITEMS]);
        }
      }
      carry = Op::apply(carry, s_tot);
      __syncthreads();  // the chunk buffers are reused
    }
    if (MODE == M_REDUCE && tid == 0) out[s] = carry;
    __syncthreads();  // every thread has read s_seg before it is replaced
  }
}

// --------------------------------------------------- one warp per segment
// A warp takes WBATCH consecutive segments from a counter at a time.
constexpr int WBATCH = 8, WNT = 256;
template <class Op, int MODE, int ITEMS>
__global__ void __launch_bounds__(WNT) k_seg_warp(typename Op::T *__restrict__ out,
                                                  const typename Op::T *__restrict__ in,
                                                  const int *__restrict__ off, int m, unsigned *counter) {
  typedef typename Op::T T;
  constexpr int CH = 32 * ITEMS;
  __shared__ T s_buf[WNT / 32][CH + 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  T *buf = s_buf[warp];
  for (;;) {
    unsigned got = 0;
    if (lane == 0) got = atomicAdd(counter, (unsigned)WBATCH);
    const int s0 = (int)__shfl_sync(0xffffffffu, got, 0);
    if (s0 >= m) return;
    const int s1 = min(m, s0 + WBATCH);
    for (int s = s0; s < s1; s++) {
      const int start = __ldg(off + s), end = __ldg(off + s + 1);
      T carry = Op::init();
      for (int base = start; base < end; base += CH) {
        const int cnt = min(CH, end - base);
#pragma unroll
        for (int c = 0; c < ITEMS; c++) {
          const int e = c * 32 + lane;
          if (e < cnt) buf[e + e / ITEMS] = __ldcs(in + base + e);
        }
        __syncwarp();
        const int my = lane * ITEMS, mc = max(0, min(ITEMS, cnt - my));
        T x[ITEMS];
#pragma unroll
        for (int i = 0; i < ITEMS; i++) x[i] = i < mc ? buf[my + lane + i] : Op::ident();
        const T incl = warp_incl<Op>(thread_fold<Op, ITEMS>(x, mc), lane);
        const T tot = __shfl_sync(0xffffffffu, incl, 31);
        if (MODE == M_SCAN) {
          T ex = shfl_up(incl, 1);
          if (lane == 0) ex = Op::ident();
          T run = Op::apply(carry, ex);
#pragma unroll
          for (int i = 0; i < ITEMS; i++)
            if (i < mc) {
              const T y = run;
              run = Op::apply(run, x[i]);
              buf[my + lane + i] = y;
            }
          __syncwarp();
#pragma unroll
          for (int c = 0; c < ITEMS; c++) {
            const int e = c * 32 + lane;
            if (e < cnt) __stcs(out + base + e, buf[e + e / ITEMS]);
          }
        }
        carry = Op::apply(carry, tot);
        __syncwarp();
      }
      if (MODE == M_REDUCE && lane == 0) out[s] = carry;
    }
  }
}

// ------------------------------------- rank: one CTA per short segment
// Each CTA ranks whole segments of at most RB_MAX elements in shared
// memory: a stable LSD radix sort of (key, position) pairs, 8 bits per
// pass, each pass ranking stably with warp ballots as the flat rank does,
// and then writes d[start + position] = sorted position.  Valid only when
// every segment fits (the dispatcher masks it otherwise).
constexpr int RB_NT = 256, RB_ITEMS = 8, RB_MAX = RB_NT * RB_ITEMS;
template <class K>
__global__ void __launch_bounds__(RB_NT) k_rank_seg_block(int *__restrict__ d, const K *__restrict__ src,
                                                          const int *__restrict__ off, int m, int up,
                                                          unsigned *counter, unsigned *status) {
  constexpr int PASSES = (int)sizeof(K);
  __shared__ K s_k[2][RB_MAX];
  __shared__ unsigned short s_p[2][RB_MAX];
  __shared__ unsigned short s_cnt[RB_NT / 32][256];
  __shared__ unsigned s_loc[256];
  __shared__ unsigned s_ws[RB_NT / 32];
  __shared__ int s_seg;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const unsigned lt = (1u << lane) - 1u;
  for (;;) {
    if (tid == 0) s_seg = (int)atomicAdd(counter, 1u);
    __syncthreads();
    const int s = s_seg;
    if (s >= m) return;
    const int start = __ldg(off + s), len = __ldg(off + s + 1) - start;
    if (len > RB_MAX) {  // does not fit: flag it and leave the segment alone
      if (tid == 0) atomicOr(status, DEV_RANGE);
      __syncthreads();
      continue;
    }
    for (int e = tid; e < len; e += RB_NT) {
      K k;
      if constexpr (sizeof(K) == 8) {
        const unsigned long long b = __ldcs((const unsigned long long *)src + start + e);
        const unsigned long long t = (b >> 63) ? ~b : (b ^ (1ULL << 63));
        k = (K)(up ? t : ~t);
      } else {
        k = (K)(__ldcs((const unsigned *)src + start + e) ^ (up ? 0x80000000u : 0x7FFFFFFFu));
      }
      s_k[0][e] = k;
      s_p[0][e] = (unsigned short)e;
    }
    int cur = 0;
    for (int q = 0; q < PASSES; q++) {
      const int shift = 8 * q;
      for (int i = tid; i < (RB_NT / 32) * 256; i += RB_NT) (&s_cnt[0][0])[i] = 0;
      __syncthreads();
      unsigned wr[RB_ITEMS];
      const int wbase = warp * 32 * RB_ITEMS;
#pragma unroll
      for (int c = 0; c < RB_ITEMS; c++) {
        const int e = wbase + c * 32 + lane;
        const int dg = e < len ? (int)((s_k[cur][e] >> shift) & 255) : -1;
        const unsigned peers = warp_match8(dg);
        unsigned r = 0;
        if (dg >= 0) r = s_cnt[warp][dg] + __popc(peers & lt);
        __syncwarp();
        if (dg >= 0 && (peers & lt) == 0) s_cnt[warp][dg] = (unsigned short)(s_cnt[warp][dg] + __popc(peers));
        __syncwarp();
        wr[c] = dg >= 0 ? (r << 8) | (unsigned)dg : 0xFFFFFFFFu;
      }
      __syncthreads();
      // per digit: exclusive offsets over warps, then over digits
      unsigned tot = 0;
#pragma unroll
      for (int w = 0; w < RB_NT / 32; w++) {
        const unsigned c = s_cnt[w][tid];
        s_cnt[w][tid] = (unsigned short)tot;
        tot += c;
      }
      unsigned incl = tot;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const unsigned x = shfl_up(incl, o);
        if (lane >= o) incl += x;
      }
      if (lane == 31) s_ws[warp] = incl;
      __syncthreads();
      unsigned wp = 0;
#pragma unroll
      for (int w = 0; w < RB_NT / 32; w++) if (w < warp) wp += s_ws[w];
      s_loc[tid] = wp + incl - tot;
      __syncthreads();
#pragma unroll
      for (int c = 0; c < RB_ITEMS; c++) {
        const unsigned x = wr[c];
        if (x != 0xFFFFFFFFu) {
          const int dg = (int)(x & 255u);
          const unsigned lp = s_loc[dg] + s_cnt[warp][dg] + (x >> 8);
          const int e = wbase + c * 32 + lane;
          s_k[cur ^ 1][lp] = s_k[cur][e];
          s_p[cur ^ 1][lp] = s_p[cur][e];
        }
      }
      cur ^= 1;
      __syncthreads();
    }
    for (int e = tid; e < len; e += RB_NT) d[start + s_p[cur][e]] = e;
    __syncthreads();  // the buffers are reused by the next segment
  }
}

// ------------------------------------------------------------- launch ---
enum Variant { V_FLAT = 0, V_BLOCK_L = 1, V_BLOCK_S = 2, V_WARP_L = 3, V_WARP_S = 4, V_RANK_BLOCK = 5,
               V_COUNT = 6 };

template <class F> static int resident_grid(F kernel, int nt, int m_work) {
  int per = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, nt, 0);
  if (per < 1) per = 1;
  long g = (long)st().sm_count * per;
  if (g > m_work) g = m_work;
  return (int)(g < 1 ? 1 : g);
}

template <class Op, int MODE>
static bool run_seg_variant(int v, vec_p d, vec_p s, vec_p sd, int n, int m, unsigned *counter) {
  typedef typename Op::T T;
  SegView sv = seg_view(sd, n, m);
  T *out = (T *)d;
  const T *in = (const T *)s;
  switch (v) {
    case V_BLOCK_L: {
      auto k = k_seg_block<Op, MODE, 256, 8>;
      k<<<resident_grid(k, 256, m), 256, 0, stream()>>>(out, in, sv.off, m, counter);
      break;
    }
    case V_BLOCK_S: {
      auto k = k_seg_block<Op, MODE, 128, 4>;
      k<<<resident_grid(k, 128, m), 128, 0, stream()>>>(out, in, sv.off, m, counter);
      break;
    }
    case V_WARP_L: {
      auto k = k_seg_warp<Op, MODE, 8>;
      k<<<resident_grid(k, WNT, (m + 7) / 8), WNT, 0, stream()>>>(out, in, sv.off, m, counter);
      break;
    }
    case V_WARP_S: {
      auto k = k_seg_warp<Op, MODE, 2>;
      k<<<resident_grid(k, WNT, (m + 7) / 8), WNT, 0, stream()>>>(out, in, sv.off, m, counter);
      break;
    }
    default:
      return false;
  }
  launch_check("seg variant");
  return true;
}

}  // namespace gcvl

using namespace gcvl;

// The CVL entry points a variant can stand in for.
struct VariantPrim {
  const char *name;
  int kind;  // 0 scan, 1 reduce, 2 rank
  int is_double;
};
static const VariantPrim kPrims[] = {
    {"add_sez", 0, 0}, {"add_sed", 0, 1}, {"max_sez", 0, 0}, {"max_sed", 0, 1},
    {"add_rez", 1, 0}, {"add_red", 1, 1}, {"max_rez", 1, 0}, {"max_red", 1, 1},
    {"rku_lez", 2, 0}, {"rku_led", 2, 1}, {"rkd_lez", 2, 0}, {"rkd_led", 2, 1},
};
static const VariantPrim *find_prim(const char *name) {
  for (const auto &p : kPrims)
    if (strcmp(p.name, name) == 0) return &p;
  return nullptr;
}

// the default (flat) entry points
extern "C" {
void add_sez(vec_p, vec_p, vec_p, int, int, vec_p); void add_sed(vec_p, vec_p, vec_p, int, int, vec_p);
void max_sez(vec_p, vec_p, vec_p, int, int, vec_p); void max_sed(vec_p, vec_p, vec_p, int, int, vec_p);
void add_rez(vec_p, vec_p, vec_p, int, int, vec_p); void add_red(vec_p, vec_p, vec_p, int, int, vec_p);
void max_rez(vec_p, vec_p, vec_p, int, int, vec_p); void max_red(vec_p, vec_p, vec_p, int, int, vec_p);
void rku_lez(vec_p, vec_p, vec_p, int, int, vec_p); void rku_led(vec_p, vec_p, vec_p, int, int, vec_p);
void rkd_lez(vec_p, vec_p, vec_p, int, int, vec_p); void rkd_led(vec_p, vec_p, vec_p, int, int, vec_p);
int add_sez_scratch(int, int); int add_sed_scratch(int, int); int max_sez_scratch(int, int);
int max_sed_scratch(int, int); int add_rez_scratch(int, int); int add_red_scratch(int, int);
int max_rez_scratch(int, int); int max_red_scratch(int, int); int rku_lez_scratch(int, int);
int rku_led_scratch(int, int); int rkd_lez_scratch(int, int); int rkd_led_scratch(int, int);
}

typedef void (*SegFn)(vec_p, vec_p, vec_p, int, int, vec_p);
typedef int (*SegScratchFn)(int, int);
static SegFn flat_fn(const char *name) {
  static const struct { const char *n; SegFn f; } t[] = {
      {"add_sez", add_sez}, {"add_sed", add_sed}, {"max_sez", max_sez}, {"max_sed", max_sed},
      {"add_rez", add_rez}, {"add_red", add_red}, {"max_rez", max_rez}, {"max_red", max_red},
      {"rku_lez", rku_lez}, {"rku_led", rku_led}, {"rkd_lez", rkd_lez}, {"rkd_led", rkd_led}};
  for (const auto &e : t)
    if (strcmp(e.n, name) == 0) return e.f;
  return nullptr;
}
static SegScratchFn flat_scratch(const char *name) {
  static const struct { const char *n; SegScratchFn f; } t[] = {
      {"add_sez", add_sez_scratch}, {"add_sed", add_sed_scratch}, {"max_sez", max_sez_scratch},
      {"max_sed", max_sed_scratch}, {"add_rez", add_rez_scratch}, {"add_red", add_red_scratch},
      {"max_rez", max_rez_scratch}, {"max_red", max_red_scratch}, {"rku_lez", rku_lez_scratch},
      {"rku_led", rku_led_scratch}, {"rkd_lez", rkd_lez_scratch}, {"rkd_led", rkd_led_scratch}};
  for (const auto &e : t)
    if (strcmp(e.n, name) == 0) return e.f;
  return nullptr;
}

// Whether variant v can compute prim: scans and reductions take the flat
// kernel and the four segment-owner mappings; ranks take the flat rank and,
// when the longest segment fits a CTA's shared memory, the per-segment rank.
GCVL_EXPORT int gcvl_variant_valid(const char *prim, int v, int max_len) {
  const VariantPrim *p = find_prim(prim);
  if (!p || v < 0 || v >= V_COUNT) return 0;
  if (v == V_FLAT) return 1;
  if (p->kind == 2) return v == V_RANK_BLOCK && max_len <= RB_MAX;
  return v != V_RANK_BLOCK;
}
GCVL_EXPORT int gcvl_variant_count(void) { return V_COUNT; }

// Scratch (8-byte units) for any variant of prim: the flat kernel's, plus a
// counter for the segment-owner mappings.
GCVL_EXPORT int gcvl_variant_scratch(const char *prim, int n, int m) {
  SegScratchFn f = flat_scratch(prim);
  if (!f) return 0;
  const int u = f(n, m);
  return u > 32 ? u : 32;
}

// Runs variant v of prim (a CVL segmented entry point name) with the CVL
// argument order.  Returns 0, or a GCVL error code (5: unknown prim or an
// invalid variant).
GCVL_EXPORT int gcvl_run_variant(const char *prim, int v, vec_p d, vec_p s, vec_p sd, int n, int m,
                                 vec_p scratch) {
  ensure_init();
  const VariantPrim *p = find_prim(prim);
  if (!p || v < 0 || v >= V_COUNT) { set_error(GCVL_ERR_RANGE, "gcvl_run_variant: unknown primitive or variant"); return GCVL_ERR_RANGE; }
  if (v == V_FLAT || n <= 0 || m <= 0) {
    flat_fn(prim)(d, s, sd, n, m, scratch);
    return st().err;
  }
  unsigned *counter = (unsigned *)scratch_or_work(scratch, 256);
  if (!counter) return st().err;
  counter = (unsigned *)align_up((size_t)counter, 16);
  GCVL_CK(cudaMemsetAsync(counter, 0, 4, stream()));
  bool ok = false;
  if (p->kind == 2) {
    if (v == V_RANK_BLOCK) {
      SegView sv = seg_view(sd, n, m);
      const int up = prim[2] == 'u';
      if (p->is_double) {
        auto k = k_rank_seg_block<unsigned long long>;
        k<<<resident_grid(k, RB_NT, m), RB_NT, 0, stream()>>>((int *)d, (const unsigned long long *)s, sv.off, m,
                                                              up, counter, st().d_status);
      } else {
        auto k = k_rank_seg_block<unsigned>;
        k<<<resident_grid(k, RB_NT, m), RB_NT, 0, stream()>>>((int *)d, (const unsigned *)s, sv.off, m, up,
                                                              counter, st().d_status);
      }
      launch_check("k_rank_seg_block");
      ok = true;
    }
  } else {
    const bool add = prim[0] == 'a', scan = p->kind == 0;
    if (p->is_double) {
      if (add) ok = scan ? run_seg_variant<AddD, M_SCAN>(v, d, s, sd, n, m, counter)
                         : run_seg_variant<AddD, M_REDUCE>(v, d, s, sd, n, m, counter);
      else ok = scan ? run_seg_variant<MaxD, M_SCAN>(v, d, s, sd, n, m, counter)
                     : run_seg_variant<MaxD, M_REDUCE>(v, d, s, sd, n, m, counter);
    } else {
      if (add) ok = scan ? run_seg_variant<AddZ, M_SCAN>(v, d, s, sd, n, m, counter)
                         : run_seg_variant<AddZ, M_REDUCE>(v, d, s, sd, n, m, counter);
      else ok = scan ? run_seg_variant<MaxZ, M_SCAN>(v, d, s, sd, n, m, counter)
                     : run_seg_variant<MaxZ, M_REDUCE>(v, d, s, sd, n, m, counter);
    }
  }
  if (!ok) { set_error(GCVL_ERR_RANGE, "gcvl_run_variant: variant not valid for this primitive"); return GCVL_ERR_RANGE; }
  return st().err;
}
