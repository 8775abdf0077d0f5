// vprims.cu -- extract / replace / distribute / index (segmented forms),
// permute / back-permute, the flag and default permutes, and pack.
//
// Semantics: nesl/cvl/serial/vprims.c:207-467, vecops.c:22-286 and
// library.c:12-165.  Segmented forms find each element's segment from the
// device segment descriptor (offsets + granule table) instead of storing a
// per-element segment id, so a call reads only its own operands.
//
// Permutes with repeated indices: NESL's permute takes a permutation.  When
// an index repeats, which value lands at the collided position is
// unspecified here (the serial CVL keeps the last writer).
#include "gcvl.cuh"

// the library's own +-scan (scan.cu), used for the pack's tile offsets
extern "C" void add_suz(vec_p d, vec_p s, int len, vec_p scratch);
extern "C" int add_suz_scratch(int len);

namespace gcvl {

constexpr int VBLOCK = 256;
constexpr int SITEMS = 4;  // consecutive elements per thread in segmented maps

inline int grid_for(long work, int per_block) {
  long g = (work + per_block - 1) / per_block;
  return (int)(g < 1 ? 1 : g);
}

// Calls f(k, s, seg_start) for every element k of a segmented vector, with s
// the segment holding k.  Each thread walks SITEMS consecutive elements.
template <class F>
__global__ void __launch_bounds__(VBLOCK) k_segwalk(F f, SegView sv) {
  long k0 = ((long)blockIdx.x * VBLOCK + threadIdx.x) * SITEMS;
  if (k0 >= sv.n) return;
  int cnt = (int)min((long)SITEMS, (long)sv.n - k0);
  int s = seg_of(sv, (int)k0);
  int start = __ldg(sv.off + s), end = __ldg(sv.off + s + 1);
  for (int i = 0; i < cnt; i++) {
    int k = (int)k0 + i;
    while (k >= end) { ++s; start = end; end = __ldg(sv.off + s + 1); }
    f(k, s, start);
  }
}
template <class F> void segwalk(F f, const SegView &sv, const char *name) {
  if (sv.n <= 0 || sv.m <= 0) return;
  k_segwalk<F><<<grid_for(((long)sv.n + SITEMS - 1) / SITEMS, VBLOCK), VBLOCK, 0, stream()>>>(f, sv);
  launch_check(name);
}
// Segmented maps whose result is one value per element (DIST, INDEX,
// segmented BPERMUTE): a warp owns SMI*32 consecutive elements, each lane
// SMI consecutive ones.  Phase 1 walks the lane's elements through the
// segment descriptor (one segment lookup, then a walk) and records a token
// per element (the segment, or the source address); phase 2 fetches all
// the lane's values at once (independent loads in flight); the values pass
// through shared memory so that every global load and store is coalesced.
#ifndef GCVL_SMI
#define GCVL_SMI 16
#endif
#ifndef GCVL_SMB
#define GCVL_SMB 128
#endif
constexpr int SMI = GCVL_SMI, SMB = GCVL_SMB;
template <class F>
__global__ void __launch_bounds__(SMB) k_segmap(F f, SegView sv) {
  typedef typename F::T T;
  constexpr int WE = 32 * SMI, PADW = WE + 32;
  __shared__ T s_val[SMB / 32][PADW];
  __shared__ int s_aux[F::AUX ? SMB / 32 : 1][F::AUX ? PADW : 1];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const long wbase = ((long)blockIdx.x * (SMB / 32) + warp) * WE;
  if (wbase >= sv.n) return;
  const int wcnt = (int)min((long)WE, (long)sv.n - wbase);
  if constexpr (F::AUX) {
#pragma unroll
    for (int j = 0; j < SMI; j++) {
      const int e = j * 32 + lane;
      if (e < wcnt) s_aux[warp][e + e / SMI] = __ldcs(f.aux + wbase + e);
    }
    __syncwarp();
  }
  const int e0 = lane * SMI;
  const int cnt = max(0, min(SMI, wcnt - e0));
  long long tok[SMI];
  if (cnt > 0) {
    const int k0 = (int)(wbase + e0);
    int sg = seg_of(sv, k0);
    int start = __ldg(sv.off + sg), end = __ldg(sv.off + sg + 1);
#pragma unroll
    for (int i = 0; i < SMI; i++) {
      if (i < cnt) {
        const int k = k0 + i;
        while (k >= end) { ++sg; start = end; end = __ldg(sv.off + sg + 1); }
        int a = 0;
        if constexpr (F::AUX) a = s_aux[warp][e0 + lane + i];
        tok[i] = f.token(k, sg, start, a);
        // values that come from a per-segment table are fetched in the walk
        if constexpr (!F::GATHER) s_val[warp][e0 + lane + i] = f.fetch(tok[i]);
      }
    }
  }
  if constexpr (F::GATHER) {  // all of the lane's gathers in flight at once
    T v[SMI];
#pragma unroll
    for (int i = 0; i < SMI; i++)
      if (i < cnt) v[i] = f.fetch(tok[i]);
#pragma unroll
    for (int i = 0; i < SMI; i++)
      if (i < cnt) s_val[warp][e0 + lane + i] = v[i];
  }
  __syncwarp();
#pragma unroll
  for (int j = 0; j < SMI; j++) {
    const int e = j * 32 + lane;
    if (e < wcnt) __stcs(f.d + wbase + e, s_val[warp][e + e / SMI]);
  }
}
template <class F> void segmap(F f, const SegView &sv, const char *name) {
  if (sv.n <= 0 || sv.m <= 0) return;
  const long per = (long)SMB * SMI;
  k_segmap<F><<<(int)((sv.n + per - 1) / per), SMB, 0, stream()>>>(f, sv);
  launch_check(name);
}
// Segmented permute, d[start(seg(k)) + i[k]] = s[k]: a warp owns SMI*32
// consecutive elements; each lane walks SMI consecutive ones through the
// segment descriptor and records their segment starts in shared memory;
// then the index and value loads are coalesced (element j*32 + lane) and
// all of a lane's stores are in flight together.
template <class T>
__global__ void __launch_bounds__(SMB) k_segscatter(T *__restrict__ d, const T *__restrict__ s,
                                                    const int *__restrict__ idx, SegView sv) {
  constexpr int WE = 32 * SMI, PADW = WE + 32;
  __shared__ int s_start[SMB / 32][PADW];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const long wbase = ((long)blockIdx.x * (SMB / 32) + warp) * WE;
  if (wbase >= sv.n) return;
  const int wcnt = (int)min((long)WE, (long)sv.n - wbase);
  // index and value loads issued before the walk, so that they overlap it
  int ix[SMI];
  T v[SMI];
#pragma unroll
  for (int j = 0; j < SMI; j++) {
    const int e = j * 32 + lane;
    if (e < wcnt) { ix[j] = __ldcs(idx + wbase + e); v[j] = __ldcs(s + wbase + e); }
  }
  const int e0 = lane * SMI;
  const int cnt = max(0, min(SMI, wcnt - e0));
  if (cnt > 0) {
    const int k0 = (int)(wbase + e0);
    int sg = seg_of(sv, k0);
    int start = __ldg(sv.off + sg), end = __ldg(sv.off + sg + 1);
#pragma unroll
    for (int i = 0; i < SMI; i++) {
      if (i < cnt) {
        while (k0 + i >= end) { ++sg; start = end; end = __ldg(sv.off + sg + 1); }
        s_start[warp][e0 + lane + i] = start;  // element e at e + e / SMI
      }
    }
  }
  __syncwarp();
#pragma unroll
  for (int j = 0; j < SMI; j++) {
    const int e = j * 32 + lane;
    if (e < wcnt) d[(long)s_start[warp][e + e / SMI] + ix[j]] = v[j];
  }
}
template <class T> void segscatter(T *d, const T *s, const int *idx, const SegView &sv, const char *name) {
  if (sv.n <= 0 || sv.m <= 0) return;
  const long per = (long)SMB * SMI;
  k_segscatter<T><<<(int)((sv.n + per - 1) / per), SMB, 0, stream()>>>(d, s, idx, sv);
  launch_check(name);
}

template <class TT> struct DisMap {  // d[k] = v[seg(k)]
  typedef TT T;
  static constexpr bool AUX = false, GATHER = false;
  T *d; const T *v; const int *aux;
  __device__ long long token(int, int s, int, int) const { return s; }
  __device__ T fetch(long long s) const { return __ldg(v + s); }
};
struct IndMap {  // d[k] = init[s] + stride[s] * (k - start)
  typedef int T;
  static constexpr bool AUX = false, GATHER = false;
  int *d; const int *init; const int *stride; const int *aux;
  __device__ long long token(int k, int s, int start, int) const {
    return (int)((unsigned)__ldg(init + s) + (unsigned)__ldg(stride + s) * (unsigned)(k - start));
  }
  __device__ int fetch(long long v) const { return (int)v; }
};
template <class TT> struct BPermMap {  // d[k] = s[off_s[seg_d(k)] + i[k]], as many source as dest segments
  typedef TT T;
  static constexpr bool AUX = true, GATHER = true;
  T *d; const T *src; const int *off_s; const int *aux;
  __device__ long long token(int, int s, int, int i) const { return (long long)__ldg(off_s + s) + i; }
  __device__ T fetch(long long at) const { return __ldg(src + at); }
};

// f(i) for i in [0, n)
template <class F> __global__ void __launch_bounds__(VBLOCK) k_each(F f, long n) {
  const long stride = (long)gridDim.x * VBLOCK;
  for (long i = (long)blockIdx.x * VBLOCK + threadIdx.x; i < n; i += stride) f(i);
}
template <class F> void each(F f, long n, const char *name) {
  if (n <= 0) return;
  long g = (n + VBLOCK - 1) / VBLOCK, cap = (long)st().sm_count * 32;
  k_each<F><<<(int)(g < cap ? g : cap), VBLOCK, 0, stream()>>>(f, n);
  launch_check(name);
}

// Unsegmented gather and scatter: PITEMS elements per thread with all their
// index loads, then all their data accesses, in flight together (random
// accesses are latency-bound; one element per thread leaves HBM idle).
constexpr int GITEMS = 8;
template <class T>
__global__ void __launch_bounds__(VBLOCK) k_gather(T *__restrict__ d, const T *__restrict__ s,
                                                   const int *__restrict__ idx, long n) {
  const long i0 = (long)blockIdx.x * (VBLOCK * GITEMS) + threadIdx.x;
  int ix[GITEMS];
  T v[GITEMS];
#pragma unroll
  for (int u = 0; u < GITEMS; u++) {
    const long i = i0 + (long)u * VBLOCK;
    ix[u] = i < n ? __ldcs(idx + i) : 0;
  }
#pragma unroll
  for (int u = 0; u < GITEMS; u++)
    if (i0 + (long)u * VBLOCK < n) v[u] = __ldg(s + ix[u]);
#pragma unroll
  for (int u = 0; u < GITEMS; u++) {
    const long i = i0 + (long)u * VBLOCK;
    if (i < n) __stcs(d + i, v[u]);
  }
}
template <class T>
__global__ void __launch_bounds__(VBLOCK) k_scatter(T *__restrict__ d, const T *__restrict__ s,
                                                    const int *__restrict__ idx, long n) {
  const long i0 = (long)blockIdx.x * (VBLOCK * GITEMS) + threadIdx.x;
  int ix[GITEMS];
  T v[GITEMS];
#pragma unroll
  for (int u = 0; u < GITEMS; u++) {
    const long i = i0 + (long)u * VBLOCK;
    if (i < n) { ix[u] = __ldcs(idx + i); v[u] = __ldcs(s + i); }
  }
#pragma unroll
  for (int u = 0; u < GITEMS; u++)
    if (i0 + (long)u * VBLOCK < n) d[ix[u]] = v[u];
}
template <class T> void gather(T *d, const T *s, const int *idx, long n, const char *name) {
  if (n <= 0) return;
  k_gather<T><<<(int)((n + VBLOCK * GITEMS - 1) / (VBLOCK * GITEMS)), VBLOCK, 0, stream()>>>(d, s, idx, n);
  launch_check(name);
}
// bit moves: int and cvl_bool as 32-bit words, double as 64-bit words
template <class T> struct Bits { typedef unsigned type; };
template <> struct Bits<double> { typedef unsigned long long type; };
// gather from a source of n_src elements: partitioned by source window when
// the source is larger than L2 can serve random reads from
template <class T> void gather_src(T *d, const T *s, const int *idx, int n, int n_src, vec_p scratch,
                                   const char *name) {
  typedef typename Bits<T>::type U;
  if (n <= 0) return;
  if (gather_partitioned_wanted(n_src, n, sizeof(T))) {
    gather_partitioned<U>((U *)d, (const U *)s, idx, n, n_src, scratch);
    return;
  }
  gather<T>(d, s, idx, n, name);
}
template <class T> int gather_units(int n_src, int n) {
  if (n <= 0 || !gather_partitioned_wanted(n_src, n, sizeof(T))) return 0;
  return (int)((gather_partitioned_bytes(n, sizeof(T)) + 7) / 8);
}
template <class T> void scatter(T *d, const T *s, const int *idx, int n, int n_d, vec_p scratch, const char *name) {
  typedef typename Bits<T>::type U;
  if (n <= 0) return;
  if (scatter_partitioned_wanted(n_d, sizeof(T))) {
    scatter_partitioned<U>((U *)d, (const U *)s, idx, n, n_d, scratch);
    return;
  }
  k_scatter<T><<<(int)(((long)n + VBLOCK * GITEMS - 1) / (VBLOCK * GITEMS)), VBLOCK, 0, stream()>>>(d, s, idx, n);
  launch_check(name);
}
template <class T> int scatter_units(int n, int n_d) {
  if (n <= 0 || !scatter_partitioned_wanted(n_d, sizeof(T))) return 0;
  return (int)((scatter_partitioned_bytes(n, sizeof(T)) + 7) / 8);
}

// ----------------------------------------------------------- functors ---
template <class T> struct ExtSeg {  // d[g] = s[off[g] + i[g]]
  T *d; const T *s; const int *i; const int *off;
  __device__ void operator()(long g) const { d[g] = s[(long)off[g] + i[g]]; }
};
template <class T> struct RepSeg {  // d[off[g] + i[g]] = v[g]
  T *d; const int *i; const T *v; const int *off;
  __device__ void operator()(long g) const { d[(long)off[g] + i[g]] = v[g]; }
};
template <class T> struct BPermSeg {  // d[k] = s[off_s[seg_d(k)] + i[k]]
  T *d; const T *s; const int *i; const int *off_s; int m_s;
  __device__ void operator()(int k, int sg, int) const {
    if (sg < m_s) d[k] = __ldg(s + (long)__ldg(off_s + sg) + __ldg(i + k));
  }
};
template <class T> struct FPerm {  // if f[k]: d[i[k]] = s[k]
  T *d; const T *s; const int *i; const int *f;
  __device__ void operator()(long k) const { if (__ldg(f + k)) d[__ldg(i + k)] = __ldcs(s + k); }
};
template <class T> struct FPermSeg {  // if f[k]: d[off_d[seg_s(k)] + i[k]] = s[k]
  T *d; const T *s; const int *i; const int *f; const int *off_d; int m_d;
  __device__ void operator()(int k, int sg, int) const {
    if (sg < m_d && (f == nullptr || __ldg(f + k)))
      d[(long)__ldg(off_d + sg) + __ldg(i + k)] = __ldcs(s + k);
  }
};
// ------------------------------------------------ repeated destinations ---
// The serial CVL's scatters with a default or flags (dpe_*, fpm_*, dfp_*;
// nesl/cvl/serial/vecops.c) write element by element, so where elements
// share a destination the last one's value stays.  NESL's library relies on
// some value winning (remove_duplicates, union and intersection put with
// repeated indices and read back which one won) and the reference's test
// suite checks the serial answer.  Here the scatter itself lets any writer
// win; a pass before it marks every destination in a bitmap (atomicOr; the
// bitmap is n_d / 8 bytes, so it stays in L2) and raises a flag when one is
// marked twice.  Only then do the gated passes after the scatter run: each
// destination's largest source position (atomicMax), then a rewrite of the
// destinations from their last writers.
struct LwMem {
  unsigned *bits, *flag;  // destination bitmap; flag word (+1: spare)
  int *win;               // last writer per destination
  int *gd;                // global destinations (segmented forms)
  char *rest;             // what follows (the scatter's own scratch)
};
inline size_t lw_bytes(long n_s, long n_d, bool seg) {
  return align_up((size_t)(n_d + 31) / 32 * 4 + 16, 256) + align_up((size_t)n_d * 4, 256) +
         (seg ? align_up((size_t)n_s * 4, 256) : 0) + 256;
}
inline LwMem lw_carve(void *raw, long n_s, long n_d, bool seg) {
  char *m = (char *)align_up((size_t)raw, 256);
  LwMem L;
  const size_t nb = (size_t)(n_d + 31) / 32 * 4;
  L.bits = (unsigned *)m;
  L.flag = (unsigned *)(m + nb);
  m += align_up(nb + 16, 256);
  L.win = (int *)m;
  m += align_up((size_t)n_d * 4, 256);
  L.gd = seg ? (int *)m : nullptr;
  if (seg) m += align_up((size_t)n_s * 4, 256);
  L.rest = m;
  return L;
}
__device__ __forceinline__ bool lw_gate(const unsigned *flag) { return *(const volatile unsigned *)flag != 0; }
__device__ __forceinline__ bool lw_mark(unsigned *bits, long g) {  // true if g was marked before
  const unsigned b = 1u << (g & 31);
  return (atomicOr(bits + (g >> 5), b) & b) != 0;
}
// Destinations that strictly ascend cannot repeat: a streaming check sets
// *need when they might (an index out of [0, n_d), or not above the one
// before it), and only then does the bitmap pass run -- a quicksort's
// DPERMUTEs ascend, and the bitmap's random atomics were most of their
// cost.  One vote and at most one atomic per warp.
__global__ void __launch_bounds__(VBLOCK) k_lw_ascent(const int *__restrict__ i, long n, long n_d, unsigned *need) {
  bool bad = false;
  const long stride = (long)gridDim.x * VBLOCK;
  for (long k = (long)blockIdx.x * VBLOCK + threadIdx.x; k < n; k += stride) {
    const int g = __ldg(i + k);
    // the predecessor's load usually hits the line just read by the lane before
    if (g < 0 || g >= n_d || (k > 0 && g <= __ldg(i + k - 1))) bad = true;
  }
  if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(need, 1u);
}
// The segmented form: within every source segment the local indices
// strictly ascend and lie inside the matching destination segment (the
// segments' destination ranges are disjoint and in order, so the global
// destinations ascend too).
__global__ void __launch_bounds__(VBLOCK) k_lw_ascent_seg(const int *__restrict__ i, SegView sv,
                                                          const int *__restrict__ off_d, int m_d, unsigned *need) {
  bool bad = false;
  const long k0 = ((long)blockIdx.x * VBLOCK + threadIdx.x) * SITEMS;
  if (k0 < sv.n) {
    const int cnt = (int)min((long)SITEMS, (long)sv.n - k0);
    int s = seg_of(sv, (int)k0);
    int start = __ldg(sv.off + s), end = __ldg(sv.off + s + 1);
    int len_d = s < m_d ? __ldg(off_d + s + 1) - __ldg(off_d + s) : 0;
    int prev = (int)k0 > start ? __ldg(i + k0 - 1) : -1;
    for (int q = 0; q < cnt; q++) {
      const int k = (int)k0 + q;
      while (k >= end) {
        ++s; start = end; end = __ldg(sv.off + s + 1);
        len_d = s < m_d ? __ldg(off_d + s + 1) - __ldg(off_d + s) : 0;
        prev = -1;
      }
      const int g = __ldg(i + k);
      if (s < m_d && (g < 0 || g >= len_d || g <= prev)) bad = true;
      prev = g;
    }
  }
  if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(need, 1u);
}
// destinations i[k] of the elements whose flag is set (all when f is null);
// with `need`, only when *need is set
__global__ void __launch_bounds__(VBLOCK) k_lw_detect(const int *__restrict__ i, const int *__restrict__ f, long n,
                                                      long n_d, unsigned *bits, unsigned *flag,
                                                      const unsigned *need) {
  if (need && !lw_gate(need)) return;
  bool dup = false;
  const long stride = (long)gridDim.x * VBLOCK;
  for (long k = (long)blockIdx.x * VBLOCK + threadIdx.x; k < n; k += stride) {
    if (f && !__ldg(f + k)) continue;
    const long g = __ldg(i + k);
    if (g >= 0 && g < n_d && lw_mark(bits, g)) dup = true;
  }
  if (dup) atomicOr(flag, 1u);
}
__global__ void __launch_bounds__(VBLOCK) k_lw_fill(int *win, long n_d, const unsigned *flag) {
  if (!lw_gate(flag)) return;
  const long stride = (long)gridDim.x * VBLOCK;
  for (long j = (long)blockIdx.x * VBLOCK + threadIdx.x; j < n_d; j += stride) win[j] = -1;
}
__global__ void __launch_bounds__(VBLOCK) k_lw_max(const int *__restrict__ i, const int *__restrict__ f, long n,
                                                   long n_d, int *win, const unsigned *flag) {
  if (!lw_gate(flag)) return;
  const long stride = (long)gridDim.x * VBLOCK;
  for (long k = (long)blockIdx.x * VBLOCK + threadIdx.x; k < n; k += stride) {
    if (f && !__ldg(f + k)) continue;
    const long g = __ldg(i + k);
    if (g >= 0 && g < n_d) atomicMax(win + g, (int)k);
  }
}
template <class T>
__global__ void __launch_bounds__(VBLOCK) k_lw_write(T *d, const T *__restrict__ s, const int *__restrict__ i,
                                                     const int *__restrict__ f, long n, long n_d,
                                                     const int *__restrict__ win, const unsigned *flag) {
  if (!lw_gate(flag)) return;
  const long stride = (long)gridDim.x * VBLOCK;
  for (long k = (long)blockIdx.x * VBLOCK + threadIdx.x; k < n; k += stride) {
    if (f && !__ldg(f + k)) continue;
    const long g = __ldg(i + k);
    if (g >= 0 && g < n_d && __ldg(win + g) == (int)k) d[g] = s[k];
  }
}
// the segmented forms: the destination of k is off_d[segment of k] + i[k]
struct LwDetectSeg {
  const int *i; const int *f; const int *off_d; int m_d; long n_d; unsigned *bits; unsigned *flag;
  __device__ void operator()(int k, int sg, int) const {
    if (sg < m_d && (f == nullptr || __ldg(f + k))) {
      const long g = (long)__ldg(off_d + sg) + __ldg(i + k);
      if (g >= 0 && g < n_d && lw_mark(bits, g)) atomicOr(flag, 1u);
    }
  }
};
struct LwDestSeg {  // gd[k] = the global destination, or -1 (no write)
  const int *i; const int *f; const int *off_d; int m_d; int *gd;
  __device__ void operator()(int k, int sg, int) const {
    gd[k] = (sg < m_d && (f == nullptr || __ldg(f + k))) ? __ldg(off_d + sg) + __ldg(i + k) : -1;
  }
};
template <class F>
__global__ void __launch_bounds__(VBLOCK) k_segwalk_gated(F f, SegView sv, const unsigned *flag) {
  if (!lw_gate(flag)) return;
  long k0 = ((long)blockIdx.x * VBLOCK + threadIdx.x) * SITEMS;
  if (k0 >= sv.n) return;
  int cnt = (int)min((long)SITEMS, (long)sv.n - k0);
  int s = seg_of(sv, (int)k0);
  int end = __ldg(sv.off + s + 1);
  for (int q = 0; q < cnt; q++) {
    int k = (int)k0 + q;
    while (k >= end) { ++s; end = __ldg(sv.off + s + 1); }
    f(k, s, 0);
  }
}
inline int lw_grid(long n) {
  long g = (n + VBLOCK - 1) / VBLOCK, cap = (long)st().sm_count * 16;
  return (int)(g < 1 ? 1 : (g < cap ? g : cap));
}
// before the scatter: clear the bitmap and flags (flag[0]: some destination
// repeats; flag[1]: the destinations may repeat), mark the destinations
// unless they strictly ascend (forms without flags)
inline void lw_detect(const LwMem &L, const int *i, const int *f, long n, long n_d) {
  GCVL_CK(cudaMemsetAsync(L.bits, 0, (size_t)(n_d + 31) / 32 * 4 + 16, stream()));
  if (n <= 0) return;
  unsigned *need = nullptr;
  if (!f) {
    need = L.flag + 1;
    k_lw_ascent<<<lw_grid(n), VBLOCK, 0, stream()>>>(i, n, n_d, need);
    launch_check("k_lw_ascent");
  }
  k_lw_detect<<<lw_grid(n), VBLOCK, 0, stream()>>>(i, f, n, n_d, L.bits, L.flag, need);
  launch_check("k_lw_detect");
}
inline void lw_detect_seg(const LwMem &L, const int *i, const int *f, const SegView &ss, const SegView &sdd) {
  GCVL_CK(cudaMemsetAsync(L.bits, 0, (size_t)(sdd.n + 31) / 32 * 4 + 16, stream()));
  const LwDetectSeg det{i, f, sdd.off, sdd.m, (long)sdd.n, L.bits, L.flag};
  if (f || ss.n <= 0 || ss.m <= 0) {
    segwalk(det, ss, "k_lw_detect_seg");
    return;
  }
  const int grid = grid_for(((long)ss.n + SITEMS - 1) / SITEMS, VBLOCK);
  k_lw_ascent_seg<<<grid, VBLOCK, 0, stream()>>>(i, ss, sdd.off, sdd.m, L.flag + 1);
  launch_check("k_lw_ascent_seg");
  k_segwalk_gated<<<grid, VBLOCK, 0, stream()>>>(det, ss, L.flag + 1);
  launch_check("k_lw_detect_seg");
}
// after the scatter: the last writer of every destination, where some repeat
template <class T> void lw_fix(T *d, const T *s, const LwMem &L, const int *i, const int *f, long n, long n_d) {
  if (n <= 0 || n_d <= 0) return;
  k_lw_fill<<<lw_grid(n_d), VBLOCK, 0, stream()>>>(L.win, n_d, L.flag);
  launch_check("k_lw_fill");
  k_lw_max<<<lw_grid(n), VBLOCK, 0, stream()>>>(i, f, n, n_d, L.win, L.flag);
  launch_check("k_lw_max");
  k_lw_write<T><<<lw_grid(n), VBLOCK, 0, stream()>>>(d, s, i, f, n, n_d, L.win, L.flag);
  launch_check("k_lw_write");
}
template <class T> void lw_fix_seg(T *d, const T *s, const LwMem &L, const int *i, const int *f, const SegView &ss,
                                   const SegView &sdd) {
  if (ss.n <= 0 || ss.m <= 0) return;
  k_segwalk_gated<<<grid_for(((long)ss.n + SITEMS - 1) / SITEMS, VBLOCK), VBLOCK, 0, stream()>>>(
      LwDestSeg{i, f, sdd.off, sdd.m, L.gd}, ss, L.flag);
  launch_check("k_lw_dest_seg");
  lw_fix<T>(d, s, L, L.gd, nullptr, ss.n, sdd.n);
}

template <class T> struct BFPerm {  // d[k] = f[k] ? s[i[k]] : 0
  T *d; const T *s; const int *i; const int *f;
  __device__ void operator()(long k) const { d[k] = __ldg(f + k) ? __ldg(s + __ldg(i + k)) : (T)0; }
};
template <class T> struct BFPermSeg {  // d[k] = f[k] ? s[off_s[seg_d(k)] + i[k]] : 0
  T *d; const T *s; const int *i; const int *f; const int *off_s; int m_s;
  __device__ void operator()(int k, int sg, int) const {
    T v = (T)0;
    if (sg < m_s && __ldg(f + k)) v = __ldg(s + (long)__ldg(off_s + sg) + __ldg(i + k));
    d[k] = v;
  }
};

template <class T> void copy_dev(vec_p d, vec_p s, int n) {
  if (n <= 0 || d == s) return;
  GCVL_CK(cudaMemcpyAsync(d, s, (size_t)n * sizeof(T), cudaMemcpyDeviceToDevice, stream()));
}

// ---------------------------------------------------------------- pack ---
// Stable compaction in one pass: a CTA counts the true flags of its tile,
// gets the number of true flags in earlier tiles by decoupled look-back,
// compacts its kept values in shared memory and writes them as one
// contiguous, coalesced run.
constexpr int PBLOCK = 256, PITEMS = 16, PTILE = PBLOCK * PITEMS;

template <class T>
__global__ void __launch_bounds__(PBLOCK) k_pack(T *__restrict__ d, const T *__restrict__ s,
                                                const int *__restrict__ f, int n, LookbackMem lb,
                                                unsigned *status, int spin_limit) {
  constexpr int PE = 32;  // padding period of the int staging buffer
  __shared__ int s_rank[PTILE + PTILE / PE];
  __shared__ T s_val[PTILE];
  __shared__ int s_wsum[PBLOCK / 32];
  __shared__ int s_prefix, s_count;
  __shared__ unsigned s_tile;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) s_tile = atomicAdd(lb.counter, 1u);
  __syncthreads();
  const int tile = (int)s_tile;
  const long base = (long)tile * PTILE;
  const int valid = (int)min((long)PTILE, (long)n - base);

  // values: coalesced striped loads issued first, kept in registers until
  // their ranks are known (so their latency overlaps the ranking)
  T vals[PITEMS];
#pragma unroll
  for (int j = 0; j < PITEMS; j++) {
    int e = j * PBLOCK + tid;
    if (e < valid) vals[j] = __ldcs(s + base + e);
  }
  // flags: coalesced striped loads, transposed to 16 consecutive per thread
  const int wbase = warp * 32 * PITEMS;
#pragma unroll
  for (int j = 0; j < PITEMS; j++) {
    int e = wbase + j * 32 + lane;
    s_rank[e + e / PE] = (e < valid) ? (__ldcs(f + base + e) != 0) : 0;
  }
  __syncwarp();
  unsigned bits = 0;
#pragma unroll
  for (int i = 0; i < PITEMS; i++) {
    int e = tid * PITEMS + i;
    bits |= (unsigned)s_rank[e + e / PE] << i;
  }
  // exclusive scan of the per-thread counts across the CTA
  int c = __popc(bits), incl = c;
#pragma unroll
  for (int dd = 1; dd < 32; dd <<= 1) {
    int o = shfl_up(incl, dd);
    if (lane >= dd) incl += o;
  }
  if (lane == 31) s_wsum[warp] = incl;
  __syncthreads();
  int wpre = 0, total = 0;
#pragma unroll
  for (int w = 0; w < PBLOCK / 32; w++) {
    int v = s_wsum[w];
    if (w < warp) wpre += v;
    total += v;
  }
  int r = wpre + incl - c;
  // rank of every element within the tile's output (-1 when dropped)
#pragma unroll
  for (int i = 0; i < PITEMS; i++) {
    int e = tid * PITEMS + i;
    s_rank[e + e / PE] = ((bits >> i) & 1u) ? r++ : -1;
  }

  // decoupled look-back over tile counts (int add, no segments)
  if (warp == 0) {
    if (lane == 0) lb_publish(lb.word + tile, tile == 0 ? TS_INC : TS_AGG, (unsigned long long)(unsigned)total);
    int P = 0;
    if (tile > 0) {
      P = lookback_prefix<AddZ>(lb.word, tile, status, spin_limit);
      if (lane == 0) lb_publish(lb.word + tile, TS_INC, (unsigned long long)(unsigned)(P + total));
    }
    if (lane == 0) { s_prefix = (int)P; s_count = total; }
  }
  __syncthreads();
  // values: coalesced striped loads, placed at their rank in shared memory
#pragma unroll
  for (int j = 0; j < PITEMS; j++) {
    int e = j * PBLOCK + tid;
    int rk = e < valid ? s_rank[e + e / PE] : -1;
    if (rk >= 0) s_val[rk] = vals[j];
  }
  __syncthreads();
  const long out0 = s_prefix;
  const int cnt = s_count;
  for (int e = tid; e < cnt; e += PBLOCK) d[out0 + e] = s_val[e];
}

// Pack of long vectors in two passes, no tile waiting for another (at large
// n the one-pass kernel's look-back chain, not HBM, bounds it).  Pass 1
// reads the flags once, writes them as a bit mask (element k: bit k&31 of
// word k>>5) and every tile's count of true flags; an exclusive +-scan of
// the counts gives each tile its output offset; pass 2 reads the mask (one
// bit per element instead of the 4-byte flag) and the values, and writes
// each tile's kept values as one coalesced run.
constexpr int PACK_TWO_PASS_TILES = 64;
constexpr int PWORDS = PTILE / 32;  // mask words per tile

__global__ void __launch_bounds__(PBLOCK) k_pack_count(const int *__restrict__ f, int n,
                                                      unsigned *__restrict__ bits, int *__restrict__ cnt) {
  __shared__ unsigned s_bits[PWORDS];
  __shared__ int s_c[PBLOCK / 32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const long base = (long)blockIdx.x * PTILE;
  const int valid = (int)min((long)PTILE, (long)n - base);
  int fl[PITEMS];
#pragma unroll
  for (int j = 0; j < PITEMS; j++) {
    const int e = j * PBLOCK + tid;
    fl[j] = e < valid ? __ldcs(f + base + e) : 0;
  }
  int c = 0;
#pragma unroll
  for (int j = 0; j < PITEMS; j++) {
    // elements j*PBLOCK + warp*32 + lane: mask word j*8 + warp of the tile
    const unsigned b = __ballot_sync(0xffffffffu, fl[j] != 0);
    if (lane == 0) s_bits[j * (PBLOCK / 32) + warp] = b;
    c += __popc(b);
  }
  if (lane == 0) s_c[warp] = c;
  __syncthreads();
  const int nw = (valid + 31) >> 5;
  if (tid < nw) bits[(base >> 5) + tid] = s_bits[tid];
  if (tid == 0) {
    int t = 0;
#pragma unroll
    for (int w = 0; w < PBLOCK / 32; w++) t += s_c[w];
    cnt[blockIdx.x] = t;
  }
}

template <class T>
__global__ void __launch_bounds__(PBLOCK) k_pack_place(T *__restrict__ d, const T *__restrict__ s,
                                                      const unsigned *__restrict__ bits,
                                                      const int *__restrict__ offs, int n) {
  __shared__ T s_val[PTILE];
  __shared__ unsigned s_word[PWORDS];
  __shared__ int s_wpre[PWORDS + 1];
  __shared__ int s_ws[PWORDS / 32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const long base = (long)blockIdx.x * PTILE;
  const int valid = (int)min((long)PTILE, (long)n - base);
  // the values' loads first, kept in registers while the mask is ranked
  T vals[PITEMS];
#pragma unroll
  for (int j = 0; j < PITEMS; j++) {
    const int e = j * PBLOCK + tid;
    if (e < valid) vals[j] = __ldcs(s + base + e);
  }
  const long out0 = __ldg(offs + blockIdx.x);
  // exclusive prefix of the words' popcounts (threads 0..PWORDS-1, one word each)
  if (tid < PWORDS) {
    const int nw = (valid + 31) >> 5;
    const unsigned w = tid < nw ? __ldg(bits + (base >> 5) + tid) : 0u;
    const int c = __popc(w);
    int incl = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int x = shfl_up(incl, o);
      if (lane >= o) incl += x;
    }
    if (lane == 31) s_ws[warp] = incl;
    s_word[tid] = w;
    s_wpre[tid] = incl - c;
  }
  __syncthreads();
  if (tid < PWORDS) {
    int p = 0;
#pragma unroll
    for (int w = 0; w < PWORDS / 32; w++) if (w < warp) p += s_ws[w];
    s_wpre[tid] += p;
    if (tid == PWORDS - 1) s_wpre[PWORDS] = p + s_ws[warp];
  }
  __syncthreads();
  const unsigned lt = (1u << lane) - 1u;
#pragma unroll
  for (int j = 0; j < PITEMS; j++) {
    const int e = j * PBLOCK + tid;
    const int wi = e >> 5;  // == j * 8 + warp: one word per warp and step
    const unsigned w = s_word[wi];
    if (e < valid && ((w >> lane) & 1u)) s_val[s_wpre[wi] + __popc(w & lt)] = vals[j];
  }
  __syncthreads();
  const int total = s_wpre[PWORDS];
  for (int e = tid; e < total; e += PBLOCK) __stcs(d + out0 + e, s_val[e]);
}

struct PackLayout { size_t bits, cnt, offs, scan, total; };
inline PackLayout pack_layout(int n) {
  const int tiles = ceil_div(n, PTILE);
  PackLayout L;
  size_t o = 0;
  auto take = [&](size_t bytes) { size_t at = o; o += align_up(bytes, 256); return at; };
  L.bits = take((size_t)ceil_div(n, 32) * 4);
  L.cnt = take((size_t)tiles * 4);
  L.offs = take((size_t)tiles * 4);
  L.scan = take((size_t)add_suz_scratch(tiles) * 8);
  L.total = o;
  return L;
}

template <class T> void pack(vec_p d, vec_p s, vec_p f, int n, vec_p scratch, const char *name) {
  ensure_init();
  State &S = st();
  if (n <= 0) return;
  int tiles = ceil_div(n, PTILE);
  if (tiles >= PACK_TWO_PASS_TILES) {
    const PackLayout L = pack_layout(n);
    char *mem = (char *)scratch_or_work(scratch, L.total);
    if (!mem) return;
    unsigned *bits = (unsigned *)(mem + L.bits);
    int *cnt = (int *)(mem + L.cnt), *offs = (int *)(mem + L.offs);
    k_pack_count<<<tiles, PBLOCK, 0, S.stream>>>((const int *)f, n, bits, cnt);
    launch_check(name);
    add_suz(offs, cnt, tiles, mem + L.scan);
    k_pack_place<T><<<tiles, PBLOCK, 0, S.stream>>>((T *)d, (const T *)s, bits, offs, n);
    launch_check(name);
    return;
  }
  void *mem = scratch_or_work(scratch, lookback_bytes(tiles));
  if (!mem) return;
  LookbackMem lb = lookback_carve(mem, tiles);
  GCVL_CK(cudaMemsetAsync(mem, 0, lookback_clear_bytes(tiles), S.stream));
  k_pack<T><<<tiles, PBLOCK, 0, S.stream>>>((T *)d, (const T *)s, (const int *)f, n, lb, S.d_status,
                                            S.spin_limit);
  launch_check(name);
}
int pack_units(int n) {
  if (n <= 0) return 0;
  const int tiles = ceil_div(n, PTILE);
  if (tiles >= PACK_TWO_PASS_TILES) return (int)((pack_layout(n).total + 7) / 8);
  return lookback_units(tiles);
}

}  // namespace gcvl

using namespace gcvl;

#define META1(NAME, INPL)                                                     \
  GCVL_EXPORT int NAME##_scratch(int len) { (void)len; return 0; }           \
  GCVL_EXPORT unsigned NAME##_inplace(void) { return INPL; }
#define META_SEG(NAME, INPL)                                                  \
  GCVL_EXPORT int NAME##_scratch(int n, int m) { (void)n; (void)m; return 0; } \
  GCVL_EXPORT unsigned NAME##_inplace(void) { return INPL; }
#define META2(NAME, INPL)                                                     \
  GCVL_EXPORT int NAME##_scratch(int a, int b) { (void)a; (void)b; return 0; } \
  GCVL_EXPORT unsigned NAME##_inplace(void) { return INPL; }
#define META_SEG2(NAME, INPL)                                                 \
  GCVL_EXPORT int NAME##_scratch(int a, int b, int c, int e) {                \
    (void)a; (void)b; (void)c; (void)e; return 0; }                          \
  GCVL_EXPORT unsigned NAME##_inplace(void) { return INPL; }

// ------------------------------------------------ extract / replace ---
// ext_vu* / rep_vu* move one element (vprims.c:207-262); extract returns to
// the host, so it synchronises.
#define EXT_REP(L, T)                                                                  \
  GCVL_EXPORT T ext_vu##L(vec_p v, int i, int len, vec_p scratch) {                    \
    (void)len; (void)scratch; ensure_init();                                          \
    T out = (T)0;                                                                      \
    GCVL_CK(cudaMemcpyAsync(st().h_small, (T *)v + i, sizeof(T), cudaMemcpyDeviceToHost, \
                            stream()));                                                \
    GCVL_CK(cudaStreamSynchronize(stream()));                                          \
    memcpy(&out, st().h_small, sizeof(T));                                             \
    return out;                                                                        \
  }                                                                                    \
  META1(ext_vu##L, INPLACE_NONE)                                                       \
  GCVL_EXPORT void ext_ve##L(vec_p d, vec_p s, vec_p i, vec_p sd, int n, int m,        \
                             vec_p scratch) {                                          \
    (void)scratch; ensure_init();                                                     \
    SegView sv = seg_view(sd, n, m);                                                   \
    each(ExtSeg<T>{(T *)d, (const T *)s, (const int *)i, sv.off}, m, "ext_ve" #L);     \
  }                                                                                    \
  META_SEG(ext_ve##L, INPLACE_2)                                                       \
  GCVL_EXPORT void rep_ve##L(vec_p d, vec_p s, vec_p v, vec_p sd, int n, int m,        \
                             vec_p scratch) {                                          \
    (void)scratch; ensure_init();                                                     \
    SegView sv = seg_view(sd, n, m);                                                   \
    each(RepSeg<T>{(T *)d, (const int *)s, (const T *)v, sv.off}, m, "rep_ve" #L);     \
  }                                                                                    \
  META_SEG(rep_ve##L, INPLACE_NONE)                                                    \
  GCVL_EXPORT void dis_ve##L(vec_p d, vec_p v, vec_p sd, int n, int m, vec_p scratch) { \
    (void)scratch; ensure_init();                                                     \
    segmap(DisMap<T>{(T *)d, (const T *)v, nullptr}, seg_view(sd, n, m), "dis_ve" #L); \
  }                                                                                    \
  META_SEG(dis_ve##L, INPLACE_NONE)
EXT_REP(z, int)
EXT_REP(b, cvl_bool)
EXT_REP(d, double)

// Replace writes one element from the host value (vprims.c:236-262).
GCVL_EXPORT void rep_vuz(vec_p v, int i, int val, int len, vec_p scratch) {
  (void)len; (void)scratch; ensure_init();
  GCVL_CK(cudaMemcpyAsync((int *)v + i, &val, 4, cudaMemcpyHostToDevice, stream()));
  GCVL_CK(cudaStreamSynchronize(stream()));
}
META1(rep_vuz, INPLACE_NONE)
GCVL_EXPORT void rep_vub(vec_p v, int i, cvl_bool val, int len, vec_p scratch) {
  (void)len; (void)scratch; ensure_init();
  int b = val != 0;
  GCVL_CK(cudaMemcpyAsync((int *)v + i, &b, 4, cudaMemcpyHostToDevice, stream()));
  GCVL_CK(cudaStreamSynchronize(stream()));
}
META1(rep_vub, INPLACE_NONE)
GCVL_EXPORT void rep_vud(vec_p v, int i, double val, int len, vec_p scratch) {
  (void)len; (void)scratch; ensure_init();
  GCVL_CK(cudaMemcpyAsync((double *)v + i, &val, 8, cudaMemcpyHostToDevice, stream()));
  GCVL_CK(cudaStreamSynchronize(stream()));
}
META1(rep_vud, INPLACE_NONE)

// Segmented index (library.c:28-49).
GCVL_EXPORT void ind_lez(vec_p d, vec_p init, vec_p stride, vec_p sd, int n, int m, vec_p scratch) {
  (void)scratch; ensure_init();
  segmap(IndMap{(int *)d, (const int *)init, (const int *)stride, nullptr}, seg_view(sd, n, m), "ind_lez");
}
META_SEG(ind_lez, INPLACE_NONE)

// ------------------------------------------------------------- permutes ---
#define PERMS(L, T)                                                                     \
  GCVL_EXPORT void smp_pu##L(vec_p d, vec_p s, vec_p i, int len, vec_p scratch) {       \
    ensure_init();                                                                      \
    scatter<T>((T *)d, (const T *)s, (const int *)i, len, len, scratch, "smp_pu" #L);   \
  }                                                                                     \
  GCVL_EXPORT int smp_pu##L##_scratch(int len) { return scatter_units<T>(len, len); }   \
  GCVL_EXPORT unsigned smp_pu##L##_inplace(void) { return INPLACE_NONE; }               \
  GCVL_EXPORT void smp_pe##L(vec_p d, vec_p s, vec_p i, vec_p sd, int n, int m,         \
                             vec_p scratch) {                                           \
    ensure_init();                                                                      \
    if (m == 1) { scatter<T>((T *)d, (const T *)s, (const int *)i, n, n, scratch, "smp_pe" #L); return; } \
    segscatter<T>((T *)d, (const T *)s, (const int *)i, seg_view(sd, n, m), "smp_pe" #L); \
  }                                                                                     \
  GCVL_EXPORT int smp_pe##L##_scratch(int n, int m) { return m == 1 ? scatter_units<T>(n, n) : 0; } \
  GCVL_EXPORT unsigned smp_pe##L##_inplace(void) { return INPLACE_NONE; }               \
  GCVL_EXPORT void bck_pu##L(vec_p d, vec_p s, vec_p i, int s_len, int d_len,           \
                             vec_p scratch) {                                           \
    ensure_init();                                                                      \
    gather_src<T>((T *)d, (const T *)s, (const int *)i, d_len, s_len, scratch, "bck_pu" #L); \
  }                                                                                     \
  GCVL_EXPORT int bck_pu##L##_scratch(int s_len, int d_len) { return gather_units<T>(s_len, d_len); } \
  GCVL_EXPORT unsigned bck_pu##L##_inplace(void) { return INPLACE_2; }                  \
  GCVL_EXPORT void bck_pe##L(vec_p d, vec_p s, vec_p i, vec_p sd_s, int n_s, int m_s,   \
                             vec_p sd_d, int n_d, int m_d, vec_p scratch) {             \
    ensure_init();                                                                      \
    if (m_s == 1) { gather_src<T>((T *)d, (const T *)s, (const int *)i, n_d, n_s, scratch, "bck_pe" #L); return; } \
    SegView ss = seg_view(sd_s, n_s, m_s);                                              \
    if (m_s == m_d)                                                                     \
      segmap(BPermMap<T>{(T *)d, (const T *)s, ss.off, (const int *)i},                  \
             seg_view(sd_d, n_d, m_d), "bck_pe" #L);                                    \
    else                                                                                \
      segwalk(BPermSeg<T>{(T *)d, (const T *)s, (const int *)i, ss.off, m_s},               \
              seg_view(sd_d, n_d, m_d), "bck_pe" #L);                                   \
  }                                                                                     \
  GCVL_EXPORT int bck_pe##L##_scratch(int n_s, int m_s, int n_d, int m_d) {              \
    (void)m_d; return m_s == 1 ? gather_units<T>(n_s, n_d) : 0;                          \
  }                                                                                     \
  GCVL_EXPORT unsigned bck_pe##L##_inplace(void) { return INPLACE_2; }                  \
  GCVL_EXPORT void fpm_pu##L(vec_p d, vec_p s, vec_p i, vec_p f, int len_src,           \
                             int len_dest, vec_p scratch) {                             \
    ensure_init();                                                                      \
    if (len_src <= 0) return;                                                           \
    void *mem = scratch_or_work(scratch, lw_bytes(len_src, len_dest, false));           \
    if (!mem) return;                                                                   \
    const LwMem W = lw_carve(mem, len_src, len_dest, false);                            \
    lw_detect(W, (const int *)i, (const int *)f, len_src, len_dest);                    \
    each(FPerm<T>{(T *)d, (const T *)s, (const int *)i, (const int *)f}, len_src, "fpm_pu" #L); \
    lw_fix<T>((T *)d, (const T *)s, W, (const int *)i, (const int *)f, len_src, len_dest); \
  }                                                                                     \
  GCVL_EXPORT int fpm_pu##L##_scratch(int len_src, int len_dest) {                      \
    return (int)((lw_bytes(len_src, len_dest, false) + 7) / 8);                         \
  }                                                                                     \
  GCVL_EXPORT unsigned fpm_pu##L##_inplace(void) { return INPLACE_NONE; }               \
  GCVL_EXPORT void fpm_pe##L(vec_p d, vec_p s, vec_p i, vec_p f, vec_p sd_s, int n_s,   \
                             int m_s, vec_p sd_d, int n_d, int m_d, vec_p scratch) {    \
    ensure_init();                                                                      \
    if (m_s == 1) { fpm_pu##L(d, s, i, f, n_s, n_d, scratch); return; }                 \
    if (n_s <= 0) return;                                                               \
    void *mem = scratch_or_work(scratch, lw_bytes(n_s, n_d, true));                     \
    if (!mem) return;                                                                   \
    const LwMem W = lw_carve(mem, n_s, n_d, true);                                      \
    SegView sdd = seg_view(sd_d, n_d, m_d), ss = seg_view(sd_s, n_s, m_s);              \
    lw_detect_seg(W, (const int *)i, (const int *)f, ss, sdd);                          \
    segwalk(FPermSeg<T>{(T *)d, (const T *)s, (const int *)i, (const int *)f, sdd.off, m_d}, ss, "fpm_pe" #L); \
    lw_fix_seg<T>((T *)d, (const T *)s, W, (const int *)i, (const int *)f, ss, sdd);    \
  }                                                                                     \
  GCVL_EXPORT int fpm_pe##L##_scratch(int n_s, int m_s, int n_d, int m_d) {             \
    (void)m_d; return (int)((lw_bytes(n_s, n_d, m_s != 1) + 7) / 8);                    \
  }                                                                                     \
  GCVL_EXPORT unsigned fpm_pe##L##_inplace(void) { return INPLACE_NONE; }               \
  GCVL_EXPORT void bfp_pu##L(vec_p d, vec_p s, vec_p i, vec_p f, int len_src,           \
                             int len_dest, vec_p scratch) {                             \
    (void)len_src; (void)scratch; ensure_init();                                        \
    each(BFPerm<T>{(T *)d, (const T *)s, (const int *)i, (const int *)f}, len_dest, "bfp_pu" #L); \
  }                                                                                     \
  META2(bfp_pu##L, INPLACE_NONE)                                                        \
  GCVL_EXPORT void bfp_pe##L(vec_p d, vec_p s, vec_p i, vec_p f, vec_p sd_s, int n_s,   \
                             int m_s, vec_p sd_d, int n_d, int m_d, vec_p scratch) {    \
    (void)scratch; ensure_init();                                                       \
    if (m_s == 1) { bfp_pu##L(d, s, i, f, n_s, n_d, scratch); return; }                 \
    SegView ss = seg_view(sd_s, n_s, m_s);                                              \
    segwalk(BFPermSeg<T>{(T *)d, (const T *)s, (const int *)i, (const int *)f, ss.off, m_s}, \
            seg_view(sd_d, n_d, m_d), "bfp_pe" #L);                                     \
  }                                                                                     \
  META_SEG2(bfp_pe##L, INPLACE_NONE)                                                    \
  GCVL_EXPORT void dpe_pu##L(vec_p d, vec_p s, vec_p i, vec_p v, int len_src,           \
                             int len_dest, vec_p scratch) {                             \
    ensure_init();                                                                      \
    copy_dev<T>(d, v, len_dest);                                                        \
    if (len_src <= 0) return;                                                           \
    const size_t lb = lw_bytes(len_src, len_dest, false);                               \
    char *mem = (char *)scratch_or_work(scratch, lb + (size_t)scatter_units<T>(len_src, len_dest) * 8); \
    if (!mem) return;                                                                   \
    const LwMem W = lw_carve(mem, len_src, len_dest, false);                            \
    lw_detect(W, (const int *)i, nullptr, len_src, len_dest);                           \
    scatter<T>((T *)d, (const T *)s, (const int *)i, len_src, len_dest, W.rest, "dpe_pu" #L); \
    lw_fix<T>((T *)d, (const T *)s, W, (const int *)i, nullptr, len_src, len_dest);     \
  }                                                                                     \
  GCVL_EXPORT int dpe_pu##L##_scratch(int len_src, int len_dest) {                      \
    return (int)((lw_bytes(len_src, len_dest, false) + 7) / 8) + scatter_units<T>(len_src, len_dest); \
  }                                                                                     \
  GCVL_EXPORT unsigned dpe_pu##L##_inplace(void) { return INPLACE_3; }                  \
  GCVL_EXPORT void dpe_pe##L(vec_p d, vec_p s, vec_p i, vec_p v, vec_p sd_s, int n_s,   \
                             int m_s, vec_p sd_d, int n_d, int m_d, vec_p scratch) {    \
    ensure_init();                                                                      \
    if (m_s == 1) { dpe_pu##L(d, s, i, v, n_s, n_d, scratch); return; }                 \
    copy_dev<T>(d, v, n_d);                                                             \
    if (n_s <= 0) return;                                                               \
    void *mem = scratch_or_work(scratch, lw_bytes(n_s, n_d, true));                     \
    if (!mem) return;                                                                   \
    const LwMem W = lw_carve(mem, n_s, n_d, true);                                      \
    SegView sdd = seg_view(sd_d, n_d, m_d), ss = seg_view(sd_s, n_s, m_s);              \
    lw_detect_seg(W, (const int *)i, nullptr, ss, sdd);                                 \
    segwalk(FPermSeg<T>{(T *)d, (const T *)s, (const int *)i, nullptr, sdd.off, m_d}, ss, "dpe_pe" #L); \
    lw_fix_seg<T>((T *)d, (const T *)s, W, (const int *)i, nullptr, ss, sdd);           \
  }                                                                                     \
  GCVL_EXPORT int dpe_pe##L##_scratch(int n_s, int m_s, int n_d, int m_d) {             \
    (void)m_d;                                                                          \
    return m_s == 1 ? dpe_pu##L##_scratch(n_s, n_d) : (int)((lw_bytes(n_s, n_d, true) + 7) / 8); \
  }                                                                                     \
  GCVL_EXPORT unsigned dpe_pe##L##_inplace(void) { return INPLACE_3; }                  \
  GCVL_EXPORT void dfp_pu##L(vec_p d, vec_p s, vec_p i, vec_p f, vec_p v, int len_src,  \
                             int len_dest, vec_p scratch) {                             \
    ensure_init();                                                                      \
    copy_dev<T>(d, v, len_dest);                                                        \
    fpm_pu##L(d, s, i, f, len_src, len_dest, scratch);                                  \
  }                                                                                     \
  GCVL_EXPORT int dfp_pu##L##_scratch(int len_src, int len_dest) { return fpm_pu##L##_scratch(len_src, len_dest); } \
  GCVL_EXPORT unsigned dfp_pu##L##_inplace(void) { return INPLACE_4; }                  \
  GCVL_EXPORT void dfp_pe##L(vec_p d, vec_p s, vec_p i, vec_p f, vec_p v, vec_p sd_s,   \
                             int n_s, int m_s, vec_p sd_d, int n_d, int m_d,            \
                             vec_p scratch) {                                           \
    ensure_init();                                                                      \
    copy_dev<T>(d, v, n_d);                                                             \
    if (m_s == 1) fpm_pu##L(d, s, i, f, n_s, n_d, scratch);                             \
    else fpm_pe##L(d, s, i, f, sd_s, n_s, m_s, sd_d, n_d, m_d, scratch);                \
  }                                                                                     \
  GCVL_EXPORT int dfp_pe##L##_scratch(int n_s, int m_s, int n_d, int m_d) {             \
    return fpm_pe##L##_scratch(n_s, m_s, n_d, m_d);                                     \
  }                                                                                     \
  GCVL_EXPORT unsigned dfp_pe##L##_inplace(void) { return INPLACE_4; }                  \
  GCVL_EXPORT void pk2_lu##L(vec_p d, vec_p s, vec_p f, int src_len, int dest_len,      \
                             vec_p scratch) {                                           \
    (void)dest_len; pack<T>(d, s, f, src_len, scratch, "pk2_lu" #L);                    \
  }                                                                                     \
  GCVL_EXPORT int pk2_lu##L##_scratch(int len) { return pack_units(len); }              \
  GCVL_EXPORT unsigned pk2_lu##L##_inplace(void) { return INPLACE_NONE; }               \
  GCVL_EXPORT void pk2_le##L(vec_p d, vec_p s, vec_p f, vec_p sd_s, int n_s, int m_s,   \
                             vec_p sd_d, int n_d, int m_d, vec_p scratch) {             \
    (void)sd_s; (void)m_s; (void)sd_d; (void)n_d; (void)m_d;                            \
    pack<T>(d, s, f, n_s, scratch, "pk2_le" #L);                                        \
  }                                                                                     \
  GCVL_EXPORT int pk2_le##L##_scratch(int a, int b, int c, int e) {                     \
    (void)b; (void)c; (void)e; return pack_units(a);                                    \
  }                                                                                     \
  GCVL_EXPORT unsigned pk2_le##L##_inplace(void) { return INPLACE_NONE; }
PERMS(z, int)
PERMS(b, cvl_bool)
PERMS(d, double)
