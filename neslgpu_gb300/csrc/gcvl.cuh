// gcvl.cuh -- shared definitions of the GB300 CVL library (libcvl_gb300.so).
//
// The library implements the C vector library ABI of NESL's VCODE
// interpreter (nesl/include/cvl.h of Nessie-Compiler/neslgpu) with
// hand-written sm_103a kernels.  vec_p is a raw device pointer (the
// HAS_VOIDP branch of cvl.h:50-53) and sizes are counted in 8-byte units
// (CVL_SIZE_UNIT = sizeof(MAXALIGN) of the serial CVL, facilt.c:92-93).
//
// One host thread, one library stream, calls ordered on that stream.
// Functions that return a scalar to the host synchronise the stream.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <limits.h>
#include <string.h>

// The public header: every export below must match its declaration there.
#include "cvl_gb300.h"

#define GCVL_EXPORT extern "C" __attribute__((visibility("default")))

namespace gcvl {

// ---------------------------------------------------------------- state ---
struct State {
  bool ready = false;
  int device = 0;
  int sm_count = 152;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  unsigned *d_status = nullptr;     // device-side error word (bounded waits)
  void *d_small = nullptr;          // 4 KB device scratch for scalar results
  void *h_small = nullptr;          // 4 KB pinned host mirror
  void *work = nullptr;             // library workspace used when the caller
  size_t work_bytes = 0;            //   passes a NULL scratch vector
  uint64_t rand48 = 0;               // lrand48 state (glibc starts unseeded draws from 0)
  int spin_limit = 1 << 22;         // bounded-wait iteration limit
  int err = 0;
  char msg[256] = {0};
  char fused_lib[1024] = {0};       // fused library named by CVL_init
  bool fused_init_done = false;     // its init() has been given the heap
};
State &st();
void ensure_init();
void set_error(int code, const char *fmt, ...);
bool check_cuda(cudaError_t e, const char *what);
#define GCVL_CK(call) ::gcvl::check_cuda((call), #call)
inline cudaStream_t stream() { return st().stream; }
// Device scratch for a call: the caller's vec_p when given, else the
// library workspace (grown on demand, kept for later calls).
void *scratch_or_work(vec_p scratch, size_t bytes);
void launch_check(const char *what);
// Status word of the no-allocation entry point (scan.cu): whether it has run
// on the current device, and folding its bits into the error state.
bool noalloc_used();
void noalloc_fold_status();

enum ErrorCode {
  GCVL_OK = 0,
  GCVL_ERR_CUDA = 1,
  GCVL_ERR_ARG = 2,
  GCVL_ERR_TIMEOUT = 3,   // a bounded device wait gave up
  GCVL_ERR_NOMEM = 4,
  GCVL_ERR_RANGE = 5,
};
// bits of the device status word
enum : unsigned { DEV_TIMEOUT = 1u, DEV_RANGE = 2u };  // DEV_RANGE: a kernel skipped input it cannot take

inline int ceil_div(long a, long b) { return (int)((a + b - 1) / b); }
inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// ------------------------------------------------------------ operators ---
// The CVL scan/reduce operators with the serial CVL's initial values
// (nesl/cvl/serial/vprims.c:33-49, defins.h:217-228).  init() is the value a
// segment starts from; ident() is a true identity used for padding lanes and
// empty partial results.  apply(a, b) has a = earlier element.
struct AddZ { typedef int T;
  __host__ __device__ static T init() { return 0; }
  __host__ __device__ static T ident() { return 0; }
  __device__ static T apply(T a, T b) { return (T)((unsigned)a + (unsigned)b); } };
struct MulZ { typedef int T;
  __host__ __device__ static T init() { return 1; }
  __host__ __device__ static T ident() { return 1; }
  __device__ static T apply(T a, T b) { return (T)((unsigned)a * (unsigned)b); } };
struct MinZ { typedef int T;
  __host__ __device__ static T init() { return INT_MAX; }
  __host__ __device__ static T ident() { return INT_MAX; }
  __device__ static T apply(T a, T b) { return a < b ? a : b; } };
struct MaxZ { typedef int T;
  __host__ __device__ static T init() { return INT_MIN; }
  __host__ __device__ static T ident() { return INT_MIN; }
  __device__ static T apply(T a, T b) { return a > b ? a : b; } };
struct AndZ { typedef int T;
  __host__ __device__ static T init() { return ~0; }
  __host__ __device__ static T ident() { return ~0; }
  __device__ static T apply(T a, T b) { return a & b; } };
struct IorZ { typedef int T;
  __host__ __device__ static T init() { return 0; }
  __host__ __device__ static T ident() { return 0; }
  __device__ static T apply(T a, T b) { return a | b; } };
struct XorZ { typedef int T;
  __host__ __device__ static T init() { return 0; }
  __host__ __device__ static T ident() { return 0; }
  __device__ static T apply(T a, T b) { return a ^ b; } };
// logical operators on cvl_bool: results are 0/1 whatever the inputs hold
struct AndB { typedef int T;
  __host__ __device__ static T init() { return 1; }
  __host__ __device__ static T ident() { return 1; }
  __device__ static T apply(T a, T b) { return (a != 0) & (b != 0); } };
struct IorB { typedef int T;
  __host__ __device__ static T init() { return 0; }
  __host__ __device__ static T ident() { return 0; }
  __device__ static T apply(T a, T b) { return (a != 0) | (b != 0); } };
struct XorB { typedef int T;
  __host__ __device__ static T init() { return 0; }
  __host__ __device__ static T ident() { return 0; }
  __device__ static T apply(T a, T b) { return (a != 0) ^ (b != 0); } };
// float64: -0.0 is the exact additive identity; min/max use +-inf as
// identity while segments start from the serial CVL's +-1e36 (as float).
struct AddD { typedef double T;
  __host__ __device__ static T init() { return 0.0; }
  __host__ __device__ static T ident() { return -0.0; }
  __device__ static T apply(T a, T b) { return __dadd_rn(a, b); } };
struct MulD { typedef double T;
  __host__ __device__ static T init() { return 1.0; }
  __host__ __device__ static T ident() { return 1.0; }
  __device__ static T apply(T a, T b) { return __dmul_rn(a, b); } };
__host__ __device__ inline double bits_to_double(unsigned long long v) {
  union { unsigned long long l; double d; } u; u.l = v; return u.d;
}
// Order key of a double: signed-integer order equals the double order for
// non-NaN values, with -0.0 and +0.0 equal (as == has them).  Min and max
// compare keys so that they run on the integer pipes, not the FP64 pipe.
__device__ __forceinline__ long long dkey(double x) {
  long long b = __double_as_longlong(x);
  if ((b << 1) == 0) return 0;
  return b ^ ((b >> 63) & 0x7FFFFFFFFFFFFFFFLL);
}
struct MinD { typedef double T;
  __host__ __device__ static T init() { return (double)(float)1.0e36; }
  __host__ __device__ static T ident() { return bits_to_double(0x7FF0000000000000ULL); }
  __device__ static T apply(T a, T b) { return dkey(a) < dkey(b) ? a : b; } };
struct MaxD { typedef double T;
  __host__ __device__ static T init() { return (double)(float)-1.0e36; }
  __host__ __device__ static T ident() { return bits_to_double(0xFFF0000000000000ULL); }
  __device__ static T apply(T a, T b) { return dkey(a) > dkey(b) ? a : b; } };
// pk1_lev counts true flags per segment: an add over (x != 0).
struct CountB { typedef int T;
  __host__ __device__ static T init() { return 0; }
  __host__ __device__ static T ident() { return 0; }
  __device__ static T apply(T a, T b) { return a + b; } };

// ------------------------------------------------------- device helpers ---
template <class T> __device__ __forceinline__ T shfl_up(T v, int d) { return __shfl_up_sync(0xffffffffu, v, d); }
// Lanes of the warp holding the same 8-bit digit as this lane (digit < 0:
// an empty lane, matched by nobody and matching nothing).  Eight ballots
// instead of match.any, whose cost grows with the number of distinct values
// and which runs on a narrow pipe: with 8-bit radix digits almost every lane
// holds a different value.
__device__ __forceinline__ unsigned warp_match8(int digit) {
  unsigned peers = __ballot_sync(0xffffffffu, digit >= 0);
#pragma unroll
  for (int b = 0; b < 8; b++) {
    const unsigned bal = __ballot_sync(0xffffffffu, (digit >> b) & 1);
    peers &= ((digit >> b) & 1) ? bal : ~bal;
  }
  return digit >= 0 ? peers : 0u;
}
template <class T> __device__ __forceinline__ T shfl_down(T v, int d) { return __shfl_down_sync(0xffffffffu, v, d); }
template <class T> __device__ __forceinline__ T shfl_idx(T v, int l) { return __shfl_sync(0xffffffffu, v, l); }

__device__ __forceinline__ unsigned ld_acquire(const unsigned *p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release(unsigned *p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
template <class T> __device__ __forceinline__ void st_relaxed(T *p, T v) {
  if constexpr (sizeof(T) == 8) {
    unsigned long long b; memcpy(&b, &v, 8);
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(b) : "memory");
  } else {
    unsigned b; memcpy(&b, &v, 4);
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(b) : "memory");
  }
}
template <class T> __device__ __forceinline__ T ld_relaxed(const T *p) {
  T v;
  if constexpr (sizeof(T) == 8) {
    unsigned long long b;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(b) : "l"(p) : "memory");
    memcpy(&v, &b, 8);
  } else {
    unsigned b;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(b) : "l"(p) : "memory");
    memcpy(&v, &b, 4);
  }
  return v;
}

// --------------------------------------------------- segment descriptor ---
// Device layout of a segment descriptor (32-bit words, in one vec_p of
// siz_fos(n, m) units):
//   [0, m)                    segment lengths (what len_fos returns)
//   [L0, L0 + m + 1)          offsets: exclusive scan of the lengths, then n
//   [L1, L1 + ng + 1)         granule table: for granule g (elements
//                             g*kGranule...), the segment that holds element
//                             g*kGranule; entry ng holds m
//   [L2, L2 + nb)             head bitmap: bit k set when element k starts a
//                             (non-empty) segment; padded with zero words to a
//                             multiple of 256 words
// with L0 = align4(m), L1 = L0 + align4(m + 1), L2 = L1 + align4(ng + 1),
// ng = ceil(n / kGranule), nb = align256(ceil(n / 32)).
// what a segmented pass produces: scan outputs, one result per segment, or
// segment offsets (the scan of the lengths, in mke_fov)
enum Mode { M_SCAN = 0, M_REDUCE = 1, M_OFFSETS = 2 };
constexpr int kGranule = 64;
struct SegView {
  const int *len;
  const int *off;
  const int *gran;
  const unsigned *bits;
  int n, m;
};
__host__ __device__ inline long segdes_off_words(int m) { return ((long)m + 3) & ~3L; }
__host__ __device__ inline long segdes_gran_words(int m) {
  return segdes_off_words(m) + (((long)m + 1 + 3) & ~3L);
}
__host__ __device__ inline long segdes_bits_words(int n, int m) {
  long ng = ((long)n + kGranule - 1) / kGranule;
  return segdes_gran_words(m) + ((ng + 1 + 3) & ~3L);
}
__host__ __device__ inline long segdes_nbits_words(int n) { return ((((long)n + 31) / 32) + 255) & ~255L; }
__host__ __device__ inline long segdes_total_words(int n, int m) {
  return segdes_bits_words(n, m) + segdes_nbits_words(n);
}
inline SegView seg_view(vec_p sd, int n, int m) {
  const int *b = (const int *)sd;
  return SegView{b, b + segdes_off_words(m), b + segdes_gran_words(m),
                 (const unsigned *)(b + segdes_bits_words(n, m)), n, m};
}

// Segment holding element k (0 <= k < n): the largest s with off[s] <= k.
// The granule table bounds the search to the segments of one granule.
__device__ __forceinline__ int seg_of(const SegView &v, int k) {
  int g = k / kGranule;
  int lo = __ldg(v.gran + g);
  int hi = __ldg(v.gran + g + 1);
  if (hi > v.m - 1) hi = v.m - 1;
  // invariant: off[lo] <= k; answer in [lo, hi]
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (__ldg(v.off + mid) <= k) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// --------------------------------------------------- tile status words ---
// Decoupled look-back state for one launch, carved out of scratch:
//   counter (u32, dynamic tile ticket), then one 16-byte word per tile:
//   {status, value bits}, written with one 128-bit store and read with one
//   128-bit load.  The word is self-contained -- no other data is read on the
//   strength of its status -- so relaxed ordering suffices, and a warp's
//   loads of many predecessors' words are all in flight at once (acquire
//   loads would each wait for the one before).
// The whole area is cleared before a launch.
enum : unsigned { TS_EMPTY = 0, TS_AGG = 1, TS_INC = 2 };
struct LookbackMem {
  unsigned *counter;
  ulonglong2 *word;
};
// The area is placed at the first 256-byte boundary of the scratch: the
// 128-bit status accesses need 16-byte alignment, and a caller's scratch
// vector (sub-allocated in 8-byte units) need not have it.
inline size_t lookback_bytes(int tiles) { return 512 + align_up((size_t)tiles * 16, 256); }
inline size_t lookback_clear_bytes(int tiles) { return lookback_bytes(tiles); }
inline LookbackMem lookback_carve(void *base, int tiles) {
  (void)tiles;
  char *p = (char *)align_up((size_t)base, 256);
  return LookbackMem{(unsigned *)p, (ulonglong2 *)(p + 256)};
}
// scratch units (8 bytes) needed by a look-back launch of `tiles` tiles
inline int lookback_units(int tiles) { return (int)((lookback_bytes(tiles) + 7) / 8); }

// Partitioned scatter (rank.cu): d[idx[k]] = s[k] for k < n, idx in
// [0, n_d), by a split of the (index, value) pairs into windows of the
// output (at most 8 MB each) and a window-by-window scatter.  Worth it once
// the output is larger than L2 can absorb random writes to; scratch of
// scatter_partitioned_bytes.
bool scatter_partitioned_wanted(long n_d, size_t vsize);
size_t scatter_partitioned_bytes(long n, size_t vsize);
template <class V> void scatter_partitioned(V *d, const V *s, const int *idx, int n, int n_d, vec_p scratch);
// Gathers d[k] = s[idx[k]] from a source larger than L2 absorbs random reads
// from (rank.cu: partitioned by source window); scratch of
// gather_partitioned_bytes.
bool gather_partitioned_wanted(long n_src, long n, size_t vsize);
size_t gather_partitioned_bytes(long n, size_t vsize);
template <class V> void gather_partitioned(V *d, const V *s, const int *idx, int n, int n_src, vec_p scratch);

__device__ __forceinline__ void lb_publish(ulonglong2 *w, unsigned long long status, unsigned long long bits) {
  asm volatile("{\n .reg .b128 t;\n mov.b128 t, {%1, %2};\n st.relaxed.gpu.global.b128 [%0], t;\n}"
               ::"l"(w), "l"(status), "l"(bits) : "memory");
}
__device__ __forceinline__ void lb_read(const ulonglong2 *w, unsigned long long &status,
                                        unsigned long long &bits) {
  asm volatile("{\n .reg .b128 t;\n ld.relaxed.gpu.global.b128 t, [%2];\n mov.b128 {%0, %1}, t;\n}"
               : "=l"(status), "=l"(bits) : "l"(w) : "memory");
}

template <class T> __device__ __forceinline__ unsigned long long to_bits(T v) {
  unsigned long long b = 0; memcpy(&b, &v, sizeof(T)); return b;
}
template <class T> __device__ __forceinline__ T from_bits(unsigned long long b) {
  T v; memcpy(&v, &b, sizeof(T)); return v;
}

// Exclusive prefix of `tile` over the words earlier tiles published, run by
// one whole warp.  Each step covers 32 * LB_K predecessors (LB_K words per
// lane, loaded together), combined in element order, until an inclusive word
// is found; only the words nearer than the nearest inclusive word already
// seen are waited for.  Narrow steps measured fastest on GB300 (segmented
// float64 +-scan of 2^28 elements: 1.29 ms with 32 predecessors per step,
// 1.39 ms with 64, 1.59 ms with 128); a likely cause is that the words of
// running tiles share cache lines their CTAs are writing, and a wider step
// reads more of them per round trip.  Every wait is bounded by spin_limit.
#ifndef GCVL_LB_K
#define GCVL_LB_K 1
#endif
constexpr int LB_K = GCVL_LB_K;
template <class Op>
__device__ __forceinline__ typename Op::T lookback_prefix(const ulonglong2 *words, int tile,
                                                          unsigned *status, int spin_limit) {
  typedef typename Op::T T;
  const int lane = threadIdx.x & 31;
  T P = Op::ident();
  int pred = tile - 1;
  while (true) {
    // lane l holds predecessors pred - l*LB_K - j, j = 0 (nearest) .. LB_K-1
    unsigned long long stt[LB_K], bits[LB_K];
#pragma unroll
    for (int j = 0; j < LB_K; j++) {
      const int t = pred - lane * LB_K - j;
      stt[j] = TS_INC;
      bits[j] = to_bits<T>(Op::ident());
      if (t >= 0) lb_read(words + t, stt[j], bits[j]);
    }
    // the nearest inclusive word seen so far: nothing beyond it is needed
    int jinc = LB_K;
#pragma unroll
    for (int j = LB_K - 1; j >= 0; j--)
      if (stt[j] == TS_INC) jinc = j;
    unsigned incm = __ballot_sync(0xffffffffu, jinc < LB_K);
    int stop = incm ? __ffs(incm) - 1 : 31;
#pragma unroll
    for (int j = 0; j < LB_K; j++) {
      if (lane > stop || (lane == stop && j >= jinc)) continue;
      const int t = pred - lane * LB_K - j;
      int it = 0;
      while (stt[j] == TS_EMPTY) {
        if (++it >= spin_limit) {
          atomicOr(status, DEV_TIMEOUT);
          stt[j] = TS_INC;
          bits[j] = to_bits<T>(Op::ident());
          break;
        }
        __nanosleep(32);
        lb_read(words + t, stt[j], bits[j]);
      }
    }
    // nearest inclusive word of this lane (a waited-for word may have become
    // one), and the lane's fold from there (or from its farthest word) to
    // its nearest, in element order
    jinc = LB_K;
#pragma unroll
    for (int j = LB_K - 1; j >= 0; j--)
      if (stt[j] == TS_INC) jinc = j;
    T val = Op::ident();
#pragma unroll
    for (int j = LB_K - 1; j >= 0; j--)
      if (j <= jinc || jinc == LB_K) val = Op::apply(val, from_bits<T>(bits[j]));
    incm = __ballot_sync(0xffffffffu, jinc < LB_K);
    stop = incm ? __ffs(incm) - 1 : 31;
    if (lane > stop) val = Op::ident();
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      T o = shfl_down(val, d);
      if (lane + d < 32) val = Op::apply(o, val);
    }
    val = shfl_idx(val, 0);
    P = Op::apply(val, P);
    if (incm) break;
    pred -= 32 * LB_K;
  }
  return P;
}

}  // namespace gcvl
