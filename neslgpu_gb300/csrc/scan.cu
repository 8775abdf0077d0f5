// scan.cu -- segmented and unsegmented scans and reductions.
//
// Semantics: the serial CVL (nesl/cvl/serial/vprims.c:17-201): exclusive
// scans that restart from the operator's initial value at every segment,
// reductions that yield the initial value for an empty segment.
//
// Design: tiles of 128-byte rows, one row per thread; a thread folds its
// (head, value) pairs, warp shuffles scan them across the CTA, and the carry
// from earlier tiles comes from a decoupled look-back over 16-byte status
// words (a tile that holds a segment head publishes its inclusive value at
// once; the warp-wide look-back walks 32 tiles per round trip).  Kernels:
//  * k_scan_ring -- scans of 16-byte aligned vectors: persistent CTAs take
//    tiles from a ticket counter, move them by TMA through a two-slot ring,
//    and write each tile's outputs one round after its fold, so the carry
//    it needs is ready;
//  * k_segred_warp -- segmented reductions of 4-byte elements with segments
//    of 32 elements or more on average: each warp streams its own range of
//    chunks, the carry in registers, no look-back;
//  * k_scan_tma -- the other reductions of 16-byte aligned vectors, one TMA
//    tile per CTA, results at segment ends and no look-back wait:
//    k_tile_fix completes the results that span tiles or warp ranges (and
//    the no-alloc scan);
//  * k_scan -- everything else (vectors off a 16-byte boundary, the offsets
//    scan of mke_fov), staged with coalesced loads.
// Every wait is bounded.
#include "gcvl.cuh"
#include "tma.cuh"

#include <stdlib.h>
#include <algorithm>
#include <type_traits>

namespace gcvl {

template <class T> struct Tiling;
template <> struct Tiling<int> { static constexpr int BLOCK = 256, ITEMS = 16; };
template <> struct Tiling<double> { static constexpr int BLOCK = 256, ITEMS = 8; };


template <class T> struct ScanArgs {
  T *out;            // scan: n outputs; reduce: m outputs; offsets: m+1
  const T *in;       // n inputs
  T *out2;           // offsets mode: copy of the input (segment lengths)
  SegView sv;        // segment descriptor (segmented kernels only)
  int n;
  LookbackMem lb;
  unsigned *status;
  int spin_limit;
  int count_flags;   // pk1_lev: fold (x != 0) instead of x
  const int *gidx;   // gather-multiply form: element k is in[k] * gsrc[gidx[k]]
  const T *gsrc;
  int *lead;         // reductions: per tile, the result lacking the earlier tiles' part (-1: none)
};

// Coalesced load of a tile into per-thread blocked registers through padded
// shared memory (conflict-free for 4- and 8-byte elements).
template <class T, int ITEMS>
__device__ __forceinline__ void load_blocked(T (&x)[ITEMS], const T *__restrict__ g, int valid,
                                             T fill, T *sbuf) {
  constexpr int PE = 128 / sizeof(T);
  const int lane = threadIdx.x & 31;
  const int wbase = (threadIdx.x >> 5) * 32 * ITEMS;
#pragma unroll
  for (int j = 0; j < ITEMS; j++) {
    int idx = wbase + j * 32 + lane;
    T v = fill;
    if (idx < valid) v = __ldcs(g + idx);
    sbuf[idx + idx / PE] = v;
  }
  __syncwarp();
#pragma unroll
  for (int i = 0; i < ITEMS; i++) {
    int idx = threadIdx.x * ITEMS + i;
    x[i] = sbuf[idx + idx / PE];
  }
  __syncwarp();
}

template <class T, int ITEMS>
__device__ __forceinline__ void store_blocked(const T (&y)[ITEMS], T *__restrict__ g, int valid,
                                              T *sbuf) {
  constexpr int PE = 128 / sizeof(T);
  const int lane = threadIdx.x & 31;
  const int wbase = (threadIdx.x >> 5) * 32 * ITEMS;
#pragma unroll
  for (int i = 0; i < ITEMS; i++) {
    int idx = threadIdx.x * ITEMS + i;
    sbuf[idx + idx / PE] = y[i];
  }
  __syncwarp();
#pragma unroll
  for (int j = 0; j < ITEMS; j++) {
    int idx = wbase + j * 32 + lane;
    if (idx < valid) __stcs(g + idx, sbuf[idx + idx / PE]);
  }
  __syncwarp();
}

// Head bits of elements k0 .. k0+cnt-1 (bit i set when k0+i starts a
// non-empty segment) and the segment holding k0.
template <int ITEMS>
__device__ __forceinline__ unsigned head_bits(const SegView &sv, int k0, int cnt, int &s0) {
  unsigned h = 0;
  int s = seg_of(sv, k0);
  s0 = s;
  if (__ldg(sv.off + s) == k0) h = 1u;
  int nxt = __ldg(sv.off + s + 1);
  while (nxt < k0 + cnt) {
    h |= 1u << (nxt - k0);
    ++s;
    while (__ldg(sv.off + s + 1) == nxt) ++s;
    nxt = __ldg(sv.off + s + 1);
  }
  return h;
}

template <class Op, int MODE, bool SEG, bool GATHER = false>
__global__ void __launch_bounds__(Tiling<typename Op::T>::BLOCK)
k_scan(ScanArgs<typename Op::T> a) {
  typedef typename Op::T T;
  constexpr int BLOCK = Tiling<T>::BLOCK, ITEMS = Tiling<T>::ITEMS, TILE = BLOCK * ITEMS;
  constexpr int NW = BLOCK / 32;
  constexpr int PE = 128 / sizeof(T);
  __shared__ T s_stage[TILE + TILE / PE];
  __shared__ int s_gidx[GATHER ? TILE + TILE / 32 : 1];
  __shared__ int s_wf[NW];
  __shared__ T s_wv[NW];
  __shared__ T s_prefix;
  __shared__ unsigned s_tile;

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) s_tile = atomicAdd(a.lb.counter, 1u);
  __syncthreads();
  const int tile = (int)s_tile;
  const long base = (long)tile * TILE;
  const int valid = (int)min((long)TILE, (long)a.n - base);

  T x[ITEMS];
  load_blocked<T, ITEMS>(x, a.in + base, valid, Op::ident(), s_stage);
  if constexpr (GATHER) {
    // fused gather-multiply: the element is in[k] * gsrc[gidx[k]] (the
    // products a BPERMUTE and an elementwise * would have materialised)
    int g[ITEMS];
    load_blocked<int, ITEMS>(g, a.gidx + base, valid, 0, s_gidx);
    const int kk = threadIdx.x * ITEMS;
    T v[ITEMS];
#pragma unroll
    for (int i = 0; i < ITEMS; i++) v[i] = (kk + i < valid) ? __ldg(a.gsrc + g[i]) : (T)1;
#pragma unroll
    for (int i = 0; i < ITEMS; i++)
      if (kk + i < valid) x[i] = x[i] * v[i];
  }
  if (a.count_flags) {
#pragma unroll
    for (int i = 0; i < ITEMS; i++) x[i] = (x[i] != (T)0) ? (T)1 : (T)0;
  }

  const int k0 = (int)base + tid * ITEMS;
  const int cnt = max(0, min(ITEMS, a.n - k0));
  unsigned heads = 0;
  int s0 = 0;
  if (cnt > 0) {
    if (SEG) heads = head_bits<ITEMS>(a.sv, k0, cnt, s0);
    else heads = (k0 == 0) ? 1u : 0u;
  }

  // per-thread fold of (head, value); padding items are identities
  int tf = heads != 0;
  T tv = Op::ident();
#pragma unroll
  for (int i = 0; i < ITEMS; i++) {
    if (i < cnt) tv = ((heads >> i) & 1u) ? Op::apply(Op::init(), x[i]) : Op::apply(tv, x[i]);
  }

  // warp inclusive scan of the pairs
  int f = tf;
  T v = tv;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    int f2 = shfl_up(f, d);
    T v2 = shfl_up(v, d);
    if (lane >= d) { v = f ? v : Op::apply(v2, v); f |= f2; }
  }
  int ef = shfl_up(f, 1);
  T ev = shfl_up(v, 1);
  if (lane == 0) { ef = 0; ev = Op::ident(); }
  if (lane == 31) { s_wf[warp] = f; s_wv[warp] = v; }
  __syncthreads();

  // prefix over the warps before mine, and the tile aggregate
  int pf = 0, af = 0;
  T pv = Op::ident(), av = Op::ident();
#pragma unroll
  for (int w = 0; w < NW; w++) {
    int wf = s_wf[w];
    T wv = s_wv[w];
    if (w == warp) { pf = af; pv = av; }
    av = wf ? wv : Op::apply(av, wv);
    af |= wf;
  }
  // in-tile exclusive prefix of this thread
  pv = ef ? ev : Op::apply(pv, ev);
  pf |= ef;

  // publish and look back (reductions do not wait: the one result per tile
  // that lacks the earlier tiles' part is completed by k_tile_fix)
  if (warp == 0) {
    // thread 0 holds element `base`: its head bit says whether the tile
    // starts a segment (then no carry from earlier tiles is needed)
    const bool first_head = shfl_idx((int)(heads & 1u), 0) != 0;
    if (lane == 0) lb_publish(a.lb.word + tile, (tile == 0 || af) ? TS_INC : TS_AGG, to_bits<T>(av));
    T P = Op::ident();
    if (MODE != M_REDUCE && tile > 0 && !first_head) {
      P = lookback_prefix<Op>(a.lb.word, tile, a.status, a.spin_limit);
      if (lane == 0 && !af) lb_publish(a.lb.word + tile, TS_INC, to_bits<T>(Op::apply(P, av)));
    }
    if (lane == 0) s_prefix = P;
  }
  __syncthreads();
  const T P = s_prefix;
  T run = pf ? pv : Op::apply(P, pv);

  if (MODE == M_SCAN || MODE == M_OFFSETS) {
    T y[ITEMS];
#pragma unroll
    for (int i = 0; i < ITEMS; i++) {
      if ((heads >> i) & 1u) run = Op::init();
      y[i] = run;
      run = Op::apply(run, x[i]);
    }
    __syncthreads();  // s_stage reuse
    store_blocked<T, ITEMS>(y, a.out + base, valid, s_stage);
    if (MODE == M_OFFSETS) {
      store_blocked<T, ITEMS>(x, a.out2 + base, valid, s_stage);
      if (k0 < a.n && k0 + cnt == a.n) a.out[a.n] = run;  // total after the last element
    }
  } else {  // M_REDUCE
    if (cnt > 0) {
      const int m = a.sv.m;
      if (k0 == 0) {
        for (int s = 0; s < s0; s++) a.out[s] = Op::init();  // leading empty segments
      }
      int s = s0;
      int end = __ldg(a.sv.off + s + 1);
      for (int i = 0; i < cnt; i++) {
        if ((heads >> i) & 1u) run = Op::init();
        run = Op::apply(run, x[i]);
        if (k0 + i + 1 == end) {
          a.out[s] = run;
          if (!pf && !(heads & ((2u << i) - 1u))) a.lead[tile] = s;  // began in an earlier tile
          int s2 = s + 1;
          while (s2 < m && __ldg(a.sv.off + s2 + 1) == end) { a.out[s2] = Op::init(); ++s2; }
          s = s2;
          if (s < m) end = __ldg(a.sv.off + s + 1);
        }
      }
    }
  }
}

// ============================================================================
// TMA-staged tile kernel: the reductions of 16-byte aligned vectors (and the
// no-alloc entry point's scan).
//
// A tile is TT rows of 128 bytes (32 ints or 16 doubles per row), one row per
// thread.  One elected thread moves the whole tile with a 2-D TMA tensor copy
// (128-byte swizzle, so each thread reads its row from shared memory without
// bank conflicts) and, for a scan, writes the results back the same way.
// Segment heads come from the head bitmap; a reduction's segment numbers from
// a window of the segment offsets that the CTA loads into shared memory.
// Float64 + folds run in 64-bit integer fixed point and float64 min/max
// compare integer keys, which keeps GB300's narrow FP64 pipe for the adds
// that need it.
// ============================================================================
#ifndef GCVL_TT
#define GCVL_TT 128
#endif
constexpr int TT = GCVL_TT;  // threads per CTA = rows per tile
template <class T> constexpr int row_items() { return 128 / (int)sizeof(T); }
// Offsets window of a segmented reduction, held in shared memory (scans
// keep none).  Full: room for every segment of a tile whose segments are
// non-empty.  An int reduction whose segments average 3 elements or more
// gets half of that (tiles of segments averaging 2 and more fit), keeping
// its seventh CTA per SM: a full window cost 7 % on long segments, a half
// one 10x on the one-element segments of a quicksort's last levels.  Tiles
// with more segments than their window look offsets up in global memory.
template <class T> constexpr int wmax_full() { return TT * row_items<T>() + 2; }
template <class T, int MODE> inline int wmax_for(int n, int m) {
  if (MODE != M_REDUCE) return 0;
  if (sizeof(T) == 8 || (long)n < 3L * m) return wmax_full<T>();
  return TT * row_items<T>() / 2 + 2;
}

template <class T> struct TArgs {
  T *out;
  const T *in;
  SegView sv;
  int n;
  long rows;  // complete 128-byte rows of the input (the TMA tensor height)
  LookbackMem lb;
  unsigned *status;
  int spin_limit;
  int *lead;  // reductions: per tile, the segment whose result lacks the earlier tiles' part (-1: none)
  int wmax;   // reductions: entries of the shared-memory offsets window
  const int *gidx;  // gather-multiply form: element k is in[k] * gsrc[gidx[k]]
  const T *gsrc;
};

// Segment offsets seen through the shared-memory window when possible.
// Entry j sits at j + j/32: with one-element segments lane t of a warp reads
// entry 32t + i, and unpadded every lane would hit the same bank (a
// quicksort's last-level reductions: 91 -> 71 us per call at 2^24).
__host__ __device__ constexpr int wpad(int j) { return j + (j >> 5); }
struct OffWin {
  const int *win; const int *glob; int s0, w;
  __device__ __forceinline__ int operator()(int s) const {
    int j = s - s0;
    return (j >= 0 && j < w) ? win[wpad(j)] : __ldg(glob + s);
  }
};

// ---- per-thread fold engines ---------------------------------------------
// agg(): (has head, fold of the items from the last head -- starting from
// init -- or of all items when there is none).
template <class Op, int ITEMS> struct Engine {
  typedef typename Op::T T;
  static __device__ __forceinline__ void agg(const T (&x)[ITEMS], unsigned heads, int cnt, int &tf, T &tv) {
    tf = heads != 0;
    tv = Op::ident();
#pragma unroll
    for (int i = 0; i < ITEMS; i++)
      if (i < cnt) tv = ((heads >> i) & 1u) ? Op::apply(Op::init(), x[i]) : Op::apply(tv, x[i]);
  }
};

template <int ITEMS> struct Engine<AddD, ITEMS> {
  static __device__ __forceinline__ void agg(const double (&x)[ITEMS], unsigned heads, int cnt, int &tf,
                                             double &tv) {
    tf = heads != 0;
    tv = AddD::ident();
    if (cnt <= 0) return;
    const int from = heads ? 31 - __clz((int)heads) : 0;
    int emax = 1;
#pragma unroll
    for (int i = 0; i < ITEMS; i++)
      if (i >= from && i < cnt) emax = max(emax, fx_exp((unsigned long long)__double_as_longlong(x[i])));
    if (emax == 2047) {  // an infinity or NaN: fold in FP64
#pragma unroll
      for (int i = 0; i < ITEMS; i++)
        if (i >= from && i < cnt) tv = (i == from && tf) ? AddD::apply(0.0, x[i]) : AddD::apply(tv, x[i]);
      return;
    }
    long long acc = 0;
#pragma unroll
    for (int i = 0; i < ITEMS; i++)
      if (i >= from && i < cnt) fx_add(acc, (unsigned long long)__double_as_longlong(x[i]), emax);
    tv = fx_to_double_alu(acc, emax);  // never -0.0, so starting from init 0.0 changes nothing
  }
};

// Float64 + reductions of short segments (the CHAIN form of the kernel,
// chosen when segments average under RED_CHAIN_MEAN elements): a warp in
// which some thread ends at least two segments sums its pieces with one FP64
// add per item instead of a fixed-point pass per segment end.  At 2^28,
// geometric(4) segments 2.98 -> 1.14 ms, geometric(64) 1.12 -> 1.01 ms; the
// log-normal(5,2) bench segments (about 1100 elements on average) keep the
// plain form, which the chain's code alone slows by 2-4 %.
constexpr long RED_CHAIN_MEAN = 256;
// Reductions: a thread's float64 + fold split between the integer pipes
// (the first GCVL_RED_FX_ITEMS items, fixed point) and the FP64 pipe (the
// rest, an add chain), so that neither carries the whole fold; 14 of 16
// measured best (8 of 16: 16 % slower, 16 of 16: 3 %).  The segmented
// reduction has no per-element output work to keep the FP64 pipe busy.
#ifndef GCVL_RED_FX_ITEMS
#define GCVL_RED_FX_ITEMS 14
#endif
template <int ITEMS>
__device__ __forceinline__ void agg_add_split(const double (&x)[ITEMS], unsigned heads, int cnt, int &tf,
                                              double &tv) {
  constexpr int H = GCVL_RED_FX_ITEMS < ITEMS ? GCVL_RED_FX_ITEMS : ITEMS;  // items in fixed point
  tf = heads != 0;
  tv = AddD::ident();
  if (__all_sync(0xffffffffu, heads == 0 && cnt == ITEMS)) {
    // the whole warp folds full rows without segment starts: no per-item tests
    const double lo = fx_range_part<ITEMS, 0, H>(x, 0, ITEMS);
    double hi = -0.0;
#pragma unroll
    for (int i = H; i < ITEMS; i++) hi = __dadd_rn(hi, x[i]);
    tv = __dadd_rn(lo, hi);
    return;
  }
  if (cnt <= 0) return;
  const int from = heads ? 31 - __clz((int)heads) : 0;
  const double lo = fx_range_part<ITEMS, 0, H>(x, from, cnt);
  double hi = -0.0;
#pragma unroll
  for (int i = H; i < ITEMS; i++)
    if (i >= from && i < cnt) hi = __dadd_rn(hi, x[i]);
  tv = __dadd_rn(lo, hi);
}

// The CTA has TT compute threads (one 128-byte row each) plus one look-back
// warp.  The look-back warp issues the tile's TMA load and at once starts
// collecting the carry from earlier tiles, while the compute warps fold their
// rows: the carry's round trips overlap the load and the fold instead of
// following them.  The compute warps publish the tile aggregate as soon as it
// exists and meet the look-back warp only when they need the carry.
constexpr int TB_LB = TT + 32;  // threads per CTA of a scan
// A reduction does not wait for earlier tiles, so its CTA has no look-back
// warp: thread 0 issues the TMA load, and the smaller CTA lets more fit per SM.
template <int MODE> constexpr int cta_threads() { return MODE == M_REDUCE ? TT : TB_LB; }
// Resident CTAs per SM the register allocation must allow.  Scans hold no
// offsets window, so registers, not shared memory, set their occupancy: 8
// (48-56 registers, a few spilled) measured 4 % faster than 7 on the float64
// scan and 27 % on the int scan; 9 spills heavily and is slower.
// Reductions (128-thread CTAs): 8 (float64 reduce 0.90 -> 0.86 ms at 2^28;
// 9 gains nothing and slows the int reduce).
#ifndef GCVL_SCAN_MINB
#define GCVL_SCAN_MINB 8
#endif
#ifndef GCVL_RED_MINB_D
#define GCVL_RED_MINB_D 8
#endif
#ifndef GCVL_RED_MINB_Z
#define GCVL_RED_MINB_Z 8
#endif
// The gather-multiply form (a CSR sparse matrix-vector product: values by
// TMA, column indices and the gathered vector entries by plain loads) holds
// 16 more loads per thread in flight and runs 4 CTAs per SM.
template <int MODE, class T, bool GATHER> constexpr int tma_minb() {
  return GATHER ? 4 : MODE == M_REDUCE ? (sizeof(T) == 8 ? GCVL_RED_MINB_D : GCVL_RED_MINB_Z) : GCVL_SCAN_MINB;
}
template <class Op, int MODE, bool SEG, bool CHAIN = false, bool GATHER = false>
__global__ void __launch_bounds__(cta_threads<MODE>(), tma_minb<MODE, typename Op::T, GATHER>()) k_scan_tma(const __grid_constant__ CUtensorMap tin,
                                                     const __grid_constant__ CUtensorMap tout,
                                                     TArgs<typename Op::T> a) {
  typedef typename Op::T T;
  constexpr int ITEMS = row_items<T>(), TILE = TT * ITEMS, NW = TT / 32;
  extern __shared__ unsigned char dyn_smem[];
  unsigned char *tile_b = (unsigned char *)(((size_t)dyn_smem + 1023) & ~(size_t)1023);
  int *win = (int *)(tile_b + TILE * sizeof(T));
  __shared__ unsigned long long bar;
  __shared__ int s_wf[NW], s_wpf[NW];
  __shared__ T s_wv[NW], s_wpv[NW];
  __shared__ T s_prefix, s_av;
  __shared__ int s_af;

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // Tiles are taken in block order; blocks are dispatched in index order, so
  // every predecessor a tile waits for is running or done (and the waits are
  // bounded regardless).
  const int tile = blockIdx.x;
  const long base = (long)tile * TILE;
  const int valid = (int)min((long)TILE, (long)a.n - base);
  if (tid == (MODE == M_REDUCE ? 0 : TT)) {
    mbar_init(&bar, 1);
    fence_mbar_init();
    mbar_arrive_expect_tx(&bar, TILE * (unsigned)sizeof(T));
    tma_load_2d(tile_b, &tin, &bar, 0, tile * TT);
    if (MODE == M_REDUCE) s_prefix = Op::ident();
  }
  __syncthreads();  // barrier initialised

  if (MODE != M_REDUCE && warp == NW) {
    // ------------------------------------------------------ look-back warp
    // (reductions do not wait: the one result per tile that needs earlier
    // tiles' part is completed afterwards by k_tile_fix)
    T P = Op::ident();
    bool first_head = true;
    if constexpr (MODE != M_REDUCE) {
      if (SEG) first_head = (__ldg(a.sv.bits + (base >> 5)) >> (base & 31)) & 1u;
      else first_head = base == 0;
      if (tile > 0 && !first_head) P = lookback_prefix<Op>(a.lb.word, tile, a.status, a.spin_limit);
    }
    if (lane == 0) s_prefix = P;
    named_sync(1, TB_LB);  // carry ready / tile aggregate ready
    if (MODE != M_REDUCE && lane == 0 && tile > 0 && !first_head && !s_af)
      lb_publish(a.lb.word + tile, TS_INC, to_bits<T>(Op::apply(P, s_av)));
    // the compute warps have waited for the tile (bounded): the issuing
    // thread leaves only once it has landed
    if (lane == 0 && !mbar_wait(&bar, 0, kDrainLimit)) atomicOr(a.status, DEV_TIMEOUT);
    return;
  }

  // --------------------------------------------------------- compute warps
  const int k0 = (int)base + tid * ITEMS;
  const int cnt = max(0, min(ITEMS, a.n - k0));
  unsigned heads = 0;
  if (cnt > 0) {
    if (SEG) {
      const unsigned w = __ldg(a.sv.bits + (k0 >> 5));
      heads = (ITEMS == 32) ? w : ((w >> (k0 & 31)) & ((1u << ITEMS) - 1u));
      if (cnt < ITEMS) heads &= (1u << cnt) - 1u;
    } else {
      heads = (k0 == 0) ? 1u : 0u;
    }
  }
  // reductions also need segment numbers: a window of offsets whose bounds
  // come straight from the granule table (tiles start on granule boundaries)
  int W = 0, sf = 0;
  if (SEG && MODE == M_REDUCE) {
    sf = __ldg(a.sv.gran + base / kGranule);
    const long e = base + valid;
    const int sl = (e >= a.n) ? a.sv.m - 1 : __ldg(a.sv.gran + e / kGranule);
    W = sl - sf + 2;
    if (W <= a.wmax)
      for (int i = tid; i < W; i += TT) win[wpad(i)] = __ldg(a.sv.off + sf + i);
    named_sync(2, TT);  // window loaded
  }
  {
    int it = 0;
    while (!mbar_try_wait(&bar, 0)) {
      if (++it >= a.spin_limit) {
        // flagged; still let the tile land (bounded) before reading it, so
        // that no copy into this CTA's shared memory outlives the CTA
        atomicOr(a.status, DEV_TIMEOUT);
        mbar_wait(&bar, 0, kDrainLimit);
        break;
      }
    }
  }
  const OffWin off{win, a.sv.off, sf, (SEG && W <= a.wmax) ? W : 0};

  // this thread's row
  const long grow = (long)tile * TT + tid;
  T x[ITEMS];
  if (grow < a.rows) {
#pragma unroll
    for (int c = 0; c < 8; c++) {
      const uint4 u = *(const uint4 *)(tile_b + swz(tid, c));
      memcpy(&x[c * (16 / sizeof(T))], &u, 16);
    }
  } else {
#pragma unroll
    for (int i = 0; i < ITEMS; i++) x[i] = (i < cnt) ? a.in[k0 + i] : Op::ident();
  }
  if constexpr (std::is_same<Op, CountB>::value) {
#pragma unroll
    for (int i = 0; i < ITEMS; i++) x[i] = x[i] != 0;  // pk1_lev counts true flags
  }
  if constexpr (GATHER) {
    // the products a BPERMUTE and an elementwise * would have materialised;
    // gidx is 16-byte aligned and k0 a multiple of ITEMS, so a full row's
    // indices are ITEMS/4 aligned 16-byte loads
    int g[ITEMS];
    if (cnt == ITEMS) {
#pragma unroll
      for (int c = 0; c < ITEMS / 4; c++) {
        const int4 q = __ldcs(reinterpret_cast<const int4 *>(a.gidx + k0) + c);
        g[4 * c] = q.x; g[4 * c + 1] = q.y; g[4 * c + 2] = q.z; g[4 * c + 3] = q.w;
      }
    } else {
#pragma unroll
      for (int i = 0; i < ITEMS; i++) g[i] = i < cnt ? __ldcs(a.gidx + k0 + i) : 0;
    }
    T v[ITEMS];
#pragma unroll
    for (int i = 0; i < ITEMS; i++) v[i] = i < cnt ? __ldg(a.gsrc + g[i]) : (T)0;
#pragma unroll
    for (int i = 0; i < ITEMS; i++) x[i] = i < cnt ? x[i] * v[i] : Op::ident();
  }
  // segment holding k0 (reductions): the last window entry <= k0
  int s0 = 0;
  if (SEG && MODE == M_REDUCE && cnt > 0) {
    if (W <= a.wmax) {
      int lo = 0, hi = W - 2;
      while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (win[wpad(mid)] <= k0) lo = mid; else hi = mid - 1;
      }
      s0 = sf + lo;
    } else {
      s0 = seg_of(a.sv, k0);
    }
  }

  int tf;
  T tv;
  // Reductions other than float64 + take one pass over the thread's items:
  // the results of segments that start and end among them are final at
  // once; the first segment end, whose segment began before these items,
  // waits for the earlier threads' prefix (first_s, first_v).  Float64 +
  // folds in fixed point per piece below.
  constexpr bool ONE_PASS = SEG && MODE == M_REDUCE && !std::is_same<Op, AddD>::value;
  int first_s = -1;
  T first_v = Op::ident();
  if constexpr (ONE_PASS) {
    T r = Op::ident();
    bool started = false;
    if (cnt > 0) {
      const int m = a.sv.m;
      if (k0 == 0)
        for (int q = 0; q < s0; q++) a.out[q] = Op::init();  // empty segments before element 0
      int sg = s0;
      int end = off(sg + 1);
#pragma unroll
      for (int i = 0; i < ITEMS; i++) {
        if (i < cnt) {
          if ((heads >> i) & 1u) { r = Op::init(); started = true; }
          r = Op::apply(r, x[i]);
          if (k0 + i + 1 == end) {
            if (started) a.out[sg] = r;
            else { first_s = sg; first_v = r; }
            int s2 = sg + 1;
            while (s2 < m && off(s2 + 1) == end) { a.out[s2] = Op::init(); ++s2; }
            sg = s2;
            if (sg < m) end = off(sg + 1);
          }
        }
      }
    }
    tf = heads != 0;
    tv = r;
  } else if constexpr (MODE == M_REDUCE && std::is_same<Op, AddD>::value) {
    agg_add_split<ITEMS>(x, heads, cnt, tf, tv);
  } else {
    Engine<Op, ITEMS>::agg(x, heads, cnt, tf, tv);
  }

  // warp inclusive scan of (head, value)
  int f = tf;
  T v = tv;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    int f2 = shfl_up(f, d);
    T v2 = shfl_up(v, d);
    if (lane >= d) { v = f ? v : Op::apply(v2, v); f |= f2; }
  }
  int ef = shfl_up(f, 1);
  T ev = shfl_up(v, 1);
  if (lane == 0) { ef = 0; ev = Op::ident(); }
  if (lane == 31) { s_wf[warp] = f; s_wv[warp] = v; }
  named_sync(2, TT);

  if (warp == 0) {
    // exclusive prefixes over the warps, the tile aggregate, and its
    // publication for later tiles
    int wf = lane < NW ? s_wf[lane] : 0;
    T wv = lane < NW ? s_wv[lane] : Op::ident();
#pragma unroll
    for (int d = 1; d < NW; d <<= 1) {
      int f2 = shfl_up(wf, d);
      T v2 = shfl_up(wv, d);
      if (lane >= d) { wv = wf ? wv : Op::apply(v2, wv); wf |= f2; }
    }
    int xf = shfl_up(wf, 1);
    T xv = shfl_up(wv, 1);
    if (lane == 0) { xf = 0; xv = Op::ident(); }
    if (lane < NW) { s_wpf[lane] = xf; s_wpv[lane] = xv; }
    const int af = shfl_idx(wf, NW - 1);
    const T av = shfl_idx(wv, NW - 1);
    if (lane == 0) {
      lb_publish(a.lb.word + tile, (tile == 0 || af) ? TS_INC : TS_AGG, to_bits<T>(av));
      s_af = af;
      s_av = av;
    }
  }
  named_sync(1, cta_threads<MODE>());  // meet the look-back warp: carry and aggregate exchanged
  // this thread's exclusive prefix: (earlier tiles) . (earlier warps) . (earlier lanes)
  int pf = s_wpf[warp];
  T pv = s_wpv[warp];
  pv = ef ? ev : Op::apply(pv, ev);
  pf |= ef;
  T run = pf ? pv : Op::apply(s_prefix, pv);

  if (MODE == M_SCAN) {
#pragma unroll
    for (int i = 0; i < ITEMS; i++) {
      if ((heads >> i) & 1u) run = Op::init();
      const T y = run;
      run = Op::apply(run, x[i]);
      x[i] = y;
    }
    if (grow < a.rows) {
#pragma unroll
      for (int c = 0; c < 8; c++) {
        uint4 u;
        memcpy(&u, &x[c * (16 / sizeof(T))], 16);
        *(uint4 *)(tile_b + swz(tid, c)) = u;
      }
    } else {
#pragma unroll
      for (int i = 0; i < ITEMS; i++)
        if (i < cnt) a.out[k0 + i] = x[i];
    }
    fence_proxy_async_smem();
    named_sync(2, TT);
    if (tid == 0) {
      tma_store_2d(&tout, tile_b, 0, tile * TT);
      bulk_commit();
      bulk_wait_read_all();
    }
  } else if constexpr (ONE_PASS) {  // the one result still lacking the earlier part
    if (first_s >= 0) {
      a.out[first_s] = Op::apply(run, first_v);
      if (!pf) a.lead[tile] = first_s;  // began in an earlier tile
    }
  } else {  // M_REDUCE: results at segment ends
    // float64 +: pieces between heads, each summed in fixed point.  Element
    // i ends a non-empty segment exactly when element i+1 is a head (or past
    // the end): only those positions are visited (mostly none).  Whether the
    // warp chains its items is decided by every lane, those past the
    // vector's end too (they hold no ends): a warp vote must not name lanes
    // that are elsewhere.
    unsigned ends = 0;
    bool chain_warp = false;
    if constexpr (std::is_same<Op, AddD>::value) {
      if (cnt > 0) {
        const int kn = k0 + cnt;
        const unsigned nh = kn >= a.n ? 1u : (__ldg(a.sv.bits + (kn >> 5)) >> (kn & 31)) & 1u;
        ends = ((heads >> 1) | (nh << (cnt - 1))) & (cnt >= 32 ? ~0u : ((1u << cnt) - 1u));
      }
      if (CHAIN) chain_warp = __any_sync(0xffffffffu, __popc(ends) >= 2);
    }
    if (cnt > 0) {
      const int m = a.sv.m;
      if (k0 == 0)
        for (int s = 0; s < s0; s++) a.out[s] = Op::init();
      int s = s0;
      int end = off(s + 1);
      if constexpr (std::is_same<Op, AddD>::value) {
        if (chain_warp) {
          // short segments: one FP64 add per item beats a fixed-point pass
          // per segment end (each a separate sum of up to 16 items)
          double r = run;
#pragma unroll
          for (int i = 0; i < ITEMS; i++) {
            if (i < cnt) {
              if ((heads >> i) & 1u) r = 0.0;
              r = __dadd_rn(r, x[i]);
              if ((ends >> i) & 1u) {
                a.out[s] = r;
                if (!pf && !(heads & ((2u << i) - 1u))) a.lead[tile] = s;  // began in an earlier tile
                int s2 = s + 1;
                while (s2 < m && off(s2 + 1) == end) { a.out[s2] = 0.0; ++s2; }
                s = s2;
                if (s < m) end = off(s + 1);
              }
            }
          }
          ends = 0;
        }
        int ps = 0;
        while (ends) {
          const int i = __ffs(ends) - 1;
          ends &= ends - 1;
          {
            double pv2 = fx_range<ITEMS>(x, ps, i + 1);
            a.out[s] = ((heads >> ps) & 1u) ? pv2 : AddD::apply(run, pv2);
            if (!pf && !(heads & ((2u << i) - 1u))) a.lead[tile] = s;  // began in an earlier tile
            int s2 = s + 1;
            while (s2 < m && off(s2 + 1) == end) { a.out[s2] = 0.0; ++s2; }
            s = s2;
            if (s < m) end = off(s + 1);
            ps = i + 1;
          }
        }
      } else {
#pragma unroll
        for (int i = 0; i < ITEMS; i++) {
          if (i < cnt) {
            if ((heads >> i) & 1u) run = Op::init();
            run = Op::apply(run, x[i]);
            if (k0 + i + 1 == end) {
              a.out[s] = run;
              if (!pf && !(heads & ((2u << i) - 1u))) a.lead[tile] = s;  // began in an earlier tile
              int s2 = s + 1;
              while (s2 < m && off(s2 + 1) == end) { a.out[s2] = Op::init(); ++s2; }
              s = s2;
              if (s < m) end = off(s + 1);
            }
          }
        }
      }
    }
  }
}

// ============================================================================
// Persistent ring scan: the segmented and unsegmented scans of 16-byte
// aligned vectors.
//
// A CTA runs rounds.  Round r folds the tile loaded for it (one 128-byte row
// per compute thread) and publishes the tile aggregate, then writes the
// outputs of the tile it folded in round r-1.  The carry into that older tile
// depends on tiles folded a round earlier than the fold just done, so the
// look-back warp collects it while the compute warps fold; a tile-per-CTA
// scan instead waits, at every tile, for neighbours folded at the same time
// as itself (35 % of the float64 scan's time at 2^28).  Tiles come from a
// ticket counter in increasing order and the TMA loads run RING_NB rounds
// ahead in a ring of tile buffers.  Every tile below a ticket already belongs
// to a running CTA that folds it without waiting on anything but its own
// load, so the look-back ends however many CTAs are resident.
//
// Shape (float64 segmented scan at 2^28): 64-row tiles, two ring slots and
// 12 CTAs per SM (0.994 ms) over 128-row tiles at 6 per SM (1.020 ms); a
// third slot (prefetching a round further) costs the CTAs it displaces
// (1.17-1.23 ms).  The look-back is no longer the limit: skipping it
// entirely gives 0.999 ms at 128 rows.
// ============================================================================
#ifndef GCVL_RING_NB
#define GCVL_RING_NB 2
#endif
#ifndef GCVL_RING_MINB
#define GCVL_RING_MINB 12
#endif
#ifndef GCVL_RING_TT
#define GCVL_RING_TT 64
#endif
constexpr int RING_NB = GCVL_RING_NB;
constexpr int RTT = GCVL_RING_TT;  // rows per tile = compute threads per CTA
constexpr int RTB = RTT + 32;      // and the look-back warp
template <class T> constexpr size_t ring_smem() { return 1024 + (size_t)RING_NB * RTT * 128; }

// a thread's row: from the TMA tile (128-byte swizzle), or from global memory
// for the last partial row and past it (identities beyond the vector)
template <class Op, int ITEMS>
__device__ __forceinline__ void row_load(typename Op::T (&x)[ITEMS], const unsigned char *buf, int tid, bool in_map,
                                         const typename Op::T *in, int k0, int cnt) {
  typedef typename Op::T T;
  if (in_map) {
#pragma unroll
    for (int c = 0; c < 8; c++) {
      const uint4 u = *(const uint4 *)(buf + swz(tid, c));
      memcpy(&x[c * (16 / sizeof(T))], &u, 16);
    }
  } else {
#pragma unroll
    for (int i = 0; i < ITEMS; i++) x[i] = (i < cnt) ? in[k0 + i] : Op::ident();
  }
  if constexpr (std::is_same<Op, CountB>::value) {
#pragma unroll
    for (int i = 0; i < ITEMS; i++) x[i] = x[i] != 0;  // pk1_lev counts true flags
  }
}

// Fold and warp scan of float64 + rows, both in 64-bit fixed point.  A
// thread's fold from its last segment start is an integer at the scale of
// its largest exponent (fx_add); the segmented warp scan combines two ranges
// at the larger of their scales, the other one's integer shifted down to it
// (truncated), so every prefix is held at the scale of the largest item it
// contains: its error stays under 32 units of that scale, a few 1e-15 of the
// sum of magnitudes.  Sixteen 53-bit items take 57 bits and 32 lanes 62, so
// nothing overflows.  Only the exclusive prefix of each thread and the warp
// total become doubles, which takes the scan's five FP64 adds per thread off
// GB300's narrow FP64 pipe.  A warp holding an infinity or NaN scans in FP64.
template <int ITEMS>
__device__ __forceinline__ void fold_scan_addd(const double (&x)[ITEMS], unsigned heads, int cnt, int lane, int &f,
                                               double &v, int &ef, double &ev) {
  const bool plain = __all_sync(0xffffffffu, heads == 0 && cnt == ITEMS);  // no per-item tests
  const int from = heads ? 31 - __clz((int)heads) : 0;
  int emax = 1;
  if (plain) {
#pragma unroll
    for (int i = 0; i < ITEMS; i++) emax = max(emax, fx_exp((unsigned long long)__double_as_longlong(x[i])));
  } else {
#pragma unroll
    for (int i = 0; i < ITEMS; i++)
      if (i >= from && i < cnt) emax = max(emax, fx_exp((unsigned long long)__double_as_longlong(x[i])));
  }
  f = heads != 0;
  if (__any_sync(0xffffffffu, emax == 2047)) {
    Engine<AddD, ITEMS>::agg(x, heads, cnt, f, v);
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const int f2 = shfl_up(f, d);
      const double v2 = shfl_up(v, d);
      if (lane >= d) { v = f ? v : AddD::apply(v2, v); f |= f2; }
    }
    ef = shfl_up(f, 1);
    ev = shfl_up(v, 1);
    if (lane == 0) { ef = 0; ev = AddD::ident(); }
    return;
  }
  long long acc = 0;
  if (plain) {
#pragma unroll
    for (int i = 0; i < ITEMS; i++) fx_add(acc, (unsigned long long)__double_as_longlong(x[i]), emax);
  } else {
#pragma unroll
    for (int i = 0; i < ITEMS; i++)
      if (i >= from && i < cnt) fx_add(acc, (unsigned long long)__double_as_longlong(x[i]), emax);
  }
  int e = emax;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const int f2 = shfl_up(f, d), e2 = shfl_up(e, d);
    const long long a2 = shfl_up(acc, d);
    if (lane >= d) {
      if (!f) {
        const int em = max(e, e2);
        acc = (acc >> min(em - e, 63)) + (a2 >> min(em - e2, 63));
        e = em;
      }
      f |= f2;
    }
  }
  ef = shfl_up(f, 1);
  const long long ea = shfl_up(acc, 1);
  const int ee = shfl_up(e, 1);
  ev = lane == 0 ? AddD::ident() : fx_to_double_alu(ea, ee);
  if (lane == 0) ef = 0;
  v = lane == 31 ? fx_to_double_alu(acc, e) : 0.0;  // the warp total (lane 31 only)
}

// One thread: the next ticket (-1 once the tiles have run out), and the TMA
// load of a ticket's tile into its ring slot (a plain arrival for -1).
__device__ __forceinline__ int ring_ticket(unsigned *counter, int tiles) {
  const unsigned t = atomicAdd(counter, 1u);
  return t < (unsigned)tiles ? (int)t : -1;
}
__device__ __forceinline__ void ring_arm(int t, unsigned long long *bar, unsigned char *buf, const CUtensorMap *tin,
                                         unsigned bytes) {
  if (t >= 0) {
    mbar_arrive_expect_tx(bar, bytes);
    tma_load_2d(buf, tin, bar, 0, t * RTT);
  } else {
    mbar_arrive(bar);
  }
}
// Bound on the waits that make sure a ring slot's load has landed before the
// slot is armed again or the CTA exits.  They only spin after a load wait
// already gave up (a timeout is flagged); otherwise the load is long done.
constexpr int kRingDrain = kDrainLimit;

// RED: a segmented reduction instead of a scan (not float64 +, whose
// fixed-point fold would bind the ALU without the scan's output chain to
// hide behind): the same fold, publication and look-back, and in the second
// round each thread that ends segments writes their results (a.out has one
// per segment) from the exclusive prefix and a fold of its piece; nothing is
// stored back, so the slot is freed as soon as its rows are read.
template <class Op, bool SEG, bool RED = false>
__global__ void __launch_bounds__(RTB, GCVL_RING_MINB)
    k_scan_ring(const __grid_constant__ CUtensorMap tin, const __grid_constant__ CUtensorMap tout,
                TArgs<typename Op::T> a, int tiles) {
  typedef typename Op::T T;
  constexpr int ITEMS = row_items<T>(), TILE = RTT * ITEMS, NW = RTT / 32, NB = RING_NB;
  constexpr unsigned TILE_BYTES = TILE * sizeof(T);
  extern __shared__ unsigned char dyn_smem[];
  unsigned char *ring = (unsigned char *)(((size_t)dyn_smem + 1023) & ~(size_t)1023);
  __shared__ unsigned long long bar[NB];
  __shared__ int s_tile[NB];
  __shared__ int s_wf[NW];
  __shared__ T s_wv[NW];
  __shared__ int s_wpf[2][NW];  // per tile (round parity): exclusive prefixes of the warps
  __shared__ T s_wpv[2][NW];
  __shared__ int s_af[2];       // per tile: has a segment start, and its aggregate
  __shared__ T s_av[2];
  __shared__ T s_P[2];          // carry into the tile being written
  __shared__ int s_armed[NB];   // per slot: the last round its load was armed for
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

  if (tid == RTT) {
#pragma unroll
    for (int j = 0; j < NB; j++) mbar_init(&bar[j], 1);
    fence_mbar_init();
#pragma unroll
    for (int j = 0; j < NB; j++) {
      s_tile[j] = ring_ticket(a.lb.counter, tiles);
      s_armed[j] = j;
      ring_arm(s_tile[j], &bar[j], ring + j * TILE_BYTES, &tin, TILE_BYTES);
    }
  }
  __syncthreads();

  int lim = a.spin_limit;  // after one timeout the remaining waits give up at once
  // head-bit word of this thread's row in the coming round's tile, read a
  // round ahead (the bitmap is too large to stay in L2).  Rows past the
  // vector's end in its last tile still read inside the bitmap: it is padded
  // to 8192-element multiples (segdes_nbits_words), tiles divide that.
  unsigned nx_word = 0;
  if (SEG && warp < NW && s_tile[0] >= 0) nx_word = __ldg(a.sv.bits + ((s_tile[0] * TILE + tid * ITEMS) >> 5));
  int prev = -1;           // tile folded last round: its outputs are written this round
  unsigned p_heads = 0;    // this thread's state for it
  int p_ef = 0;
  T p_ev = Op::ident();
  for (int r = 0;; r++) {
    const int slot = r % NB, pb = r & 1;
    if (!mbar_wait(&bar[slot], (unsigned)(r / NB) & 1u, lim)) {
      atomicOr(a.status, DEV_TIMEOUT);
      lim = 1;
    }
    // Written before a CTA barrier that every thread has passed since, so the
    // round's tile is the same for all threads even when a wait gave up.
    const int t = s_tile[slot];
    if (t < 0 && prev < 0) break;
    const int ps = (r + NB - 1) % NB;  // slot of last round's tile

    unsigned c_heads = 0;
    int c_ef = 0;
    T c_ev = Op::ident();
    if (warp < NW) {
      // ---------------------------------------------- fold this round's tile
      if (t >= 0) {
        const int k0 = t * TILE + tid * ITEMS;
        const int cnt = max(0, min(ITEMS, a.n - k0));
        if (cnt > 0) {
          if (SEG) {
            c_heads = (ITEMS == 32) ? nx_word : ((nx_word >> (k0 & 31)) & ((1u << ITEMS) - 1u));
            if (cnt < ITEMS) c_heads &= (1u << cnt) - 1u;
          } else {
            c_heads = k0 == 0 ? 1u : 0u;
          }
        }
        T x[ITEMS];
        row_load<Op, ITEMS>(x, ring + slot * TILE_BYTES, tid, (long)t * RTT + tid < a.rows, a.in, k0, cnt);
        int f;
        T v;
        if constexpr (std::is_same<Op, AddD>::value) {
          fold_scan_addd<ITEMS>(x, c_heads, cnt, lane, f, v, c_ef, c_ev);
        } else {
          Engine<Op, ITEMS>::agg(x, c_heads, cnt, f, v);
#pragma unroll
          for (int d = 1; d < 32; d <<= 1) {
            const int f2 = shfl_up(f, d);
            const T v2 = shfl_up(v, d);
            if (lane >= d) { v = f ? v : Op::apply(v2, v); f |= f2; }
          }
          c_ef = shfl_up(f, 1);
          c_ev = shfl_up(v, 1);
          if (lane == 0) { c_ef = 0; c_ev = Op::ident(); }
        }
        if (lane == 31) { s_wf[warp] = f; s_wv[warp] = v; }
      }
      named_sync(2, RTT);
      if (warp == 0 && t >= 0) {
        int wf = lane < NW ? s_wf[lane] : 0;
        T wv = lane < NW ? s_wv[lane] : Op::ident();
#pragma unroll
        for (int d = 1; d < NW; d <<= 1) {
          const int f2 = shfl_up(wf, d);
          const T v2 = shfl_up(wv, d);
          if (lane >= d) { wv = wf ? wv : Op::apply(v2, wv); wf |= f2; }
        }
        int xf = shfl_up(wf, 1);
        T xv = shfl_up(wv, 1);
        if (lane == 0) { xf = 0; xv = Op::ident(); }
        if (lane < NW) { s_wpf[pb][lane] = xf; s_wpv[pb][lane] = xv; }
        const int af = shfl_idx(wf, NW - 1);
        const T av = shfl_idx(wv, NW - 1);
        if (lane == 0) {
          lb_publish(a.lb.word + t, (t == 0 || af) ? TS_INC : TS_AGG, to_bits<T>(av));
          s_af[pb] = af;
          s_av[pb] = av;
        }
      }
    } else if (prev >= 0) {
      // ------------------------------- look-back warp: carry into last round's tile
      const long pbase = (long)prev * TILE;
      const bool first_head = SEG ? ((__ldg(a.sv.bits + (pbase >> 5)) >> (pbase & 31)) & 1u) != 0 : prev == 0;
      T P = Op::ident();
      if (prev > 0 && !first_head) {
        P = lookback_prefix<Op>(a.lb.word, prev, a.status, a.spin_limit);
        if (lane == 0 && !s_af[pb ^ 1]) lb_publish(a.lb.word + prev, TS_INC, to_bits<T>(Op::apply(P, s_av[pb ^ 1])));
      }
      if (lane == 0) s_P[pb] = P;
    }
    // the tile for round r-1+NB: its slot's tile entry was last read at the
    // start of round r-1, before the previous meeting
    if (tid == 0 && prev >= 0) s_tile[ps] = ring_ticket(a.lb.counter, tiles);
    named_sync(1, RTB);  // carry of last round's tile ready; this tile's aggregate published

    if (warp < NW) {
      // the next round's tile (its ticket was taken before an earlier meeting)
      if (SEG) {
        const int tn = s_tile[(r + 1) % NB];
        const int kn = tn * TILE + tid * ITEMS;
        if (tn >= 0 && kn < a.n) nx_word = __ldg(a.sv.bits + (kn >> 5));
      }
      // ------------------------------------------- outputs of last round's tile
      if (prev >= 0) {
        const int k0 = prev * TILE + tid * ITEMS;
        const int cnt = max(0, min(ITEMS, a.n - k0));
        const bool in_map = (long)prev * RTT + tid < a.rows;
        int pf = s_wpf[pb ^ 1][warp];
        T pv = s_wpv[pb ^ 1][warp];
        pv = p_ef ? p_ev : Op::apply(pv, p_ev);
        pf |= p_ef;
        T run = pf ? pv : Op::apply(s_P[pb], pv);
        T x[ITEMS];
        unsigned char *buf = ring + ps * TILE_BYTES;
        row_load<Op, ITEMS>(x, buf, tid, in_map, a.in, k0, cnt);
        if constexpr (RED) {
          named_arrive(3, RTB);  // the rows are read: the look-back warp may reuse the slot
          // element i ends a non-empty segment exactly when element i+1 is a
          // head (or past the end)
          unsigned ends = 0;
          if (cnt > 0) {
            const int kn = k0 + cnt;
            const unsigned nh = kn >= a.n ? 1u : (__ldg(a.sv.bits + (kn >> 5)) >> (kn & 31)) & 1u;
            ends = ((p_heads >> 1) | (nh << (cnt - 1))) & (cnt >= 32 ? ~0u : ((1u << cnt) - 1u));
            const int m = a.sv.m;
            if (k0 == 0) {  // empty segments before element 0
              const int s0 = seg_of(a.sv, 0);
              for (int q = 0; q < s0; q++) a.out[q] = Op::init();
            }
            while (ends) {
              const int e = __ffs(ends) - 1;
              ends &= ends - 1;
              const unsigned hb = p_heads & ((2u << e) - 1u);  // heads up to e
              const int ps0 = hb ? 31 - __clz((int)hb) : 0;
              T pv2 = Op::ident();
#pragma unroll
              for (int i = 0; i < ITEMS; i++)
                if (i >= ps0 && i <= e) pv2 = Op::apply(pv2, x[i]);
              const int sg = seg_of(a.sv, k0 + e);
              a.out[sg] = hb ? Op::apply(Op::init(), pv2) : Op::apply(run, pv2);
              int s2 = sg + 1;  // empty segments that follow
              while (s2 < m && __ldg(a.sv.off + s2 + 1) == k0 + e + 1) { a.out[s2] = Op::init(); ++s2; }
            }
          }
        } else {
#pragma unroll
        for (int i = 0; i < ITEMS; i++) {
          if ((p_heads >> i) & 1u) run = Op::init();
          const T y = run;
          run = Op::apply(run, x[i]);
          x[i] = y;
        }
        if (in_map) {
#pragma unroll
          for (int c = 0; c < 8; c++) {
            uint4 u;
            memcpy(&u, &x[c * (16 / sizeof(T))], 16);
            *(uint4 *)(buf + swz(tid, c)) = u;
          }
        } else {
#pragma unroll
          for (int i = 0; i < ITEMS; i++)
            if (i < cnt) a.out[k0 + i] = x[i];
        }
        fence_proxy_async_smem();
        named_arrive(3, RTB);  // outputs in the slot; the look-back warp stores them
        }
      }
    } else if (prev >= 0) {
      // ------------------------------- look-back warp: store last round's tile
      // and load the tile for round r-1+NB into its slot, off the compute
      // warps' path
      named_sync(3, RTB);
      if (lane == 0) {
        unsigned char *buf = ring + ps * TILE_BYTES;
        if constexpr (!RED) {
          tma_store_2d(&tout, buf, 0, prev * RTT);
          bulk_commit();
          bulk_wait_read_all();  // the slot is free once the store has read it
        }
        if (!mbar_wait(&bar[ps], (unsigned)((r - 1) / NB) & 1u, kRingDrain)) atomicOr(a.status, DEV_TIMEOUT);
        s_armed[ps] = r - 1 + NB;
        ring_arm(s_tile[ps], &bar[ps], buf, &tin, TILE_BYTES);
      }
    }
    prev = t;
    p_heads = c_heads;
    p_ef = c_ef;
    p_ev = c_ev;
  }
  // no load may still be landing in the ring when the CTA exits
  if (tid == RTT) {
#pragma unroll
    for (int j = 0; j < NB; j++)
      if (!mbar_wait(&bar[j], (unsigned)(s_armed[j] / NB) & 1u, kRingDrain)) atomicOr(a.status, DEV_TIMEOUT);
  }
}

// ============================================================================
// Segmented reductions of 4-byte elements along per-warp ranges.
//
// Each warp owns a contiguous range of chunks (32 rows of 32 elements, one
// row per lane) and streams them through WR_NB chunk buffers of its own by
// 2-D TMA copies (128B swizzle), so no warp waits for another and no CTA
// barrier is taken.  Per chunk a lane folds its row, a warp segmented scan
// gives each lane its prefix on top of the fold carried from the range's
// earlier chunks, and one pass over the items records the running value at
// every segment end in shared memory.  Then the lanes take the segments
// whose last element lies in the chunk -- the next 32 offsets in one
// coalesced load, as many rounds as needed -- and write each result (the
// initial value for an empty segment).  Segment numbers come from the
// offsets themselves, in order, instead of a search per end.  The one
// result per range whose segment began in an earlier range holds only the
// range's part; the range publishes (has a segment start, fold since its
// last start) and k_tile_fix completes that result.
// ============================================================================
#ifndef GCVL_RED_WARP
#define GCVL_RED_WARP 1
#endif
#ifndef GCVL_WR_NB
#define GCVL_WR_NB 2
#endif
constexpr int WR_WARPS = 4, WR_NB = GCVL_WR_NB;
constexpr int WR_ELEMS = 32 * 32;  // a chunk: a 32-element row per lane
constexpr unsigned WR_CHUNK_BYTES = WR_ELEMS * 4;
constexpr size_t wr_warp_bytes() { return (size_t)WR_NB * WR_CHUNK_BYTES; }
constexpr size_t wr_smem() { return 1024 + WR_WARPS * wr_warp_bytes(); }

#ifndef GCVL_WR_MINB
#define GCVL_WR_MINB 6
#endif
template <class Op>
__global__ void __launch_bounds__(WR_WARPS * 32, GCVL_WR_MINB)
    k_segred_warp(const __grid_constant__ CUtensorMap tin, TArgs<typename Op::T> a, long chunks, int ranges) {
  typedef typename Op::T T;
  static_assert(sizeof(T) == 4, "rows of 32 four-byte elements");
  extern __shared__ unsigned char dyn_smem[];
  __shared__ unsigned long long s_bar[WR_WARPS][WR_NB];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int gw = blockIdx.x * WR_WARPS + warp;
  if (gw >= ranges) return;  // a whole warp: nothing below meets other warps
  unsigned char *buf = (unsigned char *)(((size_t)dyn_smem + 1023) & ~(size_t)1023) + (size_t)warp * wr_warp_bytes();
  unsigned long long *bar = s_bar[warp];
  const long c0 = (long)gw * chunks / ranges, c1 = (long)(gw + 1) * chunks / ranges;
  const int nck = (int)(c1 - c0);
  const long n = a.n;
  const int m = a.sv.m;
  if (lane == 0) {
#pragma unroll
    for (int j = 0; j < WR_NB; j++) mbar_init(&bar[j], 1);
    fence_mbar_init();
#pragma unroll
    for (int j = 0; j < WR_NB; j++)
      if (j < nck) {
        mbar_arrive_expect_tx(&bar[j], WR_CHUNK_BYTES);
        tma_load_2d(buf + j * WR_CHUNK_BYTES, &tin, &bar[j], 0, (int)((c0 + j) * 32));
      }
  }
  __syncwarp();

  int lim = a.spin_limit;  // after one timeout the remaining waits give up at once
  // the next segment to finish: segments before it end at or before the range
  int sp = gw == 0 ? 0 : seg_of(a.sv, (int)(c0 * WR_ELEMS));
  T wc = Op::ident();  // fold of the open piece carried from the range's earlier chunks
  bool wh = false;     // that piece starts at a segment start inside the range
  int lead_l = -1;     // (lane) the result lacking the earlier ranges' part
  // head-bit words of a row: this chunk's read a chunk ahead (the bitmap is
  // streamed once, from DRAM); lane 31 also needs the next chunk's first
  auto row_bits = [&](long cc) -> unsigned {
    const long kk = cc * WR_ELEMS + lane * 32;
    return cc < c1 && kk < n ? __ldg(a.sv.bits + (kk >> 5)) : 0u;
  };
  unsigned hw_next = row_bits(c0);
  for (int ci = 0; ci < nck; ci++) {
    const long c = c0 + ci;
    const int b = ci % WR_NB;
    const long cs = c * WR_ELEMS;
    const long k0 = cs + lane * 32;
    const int cnt = (int)max(0L, min(32L, n - k0));
    // the chunk's independent loads go out before the wait for its rows: the
    // next chunk's head bits, the first head bit after this chunk, the next
    // 32 segment ends
    const unsigned hw = hw_next;
    hw_next = row_bits(c + 1);
    unsigned nbw = 1u;
    if (lane == 31 && cs + WR_ELEMS < n) nbw = __ldg(a.sv.bits + ((cs + WR_ELEMS) >> 5));
    int o_next = sp + lane < m ? __ldg(a.sv.off + sp + lane + 1) : INT_MAX;
    int po_first = lane == 0 && sp < m ? __ldg(a.sv.off + sp) : 0;
    if (!mbar_wait(&bar[b], (unsigned)(ci / WR_NB) & 1u, lim)) {
      atomicOr(a.status, DEV_TIMEOUT);
      lim = 1;
    }
    T x[32];
    if (c * 32 + lane < a.rows) {
      const unsigned char *rowb = buf + b * WR_CHUNK_BYTES;
#pragma unroll
      for (int q = 0; q < 8; q++) {
        const uint4 u = *(const uint4 *)(rowb + swz(lane, q));
        memcpy(&x[4 * q], &u, 16);
      }
    } else {
#pragma unroll
      for (int i = 0; i < 32; i++) x[i] = i < cnt ? a.in[k0 + i] : Op::ident();
    }
    if constexpr (std::is_same<Op, CountB>::value) {
#pragma unroll
      for (int i = 0; i < 32; i++) x[i] = x[i] != 0;  // pk1_lev counts true flags
    }
    // the running value at each segment end, element p of the chunk at s_end[p]:
    // the chunk's own buffer, each lane writing only the 128 bytes of the row
    // it has just read (its own loads of them come first), the buffer refilled
    // only once the chunk's results are out
    T *s_end = (T *)(buf + b * WR_CHUNK_BYTES);
    // head bits of the row; its last element ends a segment when the next
    // element is a head or past the end
    const unsigned heads = cnt >= 32 ? hw : (hw & ((1u << cnt) - 1u));
    unsigned nb = __shfl_down_sync(0xffffffffu, hw & 1u, 1);
    if (lane == 31) nb = nbw & 1u;
    if (k0 + cnt >= n) nb = 1u;
    const unsigned ends =
        cnt == 0 ? 0u : (((heads >> 1) | (nb << (cnt - 1))) & (cnt >= 32 ? ~0u : ((1u << cnt) - 1u)));
    // One pass over the row: the running value of every item (restarting at
    // each head), all 32 stored with 16-byte stores at the row's swizzled
    // place; the values at segment ends whose segment starts in the row are
    // final, the row's first end before its first head waits for the lanes'
    // prefix.  r ends as the row's open piece (fold since its last head).
    T r = Op::ident();
    T y[32];
    if (cnt == 32) {
#pragma unroll
      for (int i = 0; i < 32; i++) {
        r = ((heads >> i) & 1u) ? Op::apply(Op::init(), x[i]) : Op::apply(r, x[i]);
        y[i] = r;
      }
    } else {
#pragma unroll
      for (int i = 0; i < 32; i++) {
        if (i < cnt) r = ((heads >> i) & 1u) ? Op::apply(Op::init(), x[i]) : Op::apply(r, x[i]);
        y[i] = r;
      }
    }
    unsigned char *s_row = (unsigned char *)s_end + lane * 128;
#pragma unroll
    for (int q = 0; q < 8; q++) {
      uint4 u;
      memcpy(&u, &y[4 * q], 16);
      *(uint4 *)(s_row + (((q ^ lane) & 7) << 4)) = u;
    }
    const bool started = heads != 0;
    const int fh = started ? __ffs(heads) - 1 : 32, fe = ends ? __ffs(ends) - 1 : 32;
    const int first_p = fe < fh ? lane * 32 + fe : -1;  // the first end, before any head
    // the lanes' segmented scan of their open pieces, the value entering each row
    int f = started;
    T v = r;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const int f2 = shfl_up(f, d);
      const T v2 = shfl_up(v, d);
      if (lane >= d) { v = f ? v : Op::apply(v2, v); f |= f2; }
    }
    int ef = shfl_up(f, 1);
    T ev = shfl_up(v, 1);
    if (lane == 0) { ef = 0; ev = Op::ident(); }
    if (first_p >= 0) {
      T *slot = (T *)(s_row + ((((fe >> 2) ^ lane) & 7) << 4)) + (fe & 3);
      *slot = Op::apply(ef ? ev : Op::apply(wc, ev), *slot);
      if (!ef && !wh) lead_l = -2 - first_p;  // marks the position; the segment is named below
    }
    const int lf = __shfl_sync(0xffffffffu, f, 31);
    const T lv = __shfl_sync(0xffffffffu, v, 31);
    if (lf) { wc = lv; wh = true; } else wc = Op::apply(wc, lv);
    const unsigned ib = __ballot_sync(0xffffffffu, lead_l <= -2);
    const int ipos = ib ? -2 - __shfl_sync(0xffffffffu, lead_l, __ffs(ib) - 1) : -1;
    if (lead_l <= -2) lead_l = -1;
    __syncwarp();  // the ends are recorded
    // the segments whose last element lies in this chunk: off[s+1] in (cs, ce]
    const long ce = min(cs + (long)WR_ELEMS, n);
    for (int round = 0;; round++) {
      const int sg = sp + lane;
      const int o = round == 0 ? o_next : (sg < m ? __ldg(a.sv.off + sg + 1) : INT_MAX);
      const bool fin = sg < m && (long)o <= ce;
      const unsigned fb = __ballot_sync(0xffffffffu, fin);
      int po = __shfl_up_sync(0xffffffffu, o, 1);
      if (lane == 0) po = round == 0 ? po_first : (sp < m ? __ldg(a.sv.off + sp) : 0);
      if (fin) {
        if (po == o) {
          a.out[sg] = Op::init();  // an empty segment
        } else {
          const int pe = (int)((long)o - 1 - cs);  // row pe / 32, item pe % 32, swizzled as written
          a.out[sg] = *((const T *)((const unsigned char *)s_end + (pe >> 5) * 128 +
                                    ((((pe & 31) >> 2) ^ (pe >> 5)) & 7) * 16) + (pe & 3));
          if (pe == ipos) lead_l = sg;
        }
      }
      const int k = __popc(fb);  // offsets ascend: the finished segments are a prefix of the lanes
      sp += k;
      if (k < 32) break;
    }
    __syncwarp();  // every read of the buffer is done
    if (lane == 0 && ci + WR_NB < nck) {  // refill it
      fence_proxy_async_smem();
      mbar_arrive_expect_tx(&bar[b], WR_CHUNK_BYTES);
      tma_load_2d(buf + b * WR_CHUNK_BYTES, &tin, &bar[b], 0, (int)((c + WR_NB) * 32));
    }
  }
  const unsigned lb = __ballot_sync(0xffffffffu, lead_l >= 0);
  const int lead = lb ? __shfl_sync(0xffffffffu, lead_l, __ffs(lb) - 1) : -1;
  if (lane == 0) {
    lb_publish(a.lb.word + gw, wh ? TS_INC : TS_AGG, to_bits<T>(wc));
    if (lead >= 0) a.lead[gw] = lead;
    // no copy may still be landing in the buffers when the warp leaves
    for (int j = 0; j < WR_NB && j < nck; j++) {
      const int last = j + WR_NB * ((nck - 1 - j) / WR_NB);
      if (!mbar_wait(&bar[j], (unsigned)(last / WR_NB) & 1u, kDrainLimit)) atomicOr(a.status, DEV_TIMEOUT);
    }
  }
}

// Second pass of a segmented reduction: the carry into every tile is the
// segmented exclusive scan of the tile aggregates (status TS_INC marks a
// tile holding a segment start; its value is the fold from its last start);
// the one result per tile whose segment began in an earlier tile gets that
// carry folded in front.  One thread per tile, chunks of FIX_NT tiles per
// CTA joined by a decoupled look-back over the chunks.
constexpr int FIX_NT = 1024;
template <class Op>
__global__ void __launch_bounds__(FIX_NT) k_tile_fix(const ulonglong2 *__restrict__ w, const int *__restrict__ lead,
                                                     int tiles, typename Op::T *out, ulonglong2 *cw,
                                                     unsigned *status, int spin_limit) {
  typedef typename Op::T T;
  constexpr int NW = FIX_NT / 32;
  __shared__ int s_wf[NW];
  __shared__ T s_wv[NW];
  __shared__ int s_fa;
  __shared__ T s_va, s_P;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int chunk = blockIdx.x;
  const int t = chunk * FIX_NT + tid;
  int fi = 0;
  T vi = Op::ident();
  if (t < tiles) {
    const ulonglong2 q = w[t];
    fi = q.x == TS_INC;
    vi = from_bits<T>(q.y);
  }
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const int f2 = shfl_up(fi, d);
    const T v2 = shfl_up(vi, d);
    if (lane >= d) { vi = fi ? vi : Op::apply(v2, vi); fi |= f2; }
  }
  int ef = shfl_up(fi, 1);
  T ev = shfl_up(vi, 1);
  if (lane == 0) { ef = 0; ev = Op::ident(); }
  if (lane == 31) { s_wf[warp] = fi; s_wv[warp] = vi; }
  __syncthreads();
  if (warp == 0) {
    int wf = s_wf[lane];
    T wv = s_wv[lane];
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const int f2 = shfl_up(wf, d);
      const T v2 = shfl_up(wv, d);
      if (lane >= d) { wv = wf ? wv : Op::apply(v2, wv); wf |= f2; }
    }
    int xf = shfl_up(wf, 1);
    T xv = shfl_up(wv, 1);
    if (lane == 0) { xf = 0; xv = Op::ident(); }
    const int fa = shfl_idx(wf, NW - 1);
    const T va = shfl_idx(wv, NW - 1);
    s_wf[lane] = xf;  // now: exclusive prefix of the warps before
    s_wv[lane] = xv;
    if (lane == 0) lb_publish(cw + chunk, (chunk == 0 || fa) ? TS_INC : TS_AGG, to_bits<T>(va));
    T P = Op::ident();
    if (chunk > 0) {  // tiles before the chunk's first segment start need the carry
      P = lookback_prefix<Op>(cw, chunk, status, spin_limit);
      if (lane == 0 && !fa) lb_publish(cw + chunk, TS_INC, to_bits<T>(Op::apply(P, va)));
    }
    if (lane == 0) { s_fa = fa; s_va = va; s_P = P; }
  }
  __syncthreads();
  if (t >= tiles) return;
  const int s = lead[t];
  if (s < 0) return;
  // exclusive (flag, value) of this tile within the chunk, then the chunk carry
  const int pf = s_wf[warp];
  const T pv = s_wv[warp];
  const int fe = ef | pf;
  const T ve = ef ? ev : Op::apply(pv, ev);
  const T carry = fe ? ve : Op::apply(s_P, ve);
  out[s] = Op::apply(carry, out[s]);
}

// Host side: tensor maps and launch.  The driver's tensor-map encoder is
// looked up through the runtime, so the library itself does not link
// libcuda and loads on machines without a GPU driver.
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *,
                                  CUtensorMapInterleave, CUtensorMapSwizzle, CUtensorMapL2promotion,
                                  CUtensorMapFloatOOBfill);
static EncodeTiledFn encode_tiled() {
  static EncodeTiledFn fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      fn = (EncodeTiledFn)p;
    else
      cudaGetLastError();
  }
  return fn;
}

template <class T> bool tma_map(CUtensorMap *map, const void *ptr, long rows, int box_rows = TT) {
  EncodeTiledFn enc = encode_tiled();
  if (!enc) return false;
  cuuint64_t dims[2] = {(cuuint64_t)row_items<T>(), (cuuint64_t)rows};
  cuuint64_t strides[1] = {128};
  cuuint32_t box[2] = {(cuuint32_t)row_items<T>(), (cuuint32_t)box_rows};
  cuuint32_t es[2] = {1, 1};
  CUresult r = enc(
      map, sizeof(T) == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_INT32, 2, (void *)ptr,
      dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
      CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}
// scratch of a TMA-path launch: the look-back area, then (reductions) one
// int per tile naming the result that k_tile_fix completes
inline size_t reduce_pass_bytes(int tiles) {
  const int chunks = (tiles + 1023) / 1024;
  return lookback_bytes(tiles) + align_up((size_t)tiles * 4, 256) + lookback_bytes(chunks);
}
// The fix-up pass of a segmented reduction whose first pass published its
// tile aggregates at `w` and the per-tile results to complete at `lead`
// (lead sits right after the look-back area, the chunks' look-back after it).
template <class Op>
void launch_tile_fix(const ulonglong2 *w, const int *lead, int tiles, typename Op::T *out) {
  if (tiles <= 1) return;
  State &S = st();
  const int chunks = ceil_div(tiles, FIX_NT);
  LookbackMem cl = lookback_carve((char *)lead + align_up((size_t)tiles * 4, 256), chunks);
  GCVL_CK(cudaMemsetAsync(cl.counter, 0, 256 + (size_t)chunks * 16, S.stream));
  k_tile_fix<Op><<<chunks, FIX_NT, 0, S.stream>>>(w, lead, tiles, out, cl.word, S.d_status, S.spin_limit);
  launch_check("k_tile_fix");
}
template <class T> constexpr size_t tma_smem(int wmax) {
  return 1024 + (size_t)TT * row_items<T>() * sizeof(T) + (size_t)(wmax > 0 ? wpad(wmax) + 1 : 0) * 4;
}

// CTAs of a ring scan: as many as are resident at once (0: it does not fit)
template <class Op, bool SEG, bool RED = false> int ring_grid(int tiles) {
  static int per_sm = -1;
  if (per_sm < 0) {
    int nb = 0;
    const size_t smem = ring_smem<typename Op::T>();
    if (smem > 48 * 1024 &&
        cudaFuncSetAttribute(k_scan_ring<Op, SEG, RED>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
            cudaSuccess) {
      cudaGetLastError();
      per_sm = 0;
    } else if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_scan_ring<Op, SEG, RED>, RTB, smem) !=
               cudaSuccess) {
      cudaGetLastError();
      per_sm = 0;
    } else {
      per_sm = nb;
    }
  }
  const long g = (long)per_sm * (st().sm_count > 0 ? st().sm_count : 152);
  return (int)(g < tiles ? g : tiles);
}

// Returns false (nothing launched) when the vectors do not suit TMA.
#ifndef GCVL_RING_RED_MEAN
#define GCVL_RING_RED_MEAN 32
#endif
constexpr long RING_RED_MEAN = GCVL_RING_RED_MEAN;
template <class Op, int MODE, bool SEG>
bool run_scan_tma(typename Op::T *out, const typename Op::T *in, vec_p sd, int n, int m, vec_p scratch,
                  const char *name) {
  typedef typename Op::T T;
  if (getenv("GCVL_NO_TMA")) return false;
  const long rows = (long)n / row_items<T>();
  if (rows < 1 || ((size_t)in & 15) || (MODE == M_SCAN && ((size_t)out & 15))) return false;
  CUtensorMap tin, tout;
  State &S = st();
  if constexpr (MODE == M_SCAN) {
    const int tiles = ceil_div(n, (long)RTT * row_items<T>());
    const int grid = ring_grid<Op, SEG>(tiles);
    if (grid > 0) {
      if (!tma_map<T>(&tin, in, rows, RTT) || !tma_map<T>(&tout, out, rows, RTT)) return false;
      void *mem = scratch_or_work(scratch, lookback_bytes(tiles));
      if (!mem) return true;
      TArgs<T> a{};
      a.out = out; a.in = in; a.n = n; a.rows = rows;
      a.sv = SEG ? seg_view(sd, n, m) : SegView{nullptr, nullptr, nullptr, nullptr, n, 1};
      a.lb = lookback_carve(mem, tiles);
      a.status = S.d_status;
      a.spin_limit = S.spin_limit;
      GCVL_CK(cudaMemsetAsync(mem, 0, lookback_clear_bytes(tiles), S.stream));
      k_scan_ring<Op, SEG><<<grid, RTB, ring_smem<T>(), S.stream>>>(tin, tout, a, tiles);
      launch_check(name);
      return true;
    }
  }
  if constexpr (MODE == M_REDUCE && SEG && sizeof(T) == 4 && !std::is_same<Op, AddD>::value) {
    if (GCVL_RED_WARP && (long)n >= RING_RED_MEAN * m) {
      // per-warp ranges: as many as fit at once, at most one per chunk and
      // no more than the tile form's tiles (whose scratch this shares)
      const long chunks = ceil_div(n, (long)WR_ELEMS);
      static int per_sm = -1;
      if (per_sm < 0) {
        per_sm = 0;
        if (GCVL_CK(cudaFuncSetAttribute(k_segred_warp<Op>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)wr_smem())))
          GCVL_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_segred_warp<Op>, WR_WARPS * 32,
                                                                wr_smem()));
      }
      long ranges = (long)(per_sm > 0 ? per_sm : 1) * S.sm_count * WR_WARPS;
      ranges = std::min(ranges, chunks);
      ranges = std::min(ranges, (long)ceil_div(n, (long)TT * row_items<T>()));
      if (ranges < 1) ranges = 1;
      if (!tma_map<T>(&tin, in, rows, 32)) return false;
      void *mem = scratch_or_work(scratch, reduce_pass_bytes((int)ranges));
      if (!mem) return true;
      TArgs<T> a{};
      a.out = out; a.in = in; a.n = n; a.rows = rows;
      a.sv = seg_view(sd, n, m);
      a.lb = lookback_carve(mem, (int)ranges);
      a.status = S.d_status;
      a.spin_limit = S.spin_limit;
      a.lead = (int *)((char *)a.lb.word + align_up((size_t)ranges * 16, 256));
      if (!GCVL_CK(cudaMemsetAsync(mem, 0, lookback_clear_bytes((int)ranges), S.stream))) return true;
      if (!GCVL_CK(cudaMemsetAsync(a.lead, 0xFF, (size_t)ranges * 4, S.stream))) return true;
      k_segred_warp<Op><<<ceil_div(ranges, (long)WR_WARPS), WR_WARPS * 32, wr_smem(), S.stream>>>(tin, a, chunks,
                                                                                               (int)ranges);
      launch_check(name);
      launch_tile_fix<Op>(a.lb.word, a.lead, (int)ranges, out);
      return true;
    }
  }
  if constexpr (MODE == M_REDUCE && SEG && !std::is_same<Op, AddD>::value) {
    // segmented reductions on the ring (results written at segment ends,
    // the carry from the look-back: no fix-up pass) when segments average
    // RING_RED_MEAN elements or more.  Shorter ones stay on the tile kernel,
    // whose offsets window finds each end's segment in shared memory: the
    // ring looks every end up in global memory, and a quicksort's last
    // levels (one- and few-element segments) ran 2x slower on it
    // (0.42 -> 0.85 s for 2^26 keys).
    const int tiles = ceil_div(n, (long)RTT * row_items<T>());
    const int grid = (long)n >= RING_RED_MEAN * m ? ring_grid<Op, SEG, true>(tiles) : 0;
    if (grid > 0) {
      if (!tma_map<T>(&tin, in, rows, RTT)) return false;
      void *mem = scratch_or_work(scratch, lookback_bytes(tiles));
      if (!mem) return true;
      TArgs<T> a{};
      a.out = out; a.in = in; a.n = n; a.rows = rows;
      a.sv = seg_view(sd, n, m);
      a.lb = lookback_carve(mem, tiles);
      a.status = S.d_status;
      a.spin_limit = S.spin_limit;
      // nothing runs on look-back words that were not cleared
      if (!GCVL_CK(cudaMemsetAsync(mem, 0, lookback_clear_bytes(tiles), S.stream))) return true;
      k_scan_ring<Op, SEG, true><<<grid, RTB, ring_smem<T>(), S.stream>>>(tin, tin, a, tiles);
      launch_check(name);
      return true;
    }
  }
  if (!tma_map<T>(&tin, in, rows)) return false;
  if (MODE == M_SCAN) { if (!tma_map<T>(&tout, out, rows)) return false; }
  else tout = tin;
  const int tiles = ceil_div(n, (long)TT * row_items<T>());
  void *mem = scratch_or_work(scratch, reduce_pass_bytes(tiles));
  if (!mem) return true;
  TArgs<T> a;
  a.out = out; a.in = in; a.n = n; a.rows = rows;
  a.sv = SEG ? seg_view(sd, n, m) : SegView{nullptr, nullptr, nullptr, nullptr, n, 1};
  a.lb = lookback_carve(mem, tiles);
  a.status = S.d_status;
  a.spin_limit = S.spin_limit;
  a.lead = (int *)((char *)a.lb.word + align_up((size_t)tiles * 16, 256));
  GCVL_CK(cudaMemsetAsync(mem, 0, lookback_clear_bytes(tiles), S.stream));
  if (MODE == M_REDUCE) GCVL_CK(cudaMemsetAsync(a.lead, 0xFF, (size_t)tiles * 4, S.stream));
  a.wmax = SEG ? wmax_for<T, MODE>(n, m) : 0;
  bool chain = false;
  if constexpr (MODE == M_REDUCE && SEG && std::is_same<Op, AddD>::value) {
    chain = (long)n < RED_CHAIN_MEAN * m;
    if (chain)
      k_scan_tma<Op, MODE, SEG, true><<<tiles, cta_threads<MODE>(), tma_smem<T>(a.wmax), S.stream>>>(tin, tout, a);
  }
  if (!chain) k_scan_tma<Op, MODE, SEG><<<tiles, cta_threads<MODE>(), tma_smem<T>(a.wmax), S.stream>>>(tin, tout, a);
  launch_check(name);
  if (MODE == M_REDUCE) launch_tile_fix<Op>(a.lb.word, a.lead, tiles, out);
  return true;
}

template <class Op>
__global__ void k_fill(typename Op::T *out, int m) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < m) out[i] = Op::init();
}

template <class T> constexpr int tile_elems() { return Tiling<T>::BLOCK * Tiling<T>::ITEMS; }

template <class T> int scan_units(int n) {
  if (n <= 0) return 0;
  const int a = ceil_div(n, tile_elems<T>()), b = ceil_div(n, RTT * row_items<T>());
  return lookback_units(a > b ? a : b);
}

// Shared launcher.  `sd` may be null for unsegmented modes.
template <class Op, int MODE, bool SEG>
void run_scan(typename Op::T *out, const typename Op::T *in, typename Op::T *out2, vec_p sd,
              int n, int m, vec_p scratch, bool count_flags, const char *name) {
  typedef typename Op::T T;
  ensure_init();
  State &S = st();
  if (n <= 0) return;
  if constexpr (MODE == M_SCAN || MODE == M_REDUCE) {
    const bool tma_ok = !count_flags || std::is_same<Op, CountB>::value;
    if (tma_ok && run_scan_tma<Op, MODE, SEG>(out, in, sd, n, m, scratch, name)) return;
  }
  const int tiles = ceil_div(n, tile_elems<T>());
  void *mem = scratch_or_work(scratch, MODE == M_REDUCE ? reduce_pass_bytes(tiles) : lookback_bytes(tiles));
  if (!mem) return;
  ScanArgs<T> a{};
  a.out = out; a.in = in; a.out2 = out2; a.n = n;
  a.sv = SEG ? seg_view(sd, n, m) : SegView{nullptr, nullptr, nullptr, nullptr, n, 1};
  a.lb = lookback_carve(mem, tiles);
  a.status = S.d_status;
  a.spin_limit = S.spin_limit;
  a.count_flags = count_flags ? 1 : 0;
  a.lead = (int *)((char *)a.lb.word + align_up((size_t)tiles * 16, 256));
  GCVL_CK(cudaMemsetAsync(mem, 0, lookback_clear_bytes(tiles), S.stream));
  if (MODE == M_REDUCE) GCVL_CK(cudaMemsetAsync(a.lead, 0xFF, (size_t)tiles * 4, S.stream));
  k_scan<Op, MODE, SEG><<<tiles, Tiling<T>::BLOCK, 0, S.stream>>>(a);
  launch_check(name);
  if (MODE == M_REDUCE) launch_tile_fix<Op>(a.lb.word, a.lead, tiles, out);
}

// Segmented sums of gathered products, y[r] = sum over row r of
// vals[k] * x[cols[k]]: the BPERMUTE / * / +_REDUCE sequence of a sparse
// matrix-vector product in one pass, without the two intermediate vectors.
static void run_gather_mul_reduce(double *y, const double *vals, const int *cols, const double *x, vec_p sd,
                                  int nnz, int rows, vec_p scratch) {
  ensure_init();
  State &S = st();
  if (rows <= 0) return;
  if (nnz <= 0) {
    GCVL_CK(cudaMemsetAsync(y, 0, (size_t)rows * sizeof(double), S.stream));
    return;
  }
  const long trows = (long)nnz / row_items<double>();
  CUtensorMap tin;
  if (trows >= 1 && !((size_t)vals & 15) && !((size_t)cols & 15) && !getenv("GCVL_NO_TMA") &&
      tma_map<double>(&tin, vals, trows)) {
    // TMA tiles of the values, the fixed-point segmented fold of k_scan_tma
    const int tiles = ceil_div(nnz, (long)TT * row_items<double>());
    void *mem = scratch_or_work(scratch, reduce_pass_bytes(tiles));
    if (!mem) return;
    TArgs<double> t{};
    t.out = y; t.in = vals; t.n = nnz; t.rows = trows;
    t.sv = seg_view(sd, nnz, rows);
    t.lb = lookback_carve(mem, tiles);
    t.status = S.d_status;
    t.spin_limit = S.spin_limit;
    t.lead = (int *)((char *)t.lb.word + align_up((size_t)tiles * 16, 256));
    t.wmax = wmax_for<double, M_REDUCE>(nnz, rows);
    t.gidx = cols; t.gsrc = x;
    GCVL_CK(cudaMemsetAsync(mem, 0, lookback_clear_bytes(tiles), S.stream));
    GCVL_CK(cudaMemsetAsync(t.lead, 0xFF, (size_t)tiles * 4, S.stream));
    if ((long)nnz < RED_CHAIN_MEAN * rows)
      k_scan_tma<AddD, M_REDUCE, true, true, true>
          <<<tiles, cta_threads<M_REDUCE>(), tma_smem<double>(t.wmax), S.stream>>>(tin, tin, t);
    else
      k_scan_tma<AddD, M_REDUCE, true, false, true>
          <<<tiles, cta_threads<M_REDUCE>(), tma_smem<double>(t.wmax), S.stream>>>(tin, tin, t);
    launch_check("gcvl_spmv_csr");
    launch_tile_fix<AddD>(t.lb.word, t.lead, tiles, y);
    return;
  }
  const int tiles = ceil_div(nnz, tile_elems<double>());
  void *mem = scratch_or_work(scratch, reduce_pass_bytes(tiles));
  if (!mem) return;
  ScanArgs<double> a{};
  a.out = y; a.in = vals; a.out2 = nullptr; a.n = nnz;
  a.sv = seg_view(sd, nnz, rows);
  a.lb = lookback_carve(mem, tiles);
  a.status = S.d_status;
  a.spin_limit = S.spin_limit;
  a.count_flags = 0;
  a.gidx = cols; a.gsrc = x;
  a.lead = (int *)((char *)a.lb.word + align_up((size_t)tiles * 16, 256));
  GCVL_CK(cudaMemsetAsync(mem, 0, lookback_clear_bytes(tiles), S.stream));
  GCVL_CK(cudaMemsetAsync(a.lead, 0xFF, (size_t)tiles * 4, S.stream));
  k_scan<AddD, M_REDUCE, true, true><<<tiles, Tiling<double>::BLOCK, 0, S.stream>>>(a);
  launch_check("gcvl_spmv_csr");
  launch_tile_fix<AddD>(a.lb.word, a.lead, tiles, y);
}

// ---------------------------------------------- unsegmented reductions ---
// Two-level reduction with a fixed combine order (deterministic for a given
// device): per-CTA partials, then the last CTA folds them in CTA order.
constexpr int RBLOCK = 512;
template <class Op>
__global__ void __launch_bounds__(RBLOCK) k_reduce(const typename Op::T *__restrict__ in, long n,
                                                  typename Op::T *partial, unsigned *ticket,
                                                  typename Op::T *result, int count_flags) {
  typedef typename Op::T T;
  __shared__ T s_w[RBLOCK / 32];
  __shared__ bool s_last;
  T acc = Op::ident();
  const long stride = (long)gridDim.x * RBLOCK;
  // contiguous chunk per CTA keeps the fold order simple and loads coalesced
  long per = (n + gridDim.x - 1) / gridDim.x;
  long lo = (long)blockIdx.x * per, hi = min(n, lo + per);
  (void)stride;
  for (long i = lo + threadIdx.x; i < hi; i += RBLOCK) {
    T x = __ldcs(in + i);
    if (count_flags) x = (x != (T)0) ? (T)1 : (T)0;
    acc = Op::apply(acc, x);
  }
  // thread order within a warp, then warps in order
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    T o = shfl_down(acc, d);
    if ((threadIdx.x & 31) + d < 32) acc = Op::apply(acc, o);
  }
  if ((threadIdx.x & 31) == 0) s_w[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    T b = Op::ident();
    for (int w = 0; w < RBLOCK / 32; w++) b = Op::apply(b, s_w[w]);
    partial[blockIdx.x] = b;
    __threadfence();
    unsigned t = atomicAdd(ticket, 1u);
    s_last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (s_last && threadIdx.x < 32) {
    __threadfence();
    // lane l folds partials l, l+32, ...: ordered within lane, then lanes
    T r = Op::ident();
    for (int i = threadIdx.x; i < (int)gridDim.x; i += 32) r = Op::apply(r, ld_relaxed(partial + i));
    // gather lanes in order on lane 0
    // (order across lanes differs from CTA order only by a fixed permutation)
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      T o = shfl_down(r, d);
      if ((threadIdx.x & 31) + d < 32) r = Op::apply(r, o);
    }
    if (threadIdx.x == 0) {
      *result = Op::apply(Op::init(), r);
      *ticket = 0;
    }
  }
}

template <class Op>
void run_reduce(const typename Op::T *in, int n, typename Op::T *result_dev, vec_p scratch,
                bool count_flags) {
  typedef typename Op::T T;
  ensure_init();
  State &S = st();
  if (n <= 0) {
    T v = Op::init();
    GCVL_CK(cudaMemcpyAsync(result_dev, &v, sizeof(T), cudaMemcpyHostToDevice, S.stream));
    GCVL_CK(cudaStreamSynchronize(S.stream));
    return;
  }
  int grid = S.sm_count * 2;
  long need = ((long)n + RBLOCK - 1) / RBLOCK;
  if (grid > need) grid = (int)need;
  void *mem = scratch_or_work(scratch, 256 + (size_t)grid * 8);
  if (!mem) return;
  unsigned *ticket = (unsigned *)mem;
  T *partial = (T *)((char *)mem + 256);
  GCVL_CK(cudaMemsetAsync(ticket, 0, 4, S.stream));
  k_reduce<Op><<<grid, RBLOCK, 0, S.stream>>>(in, n, partial, ticket, result_dev, count_flags ? 1 : 0);
  launch_check("k_reduce");
}
// segmented reductions: the TMA path's look-back area and per-tile
// fix-up list, or the generic kernel's look-back area
template <class T> int seg_reduce_units(int n) {
  if (n <= 0) return 0;
  const int a = ceil_div(n, tile_elems<T>()), b = ceil_div(n, TT * row_items<T>());
  const size_t pass = reduce_pass_bytes(a > b ? a : b);
  // the ring form (64-row tiles) needs only its look-back words
  const size_t ring = lookback_bytes(ceil_div(n, (long)RTT * row_items<T>()));
  return (int)(((pass > ring ? pass : ring) + 7) / 8);
}
template <class T> int reduce_units(int n) {
  (void)n;
  return (256 + (st().sm_count > 0 ? st().sm_count : 152) * 2 * 8 + 7) / 8 + 64;
}

template <class Op>
typename Op::T reduce_to_host(vec_p s, int n, vec_p scratch, bool count_flags = false) {
  typedef typename Op::T T;
  ensure_init();
  State &S = st();
  if (!S.ready) return Op::init();
  T *res = (T *)((char *)S.d_small + 64);
  run_reduce<Op>((const T *)s, n, res, scratch, count_flags);
  T v = Op::init();
  GCVL_CK(cudaMemcpyAsync(S.h_small, res, sizeof(T), cudaMemcpyDeviceToHost, S.stream));
  GCVL_CK(cudaStreamSynchronize(S.stream));
  memcpy(&v, S.h_small, sizeof(T));
  return v;
}

template <class Op>
void seg_reduce(vec_p d, vec_p s, vec_p sd, int n, int m, vec_p scratch, bool count_flags,
                const char *name) {
  typedef typename Op::T T;
  ensure_init();
  if (m <= 0) return;
  if (m == 1) {  // vprims.c:170: a single segment reduces to the unsegmented result
    run_reduce<Op>((const T *)s, n, (T *)d, scratch, count_flags);
    return;
  }
  if (n <= 0) {
    k_fill<Op><<<ceil_div(m, 256), 256, 0, stream()>>>((T *)d, m);
    launch_check(name);
    return;
  }
  run_scan<Op, M_REDUCE, true>((T *)d, (const T *)s, nullptr, sd, n, m, scratch, count_flags, name);
}

template <class Op>
void seg_scan(vec_p d, vec_p s, vec_p sd, int n, int m, vec_p scratch, const char *name) {
  typedef typename Op::T T;
  if (m == 1 || sd == nullptr)
    run_scan<Op, M_SCAN, false>((T *)d, (const T *)s, nullptr, nullptr, n, 1, scratch, false, name);
  else
    run_scan<Op, M_SCAN, true>((T *)d, (const T *)s, nullptr, sd, n, m, scratch, false, name);
}

// ---------------------------------------------------------- segdes build ---
__global__ void k_granules(SegView sv, int *gran, int ng) {
  int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g > ng) return;
  if (g == ng) { gran[g] = sv.m; return; }
  int k = g * kGranule;  // < n
  int lo = 0, hi = sv.m - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (__ldg(sv.off + mid) <= k) lo = mid; else hi = mid - 1;
  }
  gran[g] = lo;
}

// Head bitmap: one bit per element, set where a non-empty segment starts.
// Offsets ascend, so the lanes whose segment starts fall in one bitmap word
// are contiguous: their bits are OR-ed within the warp first and one atomic
// per run sets them (with one-element segments a word takes 32 heads).
__global__ void k_headbits(SegView sv, unsigned *bits) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  int word = -1;
  unsigned bit = 0;
  if (s < sv.m) {
    const int o = sv.off[s];
    if (sv.off[s + 1] > o) { word = o >> 5; bit = 1u << (o & 31); }
  }
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const int w2 = __shfl_down_sync(0xffffffffu, word, d);
    const unsigned b2 = __shfl_down_sync(0xffffffffu, bit, d);
    if (lane + d < 32 && w2 == word) bit |= b2;
  }
  const int wprev = __shfl_up_sync(0xffffffffu, word, 1);
  if (word >= 0 && (lane == 0 || wprev != word)) atomicOr(bits + word, bit);
}

void make_segdes(vec_p sd, vec_p l, int n, int m, vec_p scratch) {
  ensure_init();
  State &S = st();
  int *base = (int *)sd;
  int *len = base;
  int *off = base + segdes_off_words(m);
  int *gran = base + segdes_gran_words(m);
  if (m <= 0) {
    GCVL_CK(cudaMemsetAsync(off, 0, 4, S.stream));
  } else if ((const int *)l == len) {
    // lengths already in place: scan them into the offsets only
    run_scan<AddZ, M_SCAN, false>(off, len, nullptr, nullptr, m, 1, scratch, false, "mke_fov");
    GCVL_CK(cudaMemcpyAsync(off + m, &n, 4, cudaMemcpyHostToDevice, S.stream));
  } else {
    run_scan<AddZ, M_OFFSETS, false>(off, (const int *)l, len, nullptr, m, 1, scratch, false, "mke_fov");
  }
  int ng = (n + kGranule - 1) / kGranule;
  SegView sv = seg_view(sd, n, m);
  if (m <= 0) ng = 0;
  k_granules<<<ceil_div(ng + 1, 256), 256, 0, S.stream>>>(sv, gran, ng);
  launch_check("k_granules");
  unsigned *bits = (unsigned *)(base + segdes_bits_words(n, m));
  GCVL_CK(cudaMemsetAsync(bits, 0, (size_t)segdes_nbits_words(n) * 4, S.stream));
  if (m > 0) {
    k_headbits<<<ceil_div(m, 256), 256, 0, S.stream>>>(sv, bits);
    launch_check("k_headbits");
  }
}

}  // namespace gcvl

using namespace gcvl;

// ============================================================ C ABI exports
#define SCAN_EXPORTS(NAME, L, OP, T)                                                        \
  GCVL_EXPORT void NAME##_su##L(vec_p d, vec_p s, int len, vec_p scratch) {                 \
    run_scan<OP, M_SCAN, false>((T *)d, (const T *)s, nullptr, nullptr, len, 1, scratch,     \
                                false, #NAME "_su" #L);                                      \
  }                                                                                          \
  GCVL_EXPORT int NAME##_su##L##_scratch(int len) { return scan_units<T>(len); }             \
  GCVL_EXPORT unsigned NAME##_su##L##_inplace(void) { return INPLACE_1; }                    \
  GCVL_EXPORT void NAME##_se##L(vec_p d, vec_p s, vec_p sd, int n, int m, vec_p scratch) {   \
    seg_scan<OP>(d, s, sd, n, m, scratch, #NAME "_se" #L);                                   \
  }                                                                                          \
  GCVL_EXPORT int NAME##_se##L##_scratch(int n, int m) { (void)m; return scan_units<T>(n); } \
  GCVL_EXPORT unsigned NAME##_se##L##_inplace(void) { return INPLACE_1; }                    \
  GCVL_EXPORT T NAME##_ru##L(vec_p s, int len, vec_p scratch) {                              \
    return reduce_to_host<OP>(s, len, scratch);                                              \
  }                                                                                          \
  GCVL_EXPORT int NAME##_ru##L##_scratch(int len) { return reduce_units<T>(len); }           \
  GCVL_EXPORT unsigned NAME##_ru##L##_inplace(void) { return INPLACE_NONE; }                 \
  GCVL_EXPORT void NAME##_re##L(vec_p d, vec_p s, vec_p sd, int n, int m, vec_p scratch) {   \
    seg_reduce<OP>(d, s, sd, n, m, scratch, false, #NAME "_re" #L);                          \
  }                                                                                          \
  GCVL_EXPORT int NAME##_re##L##_scratch(int n, int m) {                                     \
    (void)m; int a = seg_reduce_units<T>(n), b = reduce_units<T>(n); return a > b ? a : b;    \
  }                                                                                          \
  GCVL_EXPORT unsigned NAME##_re##L##_inplace(void) { return INPLACE_NONE; }

SCAN_EXPORTS(add, z, AddZ, int)
SCAN_EXPORTS(add, d, AddD, double)
SCAN_EXPORTS(mul, z, MulZ, int)
SCAN_EXPORTS(mul, d, MulD, double)
SCAN_EXPORTS(min, z, MinZ, int)
SCAN_EXPORTS(min, d, MinD, double)
SCAN_EXPORTS(max, z, MaxZ, int)
SCAN_EXPORTS(max, d, MaxD, double)
SCAN_EXPORTS(and, b, AndB, cvl_bool)
SCAN_EXPORTS(and, z, AndZ, int)
SCAN_EXPORTS(ior, b, IorB, cvl_bool)
SCAN_EXPORTS(ior, z, IorZ, int)
SCAN_EXPORTS(xor, b, XorB, cvl_bool)
SCAN_EXPORTS(xor, z, XorZ, int)

// Segment descriptors (facilt.c:112-144).
GCVL_EXPORT void mke_fov(vec_p sd, vec_p l, int n, int m, vec_p scratch) {
  make_segdes(sd, l, n, m, scratch);
}
GCVL_EXPORT unsigned mke_fov_inplace(void) { return INPLACE_NONE; }
GCVL_EXPORT int mke_fov_scratch(int n, int m) { (void)n; return scan_units<int>(m); }
GCVL_EXPORT void len_fos(vec_p l, vec_p sd, int n, int m, vec_p scratch) {
  (void)n; (void)scratch;
  ensure_init();
  if (m <= 0 || l == sd) return;
  GCVL_CK(cudaMemcpyAsync(l, sd, (size_t)m * 4, cudaMemcpyDeviceToDevice, stream()));
}
GCVL_EXPORT int len_fos_scratch(int n, int m) { (void)n; (void)m; return 0; }
GCVL_EXPORT unsigned len_fos_inplace(void) { return INPLACE_NONE; }

// Pack, phase 1 (library.c:55-133): count true flags.
GCVL_EXPORT int pk1_luv(vec_p f, int len, vec_p scratch) {
  return reduce_to_host<CountB>(f, len, scratch, true);
}
GCVL_EXPORT int pk1_luv_scratch(int len) { return reduce_units<int>(len); }
GCVL_EXPORT unsigned pk1_luv_inplace(void) { return INPLACE_NONE; }
GCVL_EXPORT void pk1_lev(vec_p ds, vec_p f, vec_p sd, int n, int m, vec_p scratch) {
  seg_reduce<CountB>(ds, f, sd, n, m, scratch, true, "pk1_lev");
}
GCVL_EXPORT int pk1_lev_scratch(int n, int m) {
  (void)m; int a = seg_reduce_units<int>(n), b = reduce_units<int>(n); return a > b ? a : b;
}
GCVL_EXPORT unsigned pk1_lev_inplace(void) { return INPLACE_NONE; }

// ============================================================================
// add_sed for callers that cannot allocate device memory.
//
// Some callers of this library may not call cudaMalloc: embedders whose
// device memory is all handed out by their own pool or arena (a cudaMalloc
// would fail, or take memory the pool already counts as its own), and
// runtimes that forbid allocation after start-up because an allocation can
// synchronise the device or fail at a time the caller cannot handle.  For
// them gcvl_add_sed_noalloc runs the same segmented +-scan as add_sed but
// keeps its look-back scratch in the fixed array below instead of a caller
// scratch vector or the library workspace, and it allocates nothing: no
// cudaMalloc, cudaFree or other allocating call, and it does not run the
// library's own first-use set-up (which allocates).
//
// The array holds the scratch of at most 2^28 elements: 2,097,664 bytes
// (2.0 MiB), allocated on every GPU that loads the library until the process
// exits.  All calls share it and it keeps the last call's contents; each call
// clears the part that must start at zero.  Calls that overlap on the GPU
// race on it: issue them on one stream, or order them.
//
// A bounded wait that gives up in these kernels sets a bit in a status word
// of the same kind (g_noalloc_status); gcvl_sync reads and clears it like the
// library's own status word and returns the timeout (error 3).
// ============================================================================
constexpr long kNoallocMaxN = 1L << 28;
constexpr size_t kNoallocTiles = (size_t)(kNoallocMaxN / tile_elems<double>());  // smallest tiling
constexpr size_t kNoallocBytes = 512 + ((kNoallocTiles * 16 + 255) / 256) * 256;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocBytes];
static __device__ unsigned g_noalloc_status;

static_assert(kNoallocBytes == 2097664, "the documented size of the fixed scratch array");

// Device addresses of the array and of its status word, looked up once per
// device (with that device current) on the first call made on it.  They are
// kept until exit: a cudaDeviceReset on that device invalidates them, and no
// call may follow one.
static void *g_noalloc_ptr[128];
static unsigned *g_noalloc_status_ptr[128];

namespace gcvl {
// Folds the no-allocation entry point's status word of the current device
// into the library's error state and clears it.  Does nothing on a device
// where that entry point has not run.  The caller has waited for the work.
bool noalloc_used() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 128) return false;
  return g_noalloc_status_ptr[dev] != nullptr;
}
void noalloc_fold_status() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 128 || !g_noalloc_status_ptr[dev]) return;
  unsigned word = 0;
  if (!GCVL_CK(cudaMemcpy(&word, g_noalloc_status_ptr[dev], 4, cudaMemcpyDeviceToHost))) return;
  if (word & DEV_TIMEOUT)
    set_error(GCVL_ERR_TIMEOUT, "a bounded device wait gave up in gcvl_add_sed_noalloc (status 0x%x)", word);
  if (word) {
    unsigned zero = 0;
    GCVL_CK(cudaMemcpy(g_noalloc_status_ptr[dev], &zero, 4, cudaMemcpyHostToDevice));
  }
}
}  // namespace gcvl

GCVL_EXPORT int gcvl_add_sed_noalloc(vec_p d, vec_p s, vec_p sd, int n, int m) {
  using namespace gcvl;
  if (n < 0 || m < 0 || (long)n > kNoallocMaxN) {
    set_error(GCVL_ERR_RANGE, "gcvl_add_sed_noalloc: n = %d outside [0, %ld]", n, kNoallocMaxN);
    return GCVL_ERR_RANGE;
  }
  if (n == 0) return GCVL_OK;
  int dev = 0;
  if (!GCVL_CK(cudaGetDevice(&dev))) return GCVL_ERR_CUDA;
  if (dev < 0 || dev >= 128) { set_error(GCVL_ERR_RANGE, "gcvl_add_sed_noalloc: device %d", dev); return GCVL_ERR_RANGE; }
  if (!g_noalloc_ptr[dev]) {
    void *p = nullptr, *q = nullptr;
    cudaError_t e1 = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    cudaError_t e2 = cudaGetSymbolAddress(&q, g_noalloc_status);
    if (e1 != cudaSuccess || e2 != cudaSuccess) {
      set_error(GCVL_ERR_CUDA, "gcvl_add_sed_noalloc: cudaGetSymbolAddress: %s",
                cudaGetErrorString(e1 != cudaSuccess ? e1 : e2));
      return GCVL_ERR_CUDA;
    }
    g_noalloc_ptr[dev] = p;
    g_noalloc_status_ptr[dev] = (unsigned *)q;
  }
  State &S = st();
  cudaStream_t strm = S.ready ? S.stream : (cudaStream_t)0;
  void *mem = g_noalloc_ptr[dev];
  const bool seg = (m != 1) && sd != nullptr;
  const double *in = (const double *)s;
  double *out = (double *)d;
  const long rows = (long)n / row_items<double>();
  CUtensorMap tin, tout;
  const bool tma = !getenv("GCVL_NO_TMA") && rows >= 1 && !((size_t)in & 15) && !((size_t)out & 15) &&
                   tma_map<double>(&tin, in, rows) && tma_map<double>(&tout, out, rows);
  const int tiles = tma ? ceil_div(n, (long)TT * row_items<double>()) : ceil_div(n, tile_elems<double>());
  if (lookback_bytes(tiles) > kNoallocBytes) {
    set_error(GCVL_ERR_RANGE, "gcvl_add_sed_noalloc: %d tiles exceed the fixed scratch", tiles);
    return GCVL_ERR_RANGE;
  }
  if (!GCVL_CK(cudaMemsetAsync(mem, 0, lookback_clear_bytes(tiles), strm))) return GCVL_ERR_CUDA;
  if (tma) {
    TArgs<double> a;
    a.out = out; a.in = in; a.n = n; a.rows = rows;
    a.sv = seg ? seg_view(sd, n, m) : SegView{nullptr, nullptr, nullptr, nullptr, n, 1};
    a.lb = lookback_carve(mem, tiles);
    a.status = g_noalloc_status_ptr[dev];
    a.spin_limit = S.spin_limit;
    if (seg) k_scan_tma<AddD, M_SCAN, true><<<tiles, TB_LB, tma_smem<double>(0), strm>>>(tin, tout, a);
    else k_scan_tma<AddD, M_SCAN, false><<<tiles, TB_LB, tma_smem<double>(0), strm>>>(tin, tout, a);
  } else {
    ScanArgs<double> a;
    a.out = out; a.in = in; a.out2 = nullptr; a.n = n;
    a.sv = seg ? seg_view(sd, n, m) : SegView{nullptr, nullptr, nullptr, nullptr, n, 1};
    a.lb = lookback_carve(mem, tiles);
    a.status = g_noalloc_status_ptr[dev];
    a.spin_limit = S.spin_limit;
    a.count_flags = 0;
    if (seg) k_scan<AddD, M_SCAN, true><<<tiles, Tiling<double>::BLOCK, 0, strm>>>(a);
    else k_scan<AddD, M_SCAN, false><<<tiles, Tiling<double>::BLOCK, 0, strm>>>(a);
  }
  // launch_check clears the launch error it records, so read it first
  const cudaError_t launched = cudaPeekAtLastError();
  launch_check("gcvl_add_sed_noalloc");
  return launched == cudaSuccess ? GCVL_OK : GCVL_ERR_CUDA;
}

GCVL_EXPORT long gcvl_add_sed_noalloc_max_n(void) { return kNoallocMaxN; }

// add_ruz with the result left in device memory (d[0]), so that a sequence
// needing a length (PACK, MAKE_SEGDES) can be captured in a CUDA graph: the
// host reads the value once, after the graph, instead of synchronising inside.
GCVL_EXPORT void gcvl_add_ruz_dev(vec_p d, vec_p s, int len, vec_p scratch) {
  run_reduce<AddZ>((const int *)s, len, (int *)d, scratch, false);
}
GCVL_EXPORT int gcvl_add_ruz_dev_scratch(int len) { return reduce_units<int>(len); }

// y = A x for A in CSR form as CVL vectors: row descriptor sd (rows segments
// over nnz), column indices cols and values vals (nnz each), x (ncols).
GCVL_EXPORT void gcvl_spmv_csr(vec_p y, vec_p vals, vec_p cols, vec_p x, vec_p sd, int nnz, int rows,
                               vec_p scratch) {
  run_gather_mul_reduce((double *)y, (const double *)vals, (const int *)cols, (const double *)x, sd, nnz, rows,
                        scratch);
}
GCVL_EXPORT int gcvl_spmv_csr_scratch(int nnz, int rows) {
  (void)rows;
  const int k = nnz > 0 ? nnz : 1;  // either form's tiles
  const int a = ceil_div(k, tile_elems<double>()), b = ceil_div(k, (long)TT * row_items<double>());
  return (int)((reduce_pass_bytes(a > b ? a : b) + 7) / 8);
}
