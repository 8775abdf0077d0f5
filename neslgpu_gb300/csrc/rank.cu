// rank.cu -- stable radix rank, up and down, int and double, segmented and
// unsegmented (nesl/cvl/serial/rank.c:49-362), and the partitioned scatter
// that large permutes share with it.
//
// d[j] is the position of element j in the stable sorted order of its
// segment.  Keys are made order-preserving unsigned integers exactly as the
// serial CVL does: int keys flip the sign bit (up) or every other bit
// (down), rank.c:94-99; double keys flip all bits of negatives and the sign
// bit of the rest, and down ranks complement that, rank.c:258-280.  A
// segmented rank is a stable sort by (segment, key): the key passes carry
// each element's segment number, then further passes sort by it.
//
// GPU design (onesweep style).  One prepare pass builds every pass's 256-bin
// digit histogram at once with shared-memory atomics (and, for segmented
// ranks, writes transformed keys, indices and segment numbers).  Then one
// pass per 8-bit digit: each warp of a CTA loads its 32 x RK_ITEMS
// consecutive keys and values into registers, ranks them stably with
// ballots, the CTA learns how many earlier tiles' elements fall in each
// digit by a per-digit decoupled look-back, reorders the tile in shared
// memory and writes coalesced runs.  The first pass of an unsegmented rank
// reads the caller's keys and transforms them itself.
//
// The result is the inverse of the sort permutation: rank[index] = position,
// a scatter to random places.  Below RK_DIRECT_MAX elements the last pass
// writes it directly (the rank vector fits in L2, which absorbs the random
// writes).  Above it the last pass writes each (index, position) pair
// grouped by the top 8 bits of the index -- 256 windows of the output, each
// element's slot from a second per-window look-back in the same pass -- and
// a streaming kernel writes each window's ranks while the window sits in
// L2, so DRAM sees whole sectors instead of a read-modify-write per 4-byte
// element.  Large permutes and gathers (smp_pu*, bck_pu*, the default and
// flag permutes) split their pairs by window with passes of their own (the
// window split below) and share the window scatter.
#include "gcvl.cuh"

#include <type_traits>
#include <utility>

namespace gcvl {

// Keys per thread of a digit pass (tile = 256 x RK_ITEMS), and the CTAs per
// SM of the 32-bit unsegmented passes, measured at 2^28 (int / double /
// segmented int rank): 16 items at 4 CTAs 9.09 / 21.4 / 18.0 ms; 20 at 3
// 9.06 / 19.8 / 17.2; 24 at 3 9.43 / 18.7 / 17.0; 32 at 2 10.1 / 25.9 / 21.9.
#ifndef GCVL_RK_ITEMS
#define GCVL_RK_ITEMS 20
#endif
constexpr int RK_BLOCK = 256, RK_ITEMS = GCVL_RK_ITEMS, RK_TILE = RK_BLOCK * RK_ITEMS;
constexpr int RK_WARPS = RK_BLOCK / 32;
constexpr int RK_MAXPASS = 12;
#ifndef GCVL_RK_LB
#define GCVL_RK_LB 4
#endif
// Resident CTAs per SM the register allocation must allow: 32-bit keys
// without segment numbers fit 64 registers (the pass holds its keys and
// values in registers); 64-bit keys and segmented passes would spill there.
#ifndef GCVL_RK_MINB
#define GCVL_RK_MINB 2
#endif
#ifndef GCVL_RK_MINB_NARROW
#define GCVL_RK_MINB_NARROW 3
#endif
constexpr int RK_LB = GCVL_RK_LB;  // predecessors read per look-back round trip
constexpr int RK_DIRECT_MAX = 1 << 23;
// 8 measured best at 2^28 (bck_puz / smp_puz): 4 items 2.87 / 2.94 ms,
// 8 items 2.63 / 2.78, 16 items 3.01 / 2.78
#ifndef GCVL_SC_ITEMS
#define GCVL_SC_ITEMS 8
#endif
constexpr int SC_ITEMS = GCVL_SC_ITEMS;  // elements per thread in the window and streaming passes
constexpr unsigned RK_INC = 0x80000000u;

// where a pass gets its tile from, and where it puts it
enum { IN_ARRAYS = 0, IN_SRC = 1 };                    // IN_SRC: caller's keys, value = position
// OUT_RANK: rank[v] = pos; OUT_WIN: (v, pos) grouped by the output window of
// v (the partition of the inverse scatter)
enum { OUT_ARRAYS = 0, OUT_RANK = 1, OUT_WIN = 3 };

__host__ __device__ inline int bit_length(unsigned x) {
  int b = 0;
  while (x) { b++; x >>= 1; }
  return b;
}

struct RankPrep {
  const void *src;
  int n, is_double, up, seg, write_arrays;
  SegView sv;
  void *key;           // uint32 or uint64 transformed keys
  unsigned *idx;
  unsigned *aux;       // segment numbers (segmented ranks)
  unsigned *hist;      // [RK_MAXPASS][256]
  int key_passes, seg_passes;
};

__device__ __forceinline__ unsigned long long rk_key64(unsigned long long b, int up) {
  unsigned long long k = (b >> 63) ? ~b : (b ^ (1ULL << 63));
  return up ? k : ~k;
}
__device__ __forceinline__ unsigned rk_key32(unsigned x, int up) { return x ^ (up ? 0x80000000u : 0x7FFFFFFFu); }

__device__ __forceinline__ void rank_prep_one(const RankPrep &p, unsigned *s_hist, long i, unsigned long long raw) {
  unsigned long long k;
  if (p.is_double) {
    k = rk_key64(raw, p.up);
    if (p.write_arrays) ((unsigned long long *)p.key)[i] = k;
  } else {
    const unsigned kk = rk_key32((unsigned)raw, p.up);
    if (p.write_arrays) ((unsigned *)p.key)[i] = kk;
    k = kk;
  }
  if (p.write_arrays) p.idx[i] = (unsigned)i;
  for (int q = 0; q < p.key_passes; q++) atomicAdd(&s_hist[q * 256 + (int)((k >> (8 * q)) & 255)], 1u);
  if (p.seg) {
    const unsigned sg = (unsigned)seg_of(p.sv, (int)i);
    p.aux[i] = sg;
    for (int q = 0; q < p.seg_passes; q++)
      atomicAdd(&s_hist[(p.key_passes + q) * 256 + ((sg >> (8 * q)) & 255)], 1u);
  }
}
__device__ __forceinline__ unsigned long long rank_prep_load(const RankPrep &p, long i) {
  return p.is_double ? __ldcs((const unsigned long long *)p.src + i) : (unsigned long long)__ldcs((const unsigned *)p.src + i);
}

__global__ void __launch_bounds__(RK_BLOCK) k_rank_prep(RankPrep p) {
  __shared__ unsigned s_hist[RK_MAXPASS * 256];
  const int passes = p.key_passes + p.seg_passes;
  for (int i = threadIdx.x; i < passes * 256; i += RK_BLOCK) s_hist[i] = 0;
  __syncthreads();
  const long stride = (long)gridDim.x * RK_BLOCK;
  long i = (long)blockIdx.x * RK_BLOCK + threadIdx.x;
  // four independent loads in flight per thread
  for (; i + 3 * stride < p.n; i += 4 * stride) {
    unsigned long long r[4];
#pragma unroll
    for (int u = 0; u < 4; u++) r[u] = rank_prep_load(p, i + u * stride);
#pragma unroll
    for (int u = 0; u < 4; u++) rank_prep_one(p, s_hist, i + u * stride, r[u]);
  }
  for (; i < p.n; i += stride) rank_prep_one(p, s_hist, i, rank_prep_load(p, i));
  __syncthreads();
  for (int i = threadIdx.x; i < passes * 256; i += RK_BLOCK)
    if (s_hist[i]) atomicAdd(&p.hist[i], s_hist[i]);
}

// d[idx[i]] = s[i] when the indices ascend (gate word zero): the stores of a
// warp then fall on few lines, and no partition is needed
template <class V>
__global__ void __launch_bounds__(RK_BLOCK) k_sorted_scatter(V *__restrict__ d, const V *__restrict__ s,
                                                             const int *__restrict__ idx, long n,
                                                             const unsigned *__restrict__ gate) {
  if (*(const volatile unsigned *)gate) return;
  for (long i0 = (long)blockIdx.x * (RK_BLOCK * SC_ITEMS) + threadIdx.x; i0 < n;
       i0 += (long)gridDim.x * (RK_BLOCK * SC_ITEMS)) {
    int k[SC_ITEMS];
    V v[SC_ITEMS];
#pragma unroll
    for (int u = 0; u < SC_ITEMS; u++) {
      const long i = i0 + (long)u * RK_BLOCK;
      if (i < n) { k[u] = __ldcs(idx + i); v[u] = __ldcs(s + i); }
    }
#pragma unroll
    for (int u = 0; u < SC_ITEMS; u++) {
      const long i = i0 + (long)u * RK_BLOCK;
      if (i < n) d[k[u]] = v[u];
    }
  }
}

// hist[q][d] -> exclusive scan over d, in place (one CTA, 256 threads)
__global__ void k_rank_digit_starts(unsigned *hist, int passes) {
  __shared__ unsigned s[256];
  for (int q = 0; q < passes; q++) {
    unsigned v = hist[q * 256 + threadIdx.x];
    s[threadIdx.x] = v;
    __syncthreads();
    for (int d = 1; d < 256; d <<= 1) {
      unsigned o = threadIdx.x >= d ? s[threadIdx.x - d] : 0u;
      __syncthreads();
      s[threadIdx.x] += o;
      __syncthreads();
    }
    hist[q * 256 + threadIdx.x] = s[threadIdx.x] - v;
    __syncthreads();
  }
}

// digit starts of a permutation of [0, n) split by index >> shift: every
// window but the last is full
__global__ void k_window_starts(unsigned *starts, int n, int shift) {
  const long s = (long)threadIdx.x << shift;
  starts[threadIdx.x] = (unsigned)(s < n ? s : n);
}

template <class K, class V> struct PassArgs {
  const K *kin; const V *vin; const unsigned *ain;
  K *kout; V *vout; unsigned *aout;
  const void *src; int up;            // IN_SRC: the caller's keys
  int *rank; const int *segoff;       // OUT_RANK / OUT_WIN (segmented: rebase by the key)
  unsigned *pidx, *ppos;              // OUT_WIN
  const unsigned *starts;             // this pass's digit starts
  unsigned *state;                    // [tiles][256] look-back words
  const unsigned *wstarts;            // OUT_WIN: first slot of every output window
  unsigned *wstate;                   // OUT_WIN: [tiles][256] look-back words of the window counts
  int wshift;                         // OUT_WIN: window of v = v >> wshift
  unsigned *counter;
  const unsigned *gate;               // non-null: the pass runs only if *gate is non-zero
  int n, shift;
  unsigned *status;
  int spin_limit;
};

template <class K, class V, bool AUX> constexpr size_t pass_smem() {
  return (size_t)RK_TILE * (sizeof(K) + sizeof(V) + (AUX ? 4 : 0)) + RK_WARPS * 256 * 2 + 256 * 4 + 256 * 8;
}

// Publish this tile's count of one bin (digit or window), then look back for
// the earlier tiles' total.  One 32-bit word per (tile, bin): 0 = not yet,
// 1 + count = this tile's count (aggregate), RK_INC | prefix = the bin's
// count in this and all earlier tiles (inclusive; < 2^31 because n is an
// int).  RK_LB predecessors per round trip, nearest first, until an
// inclusive count is found (bounded waits).  Each word is self-contained, so
// relaxed loads suffice and all RK_LB are in flight together; a warp's loads
// of one predecessor are one 128-byte line.
__device__ __forceinline__ unsigned bin_lookback(unsigned *state, int tile, int bin, unsigned tot,
                                                 unsigned *status, int spin_limit) {
  unsigned *stw = state + (long)tile * 256 + bin;
  if (tile == 0) {
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(stw), "r"(RK_INC | tot) : "memory");
    return 0;
  }
  asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(stw), "r"(1u + tot) : "memory");
  unsigned prefix = 0;
  long t0 = tile - 1;
  bool done = false;
  while (!done && t0 >= 0) {
    unsigned w[RK_LB];
#pragma unroll
    for (int j = 0; j < RK_LB; j++) {
      w[j] = RK_INC;  // beyond tile 0: an inclusive zero
      if (t0 - j >= 0)
        asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(w[j]) : "l"(state + (t0 - j) * 256 + bin) : "memory");
    }
#pragma unroll
    for (int j = 0; j < RK_LB; j++) {
      if (done) break;
      int it = 0;
      while (w[j] == 0) {
        if (++it >= spin_limit) { atomicOr(status, DEV_TIMEOUT); w[j] = RK_INC; break; }
        __nanosleep(32);
        asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(w[j]) : "l"(state + (t0 - j) * 256 + bin) : "memory");
      }
      if (w[j] & RK_INC) { prefix += w[j] & ~RK_INC; done = true; }
      else prefix += w[j] - 1u;
    }
    t0 -= RK_LB;
  }
  asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(stw), "r"(RK_INC | (prefix + tot)) : "memory");
  return prefix;
}

// Equal digits keep their order (the ballots below rank each warp's
// elements in element order).
template <class K, bool AUX> constexpr int rk_minb() { return sizeof(K) == 4 && !AUX ? GCVL_RK_MINB_NARROW : GCVL_RK_MINB; }
template <class K, class V, bool AUX, int IN, int OUT>
__global__ void __launch_bounds__(RK_BLOCK, rk_minb<K, AUX>()) k_radix_pass(PassArgs<K, V> a) {
  typedef unsigned short CntT;  // per-warp digit counts (at most 32 * RK_ITEMS)
  // 32-bit keys and values leave the reorder as one 8-byte pair
  constexpr bool PAIR = sizeof(K) == 4 && sizeof(V) == 4 && OUT == OUT_ARRAYS;
  extern __shared__ __align__(16) unsigned char rk_smem[];
  // the reordered tile (the input stays in registers)
  long long *s_gb = (long long *)rk_smem;                  // [256] global base per digit
  K *s_kout = (K *)(s_gb + 256);
  V *s_vout = (V *)(s_kout + RK_TILE);
  uint2 *s_pair = (uint2 *)s_kout;                         // PAIR: [RK_TILE] (key, value)
  unsigned *s_aout = (unsigned *)(s_vout + RK_TILE);
  unsigned *s_loc = s_aout + (AUX ? RK_TILE : 0);          // [256] tile offset per digit
  CntT *s_cnt = (CntT *)(s_loc + 256);                      // [RK_WARPS][256]
  __shared__ unsigned s_tile;
  __shared__ unsigned s_ws[RK_WARPS];

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (a.gate && *(const volatile unsigned *)a.gate == 0) return;  // the same answer for every CTA
  if (tid == 0) s_tile = atomicAdd(a.counter, 1u);
  for (int i = tid; i < RK_WARPS * 256; i += RK_BLOCK) s_cnt[i] = 0;
  __syncthreads();
  const int tile = (int)s_tile;
  const long base = (long)tile * RK_TILE;
  const int valid = (int)min((long)RK_TILE, (long)a.n - base);

  // each warp's 32 * RK_ITEMS consecutive elements straight into registers
  // (element wbase + 32c + lane in item c: coalesced, every load in flight)
  const int wbase = warp * 32 * RK_ITEMS;
  K kr[RK_ITEMS];
  V vr[RK_ITEMS];
  unsigned ar[AUX ? RK_ITEMS : 1];
#pragma unroll
  for (int c = 0; c < RK_ITEMS; c++) {
    const int e = wbase + c * 32 + lane;
    kr[c] = 0;
    vr[c] = 0;
    if (AUX) ar[c] = 0;
    if (e < valid) {
      if constexpr (IN == IN_SRC) {
        if constexpr (sizeof(K) == 8)
          kr[c] = (K)rk_key64(__ldcs((const unsigned long long *)a.src + base + e), a.up);
        else
          kr[c] = (K)rk_key32(__ldcs((const unsigned *)a.src + base + e), a.up);
        vr[c] = (V)(base + e);
      } else {
        kr[c] = __ldcs(a.kin + base + e);
        vr[c] = __ldcs(a.vin + base + e);
        if (AUX) ar[c] = __ldcs(a.ain + base + e);
      }
    }
  }

  // rank within each warp's 512 elements: (rank << 8) | digit
  CntT *cnt = s_cnt + warp * 256;
  const unsigned lt = (1u << lane) - 1u;
  unsigned wr[RK_ITEMS];
#pragma unroll
  for (int c = 0; c < RK_ITEMS; c++) {
    const int e = wbase + c * 32 + lane;
    const int d = e < valid ? (int)((kr[c] >> a.shift) & 255) : -1;
    unsigned r = 0;
    const unsigned peers = warp_match8(d);
    if (d >= 0) r = cnt[d] + __popc(peers & lt);
    __syncwarp();
    if (d >= 0 && (peers & lt) == 0) cnt[d] = (CntT)(cnt[d] + __popc(peers));
    __syncwarp();
    wr[c] = d >= 0 ? (r << 8) | (unsigned)d : 0xFFFFFFFFu;
  }
  __syncthreads();

  // per digit: tile count, per-warp exclusive offsets
  const int dd = tid;  // RK_BLOCK == 256 digits
  unsigned tot = 0;
#pragma unroll
  for (int w = 0; w < RK_WARPS; w++) {
    unsigned c = s_cnt[w * 256 + dd];
    s_cnt[w * 256 + dd] = (CntT)tot;
    tot += c;
  }
  const unsigned prefix = bin_lookback(a.state, tile, dd, tot, a.status, a.spin_limit);
  // exclusive scan of tile counts over the digits -> tile offsets
  {
    unsigned incl = tot;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      unsigned x = shfl_up(incl, o);
      if (lane >= o) incl += x;
    }
    if (lane == 31) s_ws[warp] = incl;
    __syncthreads();
    unsigned wp = 0;
#pragma unroll
    for (int w = 0; w < RK_WARPS; w++) if (w < warp) wp += s_ws[w];
    const unsigned loc = wp + incl - tot;
    s_loc[dd] = loc;
    s_gb[dd] = (long long)__ldg(a.starts + dd) + (long long)prefix - (long long)loc;
    // each warp's counter of this digit becomes the digit's slot in the
    // reordered tile for that warp (one shared-memory lookup per element
    // below instead of two; below 4096, so it fits the 16-bit counter)
#pragma unroll
    for (int w = 0; w < RK_WARPS; w++) s_cnt[w * 256 + dd] = (CntT)(s_cnt[w * 256 + dd] + loc);
  }
  __syncthreads();
  if constexpr (OUT == OUT_WIN) {
    // (v, pos) straight into the output windows of v: each element's sorted
    // position from the digit offsets (no reorder by digit), then an
    // unstable slot in its window, the windows' counts looked back over the
    // earlier tiles like the digits', and a reorder by window so that each
    // window's run leaves as one coalesced run
    unsigned pos[RK_ITEMS];
#pragma unroll
    for (int c = 0; c < RK_ITEMS; c++) {
      const unsigned x = wr[c];
      pos[c] = 0;
      if (x != 0xFFFFFFFFu) {
        const int d = (int)(x & 255u);
        long long g = s_gb[d] + s_cnt[warp * 256 + d] + (x >> 8);
        if (a.segoff) g -= __ldg(a.segoff + (int)kr[c]);
        pos[c] = (unsigned)g;
      }
    }
    __syncthreads();  // s_cnt, s_loc and s_gb are free
    unsigned *s_wc = (unsigned *)s_cnt;  // [256] window counts
    s_wc[tid] = 0;
    __syncthreads();
#pragma unroll
    for (int c = 0; c < RK_ITEMS; c++) {
      if (wr[c] != 0xFFFFFFFFu) {
        const unsigned w = (unsigned)vr[c] >> a.wshift;
        wr[c] = (atomicAdd(s_wc + w, 1u) << 8) | w;
      }
    }
    __syncthreads();
    const unsigned wtot = s_wc[tid];
    const unsigned wprefix = bin_lookback(a.wstate, tile, tid, wtot, a.status, a.spin_limit);
    {
      unsigned incl = wtot;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        unsigned xx = shfl_up(incl, o);
        if (lane >= o) incl += xx;
      }
      if (lane == 31) s_ws[warp] = incl;
      __syncthreads();
      unsigned wp = 0;
#pragma unroll
      for (int w = 0; w < RK_WARPS; w++) if (w < warp) wp += s_ws[w];
      const unsigned wloc = wp + incl - wtot;
      s_loc[tid] = wloc;
      s_gb[tid] = (long long)__ldg(a.wstarts + tid) + (long long)wprefix - (long long)wloc;
    }
    __syncthreads();
    uint2 *s_vp = (uint2 *)s_kout;  // (v, position) by window slot: one 8-byte store
#pragma unroll
    for (int c = 0; c < RK_ITEMS; c++) {
      const unsigned x = wr[c];
      if (x != 0xFFFFFFFFu) s_vp[s_loc[x & 255u] + (x >> 8)] = make_uint2((unsigned)vr[c], pos[c]);
    }
    __syncthreads();
#pragma unroll 4
    for (int e = tid; e < valid; e += RK_BLOCK) {
      const uint2 vp = s_vp[e];
      const long g = s_gb[vp.x >> a.wshift] + e;
      a.pidx[g] = vp.x;
      a.ppos[g] = vp.y;
    }
    return;
  }
  // reorder the tile in shared memory
#pragma unroll
  for (int c = 0; c < RK_ITEMS; c++) {
    const unsigned x = wr[c];
    if (x != 0xFFFFFFFFu) {
      const int d = (int)(x & 255u);
      const unsigned lp = s_cnt[warp * 256 + d] + (x >> 8);
      if constexpr (PAIR) {
        s_pair[lp] = make_uint2((unsigned)kr[c], (unsigned)vr[c]);
      } else {
        s_kout[lp] = kr[c];
        s_vout[lp] = vr[c];
      }
      if (AUX) s_aout[lp] = ar[c];
    }
  }
  __syncthreads();
  // coalesced runs out
#pragma unroll 4
  for (int e = tid; e < valid; e += RK_BLOCK) {
    K k;
    V vv;
    if constexpr (PAIR) {
      const uint2 kv = s_pair[e];
      k = (K)kv.x;
      vv = (V)kv.y;
    } else {
      k = s_kout[e];
      vv = s_vout[e];
    }
    const int d = (int)((k >> a.shift) & 255);
    const long g = s_gb[d] + e;
    if (OUT == OUT_ARRAYS) {
      a.kout[g] = k;
      a.vout[g] = vv;
      if (AUX) a.aout[g] = s_aout[e];
    } else {  // OUT_RANK
      int r = (int)g;
      if (a.segoff) r -= __ldg(a.segoff + (int)k);
      a.rank[(unsigned)vv] = r;
    }
  }
}

// d[key[i]] = val[i], streaming over pairs that a partition pass grouped by
// output window
template <class V>
__global__ void __launch_bounds__(RK_BLOCK) k_window_scatter(V *__restrict__ d, const unsigned *__restrict__ key,
                                                             const V *__restrict__ val, long n,
                                                             const unsigned *__restrict__ gate) {
  // one CTA per 2048 pairs, not a grid-stride loop: CTAs dispatched in
  // order keep the writes within a few windows of the output at a time
  // (a grid-stride form let the CTAs drift apart: rank 11.6 -> 17.1 ms)
  if (gate && *(const volatile unsigned *)gate == 0) return;
  const long i0 = (long)blockIdx.x * (RK_BLOCK * SC_ITEMS) + threadIdx.x;
  unsigned k[SC_ITEMS];
  V v[SC_ITEMS];
#pragma unroll
  for (int u = 0; u < SC_ITEMS; u++) {
    const long i = i0 + (long)u * RK_BLOCK;
    if (i < n) { k[u] = __ldcs(key + i); v[u] = __ldcs(val + i); }
  }
#pragma unroll
  for (int u = 0; u < SC_ITEMS; u++) {
    const long i = i0 + (long)u * RK_BLOCK;
    if (i < n) d[k[u]] = v[u];
  }
}

// ------------------------------------------------------ window split ---
// Groups keys by window (key >> shift, clamped below nw: the same function in
// every pass) without any tile waiting on another: a histogram pass writes
// each tile's per-window counts (window-major), their exclusive scan (the
// library's int +-scan, in place) is every (window, tile)'s first slot --
// the windows before w, then the tiles before t -- and the split pass
// places each tile's keys there.  Slots within a window and tile come from shared-memory atomics (no
// particular order); the tile is staged in shared memory by window and each
// window's run leaves as one coalesced run; with POS, pos[k] = the slot key
// k went to, written in the input order.  The partitioned gather uses it.
constexpr int WS_ITEMS = 16, WS_TILE = RK_BLOCK * WS_ITEMS, WS_MAXW = 256;
__device__ __forceinline__ unsigned ws_window(unsigned k, int shift, int nw) { return min(k >> shift, (unsigned)(nw - 1)); }
// this key's slot among the keys of window w counted in cnt[w] so far (w <
// 0: none).  One shared-memory atomic per key: a per-warp form (lanes of
// one window found by a ballot per window bit, one atomic per window) made
// the partitioned gather and scatter 1.4-1.6x slower.
__device__ __forceinline__ unsigned ws_slot(unsigned *cnt, int w) { return w >= 0 ? atomicAdd(cnt + w, 1u) : 0u; }

// counts[w * tiles + t] = keys of tile t in window w; *unsorted != 0 when
// some key exceeds its successor.  VEC: key is 16-byte aligned, and each
// thread reads four keys at a time.
template <bool VEC>
__global__ void __launch_bounds__(RK_BLOCK) k_ws_hist(const unsigned *__restrict__ key, long n, int shift, int wbits,
                                                      unsigned *__restrict__ counts, unsigned *unsorted) {
  __shared__ unsigned s_cnt[WS_MAXW];
  __shared__ int s_uns;
  const int tid = threadIdx.x, nw = 1 << wbits;
  const int tiles = gridDim.x, t = blockIdx.x;
  s_cnt[tid] = 0;
  if (tid == 0) s_uns = 0;
  __syncthreads();
  const long base = (long)t * WS_TILE;
  int uns = 0;
  if constexpr (VEC) {
    uint4 q[WS_ITEMS / 4];
    unsigned nx[WS_ITEMS / 4];
#pragma unroll
    for (int c = 0; c < WS_ITEMS / 4; c++) {
      const long e = base + 4L * (c * RK_BLOCK + tid);
      q[c] = make_uint4(0, 0, 0, 0);
      nx[c] = 0xFFFFFFFFu;
      if (e + 3 < n) {
        q[c] = __ldcs(reinterpret_cast<const uint4 *>(key + e));
        // the successor of the fourth key: the next lane's line, just read
        if (e + 4 < n) nx[c] = __ldg(key + e + 4);
      }
    }
#pragma unroll
    for (int c = 0; c < WS_ITEMS / 4; c++) {
      const long e = base + 4L * (c * RK_BLOCK + tid);
      const unsigned k4[4] = {q[c].x, q[c].y, q[c].z, q[c].w};
      if (e + 3 < n) {
        if (k4[0] > k4[1] || k4[1] > k4[2] || k4[2] > k4[3] || k4[3] > nx[c]) uns = 1;
      } else {
        for (int u = 0; u < 4; u++)  // the vector's ragged end
          if (e + u + 1 < n && __ldg(key + e + u) > __ldg(key + e + u + 1)) uns = 1;
      }
#pragma unroll
      for (int u = 0; u < 4; u++) {
        int w = -1;
        if (e + u < n) w = (int)ws_window(e + 3 < n ? k4[u] : __ldg(key + e + u), shift, nw);
        ws_slot(s_cnt, w);
      }
    }
  } else {
    unsigned k[WS_ITEMS];
#pragma unroll
    for (int c = 0; c < WS_ITEMS; c++) {
      const long e = base + c * RK_BLOCK + tid;
      k[c] = e < n ? __ldcs(key + e) : 0u;
    }
#pragma unroll
    for (int c = 0; c < WS_ITEMS; c++) {
      const long e = base + c * RK_BLOCK + tid;
      // the successor's load usually hits the line just read by the next lane
      if (e + 1 < n && k[c] > __ldg(key + e + 1)) uns = 1;
      ws_slot(s_cnt, e < n ? (int)ws_window(k[c], shift, nw) : -1);
    }
  }
  if (__any_sync(0xffffffffu, uns) && (tid & 31) == 0) s_uns = 1;
  __syncthreads();
  if (tid < nw) counts[(long)tid * tiles + t] = s_cnt[tid];
  if (tid == 0 && s_uns) atomicOr(unsorted, 1u);
}

// VAL: each key's value (val[k]) moves with it to vout.  Dynamic shared
// memory: ws_split_smem<V, VAL>() bytes.
template <class V, bool VAL> constexpr size_t ws_split_smem() { return (size_t)WS_TILE * (4 + (VAL ? sizeof(V) : 0)); }
template <bool POS, class V = unsigned, bool VAL = false>
__global__ void __launch_bounds__(RK_BLOCK) k_window_split(const unsigned *__restrict__ key, long n, int shift,
                                                           int wbits, const unsigned *__restrict__ first,
                                                           const unsigned *gate, unsigned *__restrict__ kout,
                                                           unsigned *__restrict__ pos, const V *__restrict__ val = nullptr,
                                                           V *__restrict__ vout = nullptr) {
  __shared__ unsigned s_cnt[WS_MAXW];   // the tile's count per window, then its first slot there in the tile
  __shared__ unsigned s_base[WS_MAXW];  // global slot of the window's first key of this tile
  extern __shared__ __align__(16) unsigned char rk_smem[];
  unsigned *s_key = (unsigned *)rk_smem;                  // [WS_TILE] keys by window
  V *s_val = (V *)(rk_smem + (size_t)WS_TILE * 4);        // [WS_TILE] their values (VAL)
  __shared__ unsigned s_ws[RK_WARPS];
  if (!*(const volatile unsigned *)gate) return;  // the same answer for every CTA
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = 1 << wbits;
  const int tiles = gridDim.x, t = blockIdx.x;
  s_cnt[tid] = 0;
  if (tid < nw) s_base[tid] = __ldg(first + (long)tid * tiles + t);
  __syncthreads();
  const long base = (long)t * WS_TILE;
  const int valid = (int)min((long)WS_TILE, n - base);
  unsigned k[WS_ITEMS], r[WS_ITEMS];
  V v[VAL ? WS_ITEMS : 1];
#pragma unroll
  for (int c = 0; c < WS_ITEMS; c++) {
    const int e = c * RK_BLOCK + tid;
    if (e < valid) {
      k[c] = __ldcs(key + base + e);
      if constexpr (VAL) v[c] = __ldcs(val + base + e);
    }
  }
#pragma unroll
  for (int c = 0; c < WS_ITEMS; c++)
    r[c] = ws_slot(s_cnt, c * RK_BLOCK + tid < valid ? (int)ws_window(k[c], shift, nw) : -1);
  __syncthreads();
  // the windows' first slots within the tile: exclusive scan over the bins
  const unsigned tot = s_cnt[tid];
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
  for (int q = 0; q < RK_WARPS; q++) if (q < warp) wp += s_ws[q];
  s_cnt[tid] = wp + incl - tot;
  __syncthreads();
#pragma unroll
  for (int c = 0; c < WS_ITEMS; c++) {
    const int e = c * RK_BLOCK + tid;
    if (e < valid) {
      const unsigned w = ws_window(k[c], shift, nw);
      s_key[s_cnt[w] + r[c]] = k[c];
      if constexpr (VAL) s_val[s_cnt[w] + r[c]] = v[c];
      if (POS) pos[base + e] = s_base[w] + r[c];
    }
  }
  __syncthreads();
  // coalesced runs: slot e of the tile holds window w's key e - s_cnt[w]
#pragma unroll 4
  for (int e = tid; e < valid; e += RK_BLOCK) {
    const unsigned kk = s_key[e];
    const unsigned w = ws_window(kk, shift, nw);
    const unsigned g = s_base[w] + (unsigned)e - s_cnt[w];
    kout[g] = kk;
    if constexpr (VAL) vout[g] = s_val[e];
  }
}

// p[j] = s[key[j]] over keys that a window split grouped by source window:
// CTAs dispatched in order keep the reads within a few windows of s, which
// sit in L2 while they are read.  An index outside [0, n_src) reads nothing
// (its value is 0) and sets DEV_RANGE.  p may be key itself (4-byte values).
template <class V>
__global__ void __launch_bounds__(RK_BLOCK) k_window_gather(V *p, const V *__restrict__ s, const unsigned *key,
                                                            long n, unsigned n_src, const unsigned *gate,
                                                            unsigned *status) {
  if (gate && *(const volatile unsigned *)gate == 0) return;
  const long i0 = (long)blockIdx.x * (RK_BLOCK * SC_ITEMS) + threadIdx.x;
  unsigned k[SC_ITEMS];
  V v[SC_ITEMS];
#pragma unroll
  for (int u = 0; u < SC_ITEMS; u++) {
    const long i = i0 + (long)u * RK_BLOCK;
    k[u] = i < n ? __ldcs(key + i) : 0u;
  }
  bool bad = false;
#pragma unroll
  for (int u = 0; u < SC_ITEMS; u++) {
    v[u] = (V)0;
    if (i0 + (long)u * RK_BLOCK < n) {
      if (k[u] < n_src) v[u] = __ldg(s + k[u]);
      else bad = true;
    }
  }
  if (bad) atomicOr(status, DEV_RANGE);
#pragma unroll
  for (int u = 0; u < SC_ITEMS; u++) {
    const long i = i0 + (long)u * RK_BLOCK;
    if (i < n) p[i] = v[u];
  }
}

// d[i] = s[idx[i]], run only when (*gate != 0) == when_set
template <class V>
__global__ void __launch_bounds__(RK_BLOCK) k_gather_gated(V *__restrict__ d, const V *__restrict__ s,
                                                           const unsigned *__restrict__ idx, long n,
                                                           const unsigned *gate, int when_set) {
  if ((*(const volatile unsigned *)gate != 0) != (when_set != 0)) return;
  // grid-stride: launched with one CTA per 2048 elements it makes one pass;
  // launched with few CTAs it costs little when the gate turns it away
  for (long i0 = (long)blockIdx.x * (RK_BLOCK * SC_ITEMS) + threadIdx.x; i0 < n;
       i0 += (long)gridDim.x * (RK_BLOCK * SC_ITEMS)) {
    unsigned k[SC_ITEMS];
    V v[SC_ITEMS];
#pragma unroll
    for (int u = 0; u < SC_ITEMS; u++) {
      const long i = i0 + (long)u * RK_BLOCK;
      k[u] = i < n ? __ldcs(idx + i) : 0u;
    }
#pragma unroll
    for (int u = 0; u < SC_ITEMS; u++)
      if (i0 + (long)u * RK_BLOCK < n) v[u] = __ldg(s + k[u]);
#pragma unroll
    for (int u = 0; u < SC_ITEMS; u++) {
      const long i = i0 + (long)u * RK_BLOCK;
      if (i < n) __stcs(d + i, v[u]);
    }
  }
}

template <class K, class V, bool AUX, int IN, int OUT>
void launch_pass(const PassArgs<K, V> &a, int tiles) {
  constexpr size_t sm = pass_smem<K, V, AUX>();
  static bool attr = false;
  if (!attr) {
    GCVL_CK(cudaFuncSetAttribute(k_radix_pass<K, V, AUX, IN, OUT>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    attr = true;
  }
  k_radix_pass<K, V, AUX, IN, OUT><<<tiles, RK_BLOCK, sm, stream()>>>(a);
  launch_check("k_radix_pass");
}

inline int rk_tiles(long n) { return (int)((n + RK_TILE - 1) / RK_TILE); }
inline int sc_blocks(long n) { return (int)((n + RK_BLOCK * SC_ITEMS - 1) / (RK_BLOCK * SC_ITEMS)); }
// grid of the sorted-index scatter: grid-stride over at most 16 CTAs per
// SM, so that when its gate says "not this time" it costs a few
// microseconds instead of a launch of one CTA per 2048 elements
inline int sc_grid(long n) {
  const long need = (n + RK_BLOCK * SC_ITEMS - 1) / (RK_BLOCK * SC_ITEMS);
  const long cap = (long)st().sm_count * 16;
  return (int)(need < cap ? (need < 1 ? 1 : need) : cap);
}
inline size_t rk_state_bytes(long n) { return (size_t)rk_tiles(n) * 256 * 4; }
inline int ws_tiles(long n) { return (int)((n + WS_TILE - 1) / WS_TILE); }  // tiles of the window split
// top-8-bit windows of [0, n)
inline int window_shift(int n) { int b = bit_length((unsigned)(n > 1 ? n - 1 : 1)); return b > 8 ? b - 8 : 0; }

// the window counts of every tile of idx[0, n) and the gate word
inline void ws_hist(const int *idx, long n, int shift, int wbits, int tiles, unsigned *counts, unsigned *unsorted) {
  if (((uintptr_t)idx & 15) == 0)
    k_ws_hist<true><<<tiles, RK_BLOCK, 0, stream()>>>((const unsigned *)idx, n, shift, wbits, counts, unsorted);
  else
    k_ws_hist<false><<<tiles, RK_BLOCK, 0, stream()>>>((const unsigned *)idx, n, shift, wbits, counts, unsorted);
  launch_check("k_ws_hist");
}

// ------------------------------------------------ partitioned scatter ---
// d[idx[k]] = s[k] for k < n (idx in [0, n_d)) when d is larger than L2 can
// absorb random writes to (each would cost a DRAM read-modify-write of a
// sector): the (index, value) pairs are split by destination window (windows
// of at most 8 MB, at most 256 of them, with the same histogram, scan and
// split passes as the partitioned gather), then written window by window
// while each window sits in L2.  Ascending indices take one streaming scatter instead; the
// device decides (the kernels of the branch not taken return at once).
struct ScatterLayout { size_t kout, vout, counts, scan, flags, total; };
inline ScatterLayout scatter_layout(long n, size_t vsize) {
  ScatterLayout L;
  size_t o = 0;
  auto take = [&](size_t bytes) { size_t at = o; o += align_up(bytes, 256); return at; };
  L.kout = take((size_t)n * 4);
  L.vout = take((size_t)n * vsize);
  L.counts = take((size_t)ws_tiles(n) * WS_MAXW * 4);
  L.scan = take((size_t)add_suz_scratch(ws_tiles(n) * WS_MAXW) * 8);
  L.flags = take(256);
  L.total = o + 256;  // room to align the base
  return L;
}
bool scatter_partitioned_wanted(long n_d, size_t vsize) { return (size_t)n_d * vsize > (size_t)RK_DIRECT_MAX * 4; }
size_t scatter_partitioned_bytes(long n, size_t vsize) { return scatter_layout(n, vsize).total; }
// Window sizes, measured on int32 permutations: the gather runs fastest
// with at least 8 windows of at most 64 MB (2.81 -> 2.69 ms at 2^28 against
// 32 MB windows), the scatter with windows of at most 8 MB (2^28: 3.28 ms
// with 32 MB windows, 3.06 with 16, 2.78 with 8; 2^25: 0.45, 0.40, 0.36).
#ifndef GCVL_WS_GATHER_MB
#define GCVL_WS_GATHER_MB 64
#endif
#ifndef GCVL_WS_GATHER_MINBITS
#define GCVL_WS_GATHER_MINBITS 3
#endif
#ifndef GCVL_WS_SCATTER_MB
#define GCVL_WS_SCATTER_MB 8
#endif
// windows of at most `mb` MB of `bytes`, a power of two from 2^min_bits to
// 256: (log2 of the count, shift of an index of [0, len) to its window)
inline void ws_windows(size_t bytes, long len, int mb, int min_bits, int *wbits, int *shift) {
  int wb = min_bits;
  while (wb < 8 && (bytes >> wb) > ((size_t)mb << 20)) ++wb;
  const int nb = bit_length((unsigned)(len > 1 ? len - 1 : 1));
  *wbits = wb;
  *shift = nb > wb ? nb - wb : 0;
}

template <class V>
void scatter_partitioned(V *d, const V *s, const int *idx, int n, int n_d, vec_p scratch) {
  State &S = st();
  if (n <= 0) return;
  ScatterLayout L = scatter_layout(n, sizeof(V));
  char *raw = (char *)scratch_or_work(scratch, L.total);
  if (!raw) return;
  char *mem = (char *)align_up((size_t)raw, 256);
  unsigned *kout = (unsigned *)(mem + L.kout);
  V *vout = (V *)(mem + L.vout);
  unsigned *counts = (unsigned *)(mem + L.counts);
  void *scan_scratch = mem + L.scan;
  unsigned *unsorted = (unsigned *)(mem + L.flags);  // the gate: non-zero when some index exceeds its successor
  int wbits, shift;
  ws_windows((size_t)n_d * sizeof(V), n_d, GCVL_WS_SCATTER_MB, 1, &wbits, &shift);
  const int nw = 1 << wbits;
  const int tiles = ws_tiles(n);
  constexpr size_t smem = ws_split_smem<V, true>();
  static bool attr = false;
  if (!attr) {
    GCVL_CK(cudaFuncSetAttribute(k_window_split<false, V, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem));
    attr = true;
  }
  if (!GCVL_CK(cudaMemsetAsync(unsorted, 0, 4, S.stream))) return;
  ws_hist(idx, n, shift, wbits, tiles, counts, unsorted);
  k_sorted_scatter<V><<<sc_grid(n), RK_BLOCK, 0, S.stream>>>(d, s, idx, n, unsorted);
  launch_check("k_sorted_scatter");
  add_suz(counts, counts, nw * tiles, scan_scratch);  // first slot of every (window, tile)
  k_window_split<false, V, true><<<tiles, RK_BLOCK, smem, S.stream>>>((const unsigned *)idx, n, shift, wbits, counts,
                                                                      unsorted, kout, nullptr, s, vout);
  launch_check("k_window_split");
  k_window_scatter<V><<<sc_blocks(n), RK_BLOCK, 0, S.stream>>>(d, kout, vout, n, unsorted);
  launch_check("k_window_scatter");
}

// ------------------------------------------------- partitioned gather ---
// d[k] = s[idx[k]] for k < n (idx in [0, n_src)) when s is larger than L2 can
// serve random reads from: each random 4- or 8-byte read from DRAM costs a
// whole sector, and most miss.  Instead the indices are split by source
// window (at least 8 windows of at most 64 MB, at most 256), with pos[k] = where
// index k went; a gather in window order reads each window of s while it
// sits in L2, into p; and d[k] = p[pos[k]] reads p through as many sequential
// runs as there are windows, few enough that L1 and L2 keep each run's
// current lines.  The passes stream: 4 (histogram) + 12 (split) + 12 + 12
// bytes per 4-byte element.  Ascending indices take one plain gather
// instead; the device decides, as for the scatter.
struct GatherLayout { size_t kout, pos, p, counts, scan, flags, total; };
inline GatherLayout gather_layout(long n, size_t vsize) {
  GatherLayout L;
  size_t o = 0;
  auto take = [&](size_t bytes) { size_t at = o; o += align_up(bytes, 256); return at; };
  L.kout = take((size_t)n * 4);
  L.pos = take((size_t)n * 4);
  L.p = vsize == 4 ? L.kout : take((size_t)n * vsize);  // 4-byte values overwrite their keys in place
  L.counts = take((size_t)ws_tiles(n) * WS_MAXW * 4);
  L.scan = take((size_t)add_suz_scratch(ws_tiles(n) * WS_MAXW) * 8);
  L.flags = take(256);
  L.total = o + 256;  // room to align the base
  return L;
}
bool gather_partitioned_wanted(long n_src, long n, size_t vsize) {
  return (size_t)n_src * vsize > ((size_t)64 << 20) && n >= (1L << 20);
}
size_t gather_partitioned_bytes(long n, size_t vsize) { return gather_layout(n, vsize).total; }

template <class V>
void gather_partitioned(V *d, const V *s, const int *idx, int n, int n_src, vec_p scratch) {
  State &S = st();
  if (n <= 0) return;
  GatherLayout L = gather_layout(n, sizeof(V));
  char *raw = (char *)scratch_or_work(scratch, L.total);
  if (!raw) return;
  char *mem = (char *)align_up((size_t)raw, 256);
  unsigned *kout = (unsigned *)(mem + L.kout);
  unsigned *pos = (unsigned *)(mem + L.pos);
  V *p = (V *)(mem + L.p);
  unsigned *counts = (unsigned *)(mem + L.counts);
  void *scan_scratch = mem + L.scan;
  unsigned *unsorted = (unsigned *)(mem + L.flags);  // the gate: non-zero when some index exceeds its successor
  int wbits, shift;
  ws_windows((size_t)n_src * sizeof(V), n_src, GCVL_WS_GATHER_MB, GCVL_WS_GATHER_MINBITS, &wbits, &shift);
  const int nw = 1 << wbits;
  const int tiles = ws_tiles(n);
  GCVL_CK(cudaMemsetAsync(unsorted, 0, 4, S.stream));
  ws_hist(idx, n, shift, wbits, tiles, counts, unsorted);
  k_gather_gated<V><<<sc_grid(n), RK_BLOCK, 0, S.stream>>>(d, s, (const unsigned *)idx, n, unsorted, 0);
  launch_check("k_gather_gated");
  add_suz(counts, counts, nw * tiles, scan_scratch);  // first slot of every (window, tile)
  k_window_split<true><<<tiles, RK_BLOCK, ws_split_smem<unsigned, false>(), S.stream>>>(
      (const unsigned *)idx, n, shift, wbits, counts, unsorted, kout, pos);
  launch_check("k_window_split");
  k_window_gather<V><<<sc_blocks(n), RK_BLOCK, 0, S.stream>>>(p, s, kout, n, (unsigned)n_src, unsorted,
                                                              S.d_status);
  launch_check("k_window_gather");
  k_gather_gated<V><<<sc_blocks(n), RK_BLOCK, 0, S.stream>>>(d, p, pos, n, unsorted, 1);
  launch_check("k_gather_gated");
}
template void gather_partitioned<unsigned>(unsigned *, const unsigned *, const int *, int, int, vec_p);
template void gather_partitioned<unsigned long long>(unsigned long long *, const unsigned long long *,
                                                     const int *, int, int, vec_p);
template void scatter_partitioned<unsigned>(unsigned *, const unsigned *, const int *, int, int, vec_p);
template void scatter_partitioned<unsigned long long>(unsigned long long *, const unsigned long long *,
                                                      const int *, int, int, vec_p);

// ------------------------------------------------------------- rank ---
struct RankLayout {
  size_t key_a, key_b, idx_a, idx_b, aux_a, aux_b, hist, state, wstate, counter, total;
};
inline RankLayout rank_layout(int n, int is_double, int seg) {
  RankLayout L;
  size_t ks = is_double ? 8 : 4;
  size_t o = 0;
  auto take = [&](size_t bytes) { size_t at = o; o += align_up(bytes, 256); return at; };
  L.key_a = take((size_t)n * ks);
  L.key_b = take((size_t)n * ks);
  L.idx_a = take((size_t)n * 4);
  L.idx_b = take((size_t)n * 4);
  L.aux_a = take(seg ? (size_t)n * 4 : 0);
  L.aux_b = take(seg ? (size_t)n * 4 : 0);
  L.hist = take((RK_MAXPASS + 1) * 256 * 4);  // every pass's digit starts, then the window starts
  L.counter = take((RK_MAXPASS + 1) * 4);
  L.state = take(rk_state_bytes(n));
  L.wstate = take(n > RK_DIRECT_MAX ? rk_state_bytes(n) : 0);  // the last pass's window look-back
  L.total = o + 256;  // room to align the base
  return L;
}
int rank_units(int n, int is_double, int seg) {
  if (n <= 0) return 0;
  return (int)((rank_layout(n, is_double, seg).total + 7) / 8);
}

template <class K>
void rank_impl(vec_p d, vec_p s, vec_p sd, int n, int m, vec_p scratch, int is_double, int up) {
  ensure_init();
  State &S = st();
  if (n <= 0) return;
  const bool seg = sd != nullptr && m > 1;
  RankLayout L = rank_layout(n, is_double, seg);
  char *raw = (char *)scratch_or_work(scratch, L.total);
  if (!raw) return;
  char *mem = (char *)align_up((size_t)raw, 256);
  const int key_passes = is_double ? 8 : 4;
  int seg_passes = 0;
  if (seg) seg_passes = (bit_length((unsigned)(m - 1)) + 7) / 8;
  if (seg && seg_passes == 0) seg_passes = 1;
  const int passes = key_passes + seg_passes;
  const int tiles = rk_tiles(n);
  const bool direct = n <= RK_DIRECT_MAX;
  unsigned *hist = (unsigned *)(mem + L.hist);
  unsigned *counters = (unsigned *)(mem + L.counter);
  unsigned *state = (unsigned *)(mem + L.state);
  GCVL_CK(cudaMemsetAsync(hist, 0, RK_MAXPASS * 256 * 4, S.stream));
  GCVL_CK(cudaMemsetAsync(counters, 0, (RK_MAXPASS + 1) * 4, S.stream));

  // histograms of every pass (and, segmented, the staged keys)
  RankPrep p;
  p.src = s; p.n = n; p.is_double = is_double; p.up = up; p.seg = seg ? 1 : 0;
  p.write_arrays = seg ? 1 : 0;
  p.sv = seg ? seg_view(sd, n, m) : SegView{nullptr, nullptr, nullptr, nullptr, n, 1};
  p.key = mem + L.key_a; p.idx = (unsigned *)(mem + L.idx_a);
  p.aux = seg ? (unsigned *)(mem + L.aux_a) : nullptr;
  p.hist = hist; p.key_passes = key_passes; p.seg_passes = seg_passes;
  int pg = S.sm_count * 8;
  long need = ((long)n + RK_BLOCK - 1) / RK_BLOCK;
  if (pg > need) pg = (int)need;
  k_rank_prep<<<pg, RK_BLOCK, 0, S.stream>>>(p);
  launch_check("k_rank_prep");
  k_rank_digit_starts<<<1, 256, 0, S.stream>>>(hist, passes);
  launch_check("k_rank_digit_starts");

  // ping-pong buffers
  char *kA = mem + L.key_a, *kB = mem + L.key_b;
  unsigned *iA = (unsigned *)(mem + L.idx_a), *iB = (unsigned *)(mem + L.idx_b);
  unsigned *aA = seg ? (unsigned *)(mem + L.aux_a) : nullptr, *aB = seg ? (unsigned *)(mem + L.aux_b) : nullptr;
  const int *segoff = seg ? seg_view(sd, n, m).off : nullptr;
  // last pass output when the ranks go through the window partition: the
  // pair arrays take the buffers the last pass does not read, grouped by
  // the window of the index (256 windows of the rank vector)
  unsigned *pidx = nullptr, *ppos = nullptr;
  const int wshift = window_shift(n);
  unsigned *wst = hist + RK_MAXPASS * 256;
  unsigned *wstate = (unsigned *)(mem + L.wstate);
  if (!direct) {
    k_window_starts<<<1, 256, 0, S.stream>>>(wst, n, wshift);
    launch_check("k_window_starts");
    GCVL_CK(cudaMemsetAsync(wstate, 0, rk_state_bytes(n), S.stream));
  }
  for (int q = 0; q < passes; q++) {
    GCVL_CK(cudaMemsetAsync(state, 0, rk_state_bytes(n), S.stream));
    const bool final = (q == passes - 1);
    const bool keypass = q < key_passes;
    if (final) { pidx = iB; ppos = (unsigned *)kB; }
    if (keypass) {
      PassArgs<K, unsigned> a{};
      a.kin = (const K *)kA; a.vin = iA; a.ain = aA;
      a.kout = (K *)kB; a.vout = iB; a.aout = aB;
      a.src = s; a.up = up;
      a.rank = (int *)d; a.segoff = nullptr; a.pidx = pidx; a.ppos = ppos;
      a.wstarts = wst; a.wstate = wstate; a.wshift = wshift;
      a.starts = hist + q * 256; a.state = state; a.counter = counters + q;
      a.n = n; a.shift = 8 * q; a.status = S.d_status; a.spin_limit = S.spin_limit;
      if (seg) {
        launch_pass<K, unsigned, true, IN_ARRAYS, OUT_ARRAYS>(a, tiles);
      } else if (q == 0) {
        launch_pass<K, unsigned, false, IN_SRC, OUT_ARRAYS>(a, tiles);
      } else if (!final) {
        launch_pass<K, unsigned, false, IN_ARRAYS, OUT_ARRAYS>(a, tiles);
      } else if (direct) {
        launch_pass<K, unsigned, false, IN_ARRAYS, OUT_RANK>(a, tiles);
      } else {
        launch_pass<K, unsigned, false, IN_ARRAYS, OUT_WIN>(a, tiles);
      }
    } else {
      // segment passes: the segment number is the key, indices ride along
      PassArgs<unsigned, unsigned> a{};
      const bool first_seg = (q == key_passes);
      a.kin = first_seg ? aA : (const unsigned *)kA; a.vin = iA; a.ain = nullptr;
      a.kout = (unsigned *)kB; a.vout = iB; a.aout = nullptr;
      a.rank = (int *)d; a.segoff = segoff; a.pidx = pidx; a.ppos = ppos;
      a.wstarts = wst; a.wstate = wstate; a.wshift = wshift;
      a.starts = hist + q * 256; a.state = state; a.counter = counters + q;
      a.n = n; a.shift = 8 * (q - key_passes); a.status = S.d_status; a.spin_limit = S.spin_limit;
      if (!final) launch_pass<unsigned, unsigned, false, IN_ARRAYS, OUT_ARRAYS>(a, tiles);
      else if (direct) launch_pass<unsigned, unsigned, false, IN_ARRAYS, OUT_RANK>(a, tiles);
      else launch_pass<unsigned, unsigned, false, IN_ARRAYS, OUT_WIN>(a, tiles);
    }
    if (!final) {
      std::swap(kA, kB); std::swap(iA, iB);
      if (keypass) std::swap(aA, aB);
    }
  }
  if (!direct) {
    // (index, position) pairs grouped by window of the index ->
    // rank[index] = position, one window at a time
    k_window_scatter<unsigned><<<sc_blocks(n), RK_BLOCK, 0, S.stream>>>((unsigned *)d, pidx, (const unsigned *)ppos, n,
                                                               nullptr);
    launch_check("k_window_scatter");
  }
}

}  // namespace gcvl

using namespace gcvl;

GCVL_EXPORT void rku_luz(vec_p d, vec_p s, int len, vec_p scratch) { rank_impl<unsigned>(d, s, nullptr, len, 1, scratch, 0, 1); }
GCVL_EXPORT int rku_luz_scratch(int len) { return rank_units(len, 0, 0); }
GCVL_EXPORT unsigned rku_luz_inplace(void) { return INPLACE_NONE; }
GCVL_EXPORT void rkd_luz(vec_p d, vec_p s, int len, vec_p scratch) { rank_impl<unsigned>(d, s, nullptr, len, 1, scratch, 0, 0); }
GCVL_EXPORT int rkd_luz_scratch(int len) { return rank_units(len, 0, 0); }
GCVL_EXPORT unsigned rkd_luz_inplace(void) { return INPLACE_NONE; }
GCVL_EXPORT void rku_lez(vec_p d, vec_p s, vec_p sd, int n, int m, vec_p scratch) { rank_impl<unsigned>(d, s, sd, n, m, scratch, 0, 1); }
GCVL_EXPORT int rku_lez_scratch(int n, int m) { return rank_units(n, 0, m > 1); }
GCVL_EXPORT unsigned rku_lez_inplace(void) { return INPLACE_NONE; }
GCVL_EXPORT void rkd_lez(vec_p d, vec_p s, vec_p sd, int n, int m, vec_p scratch) { rank_impl<unsigned>(d, s, sd, n, m, scratch, 0, 0); }
GCVL_EXPORT int rkd_lez_scratch(int n, int m) { return rank_units(n, 0, m > 1); }
GCVL_EXPORT unsigned rkd_lez_inplace(void) { return INPLACE_NONE; }
GCVL_EXPORT void rku_lud(vec_p d, vec_p s, int len, vec_p scratch) { rank_impl<unsigned long long>(d, s, nullptr, len, 1, scratch, 1, 1); }
GCVL_EXPORT int rku_lud_scratch(int len) { return rank_units(len, 1, 0); }
GCVL_EXPORT unsigned rku_lud_inplace(void) { return INPLACE_NONE; }
GCVL_EXPORT void rkd_lud(vec_p d, vec_p s, int len, vec_p scratch) { rank_impl<unsigned long long>(d, s, nullptr, len, 1, scratch, 1, 0); }
GCVL_EXPORT int rkd_lud_scratch(int len) { return rank_units(len, 1, 0); }
GCVL_EXPORT unsigned rkd_lud_inplace(void) { return INPLACE_NONE; }
GCVL_EXPORT void rku_led(vec_p d, vec_p s, vec_p sd, int n, int m, vec_p scratch) { rank_impl<unsigned long long>(d, s, sd, n, m, scratch, 1, 1); }
GCVL_EXPORT int rku_led_scratch(int n, int m) { return rank_units(n, 1, m > 1); }
GCVL_EXPORT unsigned rku_led_inplace(void) { return INPLACE_NONE; }
GCVL_EXPORT void rkd_led(vec_p d, vec_p s, vec_p sd, int n, int m, vec_p scratch) { rank_impl<unsigned long long>(d, s, sd, n, m, scratch, 1, 0); }
GCVL_EXPORT int rkd_led_scratch(int n, int m) { return rank_units(n, 1, m > 1); }
GCVL_EXPORT unsigned rkd_led_inplace(void) { return INPLACE_NONE; }
