// rank.cu -- stable radix rank, up and down, int and double, segmented and
// unsegmented (nesl/cvl/serial/rank.c:49-362).
//
// d[j] is the position of element j in the stable sorted order of its
// segment.  Keys are made order-preserving unsigned integers exactly as the
// serial CVL does: int keys flip the sign bit (up) or every other bit
// (down), rank.c:94-99; double keys flip all bits of negatives and the sign
// bit of the rest, and down ranks complement that, rank.c:258-280.  A
// segmented rank is a stable sort by (segment, key): the key passes carry
// each element's segment number, then further passes sort by it.
//
// GPU design (onesweep style): one prepare pass writes transformed keys and
// indices and builds every pass's 256-bin digit histogram at once with
// shared-memory atomics.  Then one scatter pass per 8-bit digit: each CTA
// ranks its tile stably with warp match/ballot, learns how many earlier
// tiles' elements fall in each digit by a per-digit decoupled look-back,
// reorders the tile in shared memory and writes coalesced runs.  The last
// pass writes d[index] = position directly.
#include "gcvl.cuh"

#include <utility>

namespace gcvl {

constexpr int RK_BLOCK = 256, RK_ITEMS = 16, RK_TILE = RK_BLOCK * RK_ITEMS;
constexpr int RK_WARPS = RK_BLOCK / 32;
constexpr int RK_MAXPASS = 12;
constexpr int RK_LB = 8;  // predecessors read per look-back round trip
enum : unsigned long long { RK_AGG = 1ULL << 62, RK_INC = 2ULL << 62, RK_MASK = (1ULL << 62) - 1 };

struct RankPrep {
  const void *src;
  int n, is_double, up, seg;
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

__global__ void __launch_bounds__(RK_BLOCK) k_rank_prep(RankPrep p) {
  __shared__ unsigned s_hist[RK_MAXPASS * 256];
  const int passes = p.key_passes + p.seg_passes;
  for (int i = threadIdx.x; i < passes * 256; i += RK_BLOCK) s_hist[i] = 0;
  __syncthreads();
  const long stride = (long)gridDim.x * RK_BLOCK;
  for (long i = (long)blockIdx.x * RK_BLOCK + threadIdx.x; i < p.n; i += stride) {
    unsigned long long k;
    if (p.is_double) {
      k = rk_key64(((const unsigned long long *)p.src)[i], p.up);
      ((unsigned long long *)p.key)[i] = k;
    } else {
      unsigned x = ((const unsigned *)p.src)[i];
      unsigned kk = x ^ (p.up ? 0x80000000u : 0x7FFFFFFFu);
      ((unsigned *)p.key)[i] = kk;
      k = kk;
    }
    p.idx[i] = (unsigned)i;
    for (int q = 0; q < p.key_passes; q++) atomicAdd(&s_hist[q * 256 + (int)((k >> (8 * q)) & 255)], 1u);
    if (p.seg) {
      unsigned sg = (unsigned)seg_of(p.sv, (int)i);
      p.aux[i] = sg;
      for (int q = 0; q < p.seg_passes; q++)
        atomicAdd(&s_hist[(p.key_passes + q) * 256 + ((sg >> (8 * q)) & 255)], 1u);
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < passes * 256; i += RK_BLOCK)
    if (s_hist[i]) atomicAdd(&p.hist[i], s_hist[i]);
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

template <class K> struct PassArgs {
  const K *kin; const unsigned *iin; const unsigned *ain;
  K *kout; unsigned *iout; unsigned *aout;
  int *rank;           // final pass output
  const int *segoff;   // final pass of a segmented rank: segment offsets
  const unsigned *starts;  // this pass's digit starts
  unsigned long long *state;  // [tiles][256]
  unsigned *counter;
  int n, shift;
  unsigned *status;
  int spin_limit;
};

template <class K, bool AUX, bool FINAL>
__global__ void __launch_bounds__(RK_BLOCK) k_rank_pass(PassArgs<K> a) {
  extern __shared__ __align__(16) unsigned char rk_smem[];
  K *s_key = (K *)rk_smem;
  unsigned *s_idx = (unsigned *)(s_key + RK_TILE);
  unsigned *s_aux = s_idx + RK_TILE;
  unsigned *s_cnt = s_aux + (AUX ? RK_TILE : 0);  // [RK_WARPS][256]
  unsigned *s_loc = s_cnt + RK_WARPS * 256;        // local digit offsets
  long long *s_gb = (long long *)(s_loc + 256);    // global base per digit
  __shared__ unsigned s_tile;

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) s_tile = atomicAdd(a.counter, 1u);
  for (int i = tid; i < RK_WARPS * 256; i += RK_BLOCK) s_cnt[i] = 0;
  __syncthreads();
  const int tile = (int)s_tile;
  const long base = (long)tile * RK_TILE;
  const int valid = (int)min((long)RK_TILE, (long)a.n - base);

  // this warp's contiguous range, 32 elements per step
  K key[RK_ITEMS];
  unsigned idx[RK_ITEMS], aux[RK_ITEMS], wr[RK_ITEMS];
  int dig[RK_ITEMS];
  const int wbase = warp * 32 * RK_ITEMS;
#pragma unroll
  for (int c = 0; c < RK_ITEMS; c++) {
    int e = wbase + c * 32 + lane;
    if (e < valid) {
      key[c] = __ldcs(a.kin + base + e);
      idx[c] = __ldcs(a.iin + base + e);
      if (AUX) aux[c] = __ldcs(a.ain + base + e);
      dig[c] = (int)((key[c] >> a.shift) & 255);
    } else {
      dig[c] = -1;
    }
  }
  unsigned *cnt = s_cnt + warp * 256;
  const unsigned lt = (1u << lane) - 1u;
#pragma unroll
  for (int c = 0; c < RK_ITEMS; c++) {
    int d = dig[c];
    unsigned peers = __match_any_sync(0xffffffffu, d);
    unsigned r = 0;
    if (d >= 0) r = cnt[d] + __popc(peers & lt);
    __syncwarp();
    if (d >= 0 && (peers & lt) == 0) cnt[d] += __popc(peers);
    __syncwarp();
    wr[c] = r;
  }
  __syncthreads();

  // per digit: tile count, per-warp exclusive offsets
  const int dd = tid;  // RK_BLOCK == 256 digits
  unsigned tot = 0;
#pragma unroll
  for (int w = 0; w < RK_WARPS; w++) {
    unsigned c = s_cnt[w * 256 + dd];
    s_cnt[w * 256 + dd] = tot;
    tot += c;
  }
  // publish this tile's digit count, then look back for earlier tiles'
  unsigned long long *st = a.state + (long)tile * 256 + dd;
  if (tile == 0) {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(st), "l"(RK_INC | tot) : "memory");
  } else {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(st), "l"(RK_AGG | tot) : "memory");
  }
  // look back for this digit: RK_LB predecessors per round trip, nearest
  // first, until an inclusive count is found (bounded waits).  Each status
  // word is self-contained, so relaxed loads suffice and all RK_LB are in
  // flight together.
  unsigned long long prefix = 0;
  if (tile > 0) {
    long t0 = tile - 1;
    bool done = false;
    while (!done && t0 >= 0) {
      unsigned long long w[RK_LB];
#pragma unroll
      for (int j = 0; j < RK_LB; j++) {
        w[j] = RK_INC;  // beyond tile 0: an inclusive zero
        if (t0 - j >= 0)
          asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(w[j]) : "l"(a.state + (t0 - j) * 256 + dd) : "memory");
      }
#pragma unroll
      for (int j = 0; j < RK_LB; j++) {
        if (done) break;
        int it = 0;
        while (w[j] == 0) {
          if (++it >= a.spin_limit) { atomicOr(a.status, DEV_TIMEOUT); w[j] = RK_INC; break; }
          __nanosleep(32);
          asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(w[j]) : "l"(a.state + (t0 - j) * 256 + dd) : "memory");
        }
        prefix += w[j] & RK_MASK;
        if (w[j] & RK_INC) done = true;
      }
      t0 -= RK_LB;
    }
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(st), "l"(RK_INC | (prefix + tot)) : "memory");
  }
  // exclusive scan of tile counts over the digits -> local offsets
  {
    unsigned v = tot, incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      unsigned x = shfl_up(incl, o);
      if (lane >= o) incl += x;
    }
    __shared__ unsigned s_ws[RK_WARPS];
    if (lane == 31) s_ws[warp] = incl;
    __syncthreads();
    unsigned wp = 0;
#pragma unroll
    for (int w = 0; w < RK_WARPS; w++) if (w < warp) wp += s_ws[w];
    unsigned loc = wp + incl - v;
    s_loc[dd] = loc;
    s_gb[dd] = (long long)__ldg(a.starts + dd) + (long long)prefix - (long long)loc;
  }
  __syncthreads();
  // reorder the tile in shared memory
#pragma unroll
  for (int c = 0; c < RK_ITEMS; c++) {
    int d = dig[c];
    if (d >= 0) {
      unsigned lp = s_loc[d] + s_cnt[warp * 256 + d] + wr[c];
      s_key[lp] = key[c];
      s_idx[lp] = idx[c];
      if (AUX) s_aux[lp] = aux[c];
    }
  }
  __syncthreads();
  // coalesced runs out
  for (int e = tid; e < valid; e += RK_BLOCK) {
    K k = s_key[e];
    int d = (int)((k >> a.shift) & 255);
    long g = s_gb[d] + e;
    if (FINAL) {
      int r = (int)g;
      if (a.segoff) r -= __ldg(a.segoff + (int)k);
      a.rank[s_idx[e]] = r;
    } else {
      a.kout[g] = k;
      a.iout[g] = s_idx[e];
      if (AUX) a.aout[g] = s_aux[e];
    }
  }
}

template <class K, bool AUX, bool FINAL> size_t pass_smem() {
  return (size_t)RK_TILE * sizeof(K) + (size_t)RK_TILE * 4 * (AUX ? 2 : 1) + RK_WARPS * 256 * 4 +
         256 * 4 + 256 * 8;
}

template <class K, bool AUX, bool FINAL>
void launch_pass(PassArgs<K> a, int tiles) {
  size_t sm = pass_smem<K, AUX, FINAL>();
  static bool attr = false;
  if (!attr) {
    GCVL_CK(cudaFuncSetAttribute(k_rank_pass<K, AUX, FINAL>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    attr = true;
  }
  k_rank_pass<K, AUX, FINAL><<<tiles, RK_BLOCK, sm, stream()>>>(a);
  launch_check("k_rank_pass");
}

struct RankLayout {
  size_t key_a, key_b, idx_a, idx_b, aux_a, aux_b, hist, state, counter, total;
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
  L.hist = take(RK_MAXPASS * 256 * 4);
  L.counter = take(RK_MAXPASS * 4);
  int tiles = (n + RK_TILE - 1) / RK_TILE;
  L.state = take((size_t)tiles * 256 * 8);
  L.total = o;
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
  char *mem = (char *)scratch_or_work(scratch, L.total);
  if (!mem) return;
  const int key_passes = is_double ? 8 : 4;
  int seg_passes = 0;
  if (seg) {
    unsigned mm = (unsigned)(m - 1);
    int bits = mm ? 32 - __builtin_clz(mm) : 1;
    seg_passes = (bits + 7) / 8;
  }
  const int passes = key_passes + seg_passes;
  const int tiles = (n + RK_TILE - 1) / RK_TILE;
  unsigned *hist = (unsigned *)(mem + L.hist);
  unsigned *counters = (unsigned *)(mem + L.counter);
  unsigned long long *state = (unsigned long long *)(mem + L.state);
  GCVL_CK(cudaMemsetAsync(hist, 0, RK_MAXPASS * 256 * 4, S.stream));
  GCVL_CK(cudaMemsetAsync(counters, 0, RK_MAXPASS * 4, S.stream));

  RankPrep p;
  p.src = s; p.n = n; p.is_double = is_double; p.up = up; p.seg = seg ? 1 : 0;
  p.sv = seg ? seg_view(sd, n, m) : SegView{nullptr, nullptr, nullptr, nullptr, n, 1};
  p.key = mem + L.key_a; p.idx = (unsigned *)(mem + L.idx_a);
  p.aux = seg ? (unsigned *)(mem + L.aux_a) : nullptr;
  p.hist = hist; p.key_passes = key_passes; p.seg_passes = seg_passes;
  int pg = S.sm_count * 4;
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
  for (int q = 0; q < passes; q++) {
    GCVL_CK(cudaMemsetAsync(state, 0, (size_t)tiles * 256 * 8, S.stream));
    const bool final = (q == passes - 1);
    const bool keypass = q < key_passes;
    if (keypass) {
      PassArgs<K> a{};
      a.kin = (const K *)kA; a.iin = iA; a.ain = aA;
      a.kout = (K *)kB; a.iout = iB; a.aout = aB;
      a.rank = (int *)d; a.segoff = nullptr;
      a.starts = hist + q * 256; a.state = state; a.counter = counters + q;
      a.n = n; a.shift = 8 * q; a.status = S.d_status; a.spin_limit = S.spin_limit;
      if (final) launch_pass<K, false, true>(a, tiles);
      else if (seg) launch_pass<K, true, false>(a, tiles);
      else launch_pass<K, false, false>(a, tiles);
    } else {
      // segment passes: the segment number is the key, indices ride along
      PassArgs<unsigned> a{};
      const bool first_seg = (q == key_passes);
      a.kin = first_seg ? aA : (const unsigned *)kA; a.iin = iA; a.ain = nullptr;
      a.kout = (unsigned *)kB; a.iout = iB; a.aout = nullptr;
      a.rank = (int *)d; a.segoff = segoff;
      a.starts = hist + q * 256; a.state = state; a.counter = counters + q;
      a.n = n; a.shift = 8 * (q - key_passes); a.status = S.d_status; a.spin_limit = S.spin_limit;
      if (final) launch_pass<unsigned, false, true>(a, tiles);
      else launch_pass<unsigned, false, false>(a, tiles);
    }
    if (!final) {
      std::swap(kA, kB); std::swap(iA, iB);
      if (keypass) std::swap(aA, aB);
    }
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
