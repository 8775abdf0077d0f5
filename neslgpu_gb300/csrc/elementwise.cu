// elementwise.cu -- the *_wu* maps (nesl/cvl/serial/elwise.c:192-298).
//
// Each map is one streaming kernel: coalesced loads, four independent
// elements in flight per thread, a grid sized to the SM count.  C
// semantics are kept exactly: int / and % truncate, shifts take the count
// modulo 32 (what the serial CVL computes on x86-64 and aarch64), rou is
// (int)(x + 0.5), floor/ceil convert with (int).  Transcendentals call the
// CUDA double-precision math library.
#include "gcvl.cuh"
#include "elt_ops.cuh"

namespace gcvl {

constexpr int EBLOCK = 256;
constexpr int EUNROLL = 4;

inline int ew_grid(long n) {
  long per_cta = (long)EBLOCK * EUNROLL;
  long g = (n + per_cta - 1) / per_cta;
  long cap = (long)st().sm_count * 16;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return (int)g;
}

template <class F, class TO, class TI>
__global__ void __launch_bounds__(EBLOCK) k_map1(TO *__restrict__ d, const TI *__restrict__ s, long n) {
  const long stride = (long)gridDim.x * EBLOCK * EUNROLL;
  for (long b = (long)blockIdx.x * EBLOCK * EUNROLL + threadIdx.x; b < n; b += stride) {
    TI x[EUNROLL];
#pragma unroll
    for (int u = 0; u < EUNROLL; u++) {
      long i = b + (long)u * EBLOCK;
      if (i < n) x[u] = __ldcs(s + i);
    }
#pragma unroll
    for (int u = 0; u < EUNROLL; u++) {
      long i = b + (long)u * EBLOCK;
      if (i < n) d[i] = F::f(x[u]);
    }
  }
}

template <class F, class TO, class TI>
__global__ void __launch_bounds__(EBLOCK) k_map2(TO *__restrict__ d, const TI *__restrict__ s1,
                                                const TI *__restrict__ s2, long n) {
  const long stride = (long)gridDim.x * EBLOCK * EUNROLL;
  for (long b = (long)blockIdx.x * EBLOCK * EUNROLL + threadIdx.x; b < n; b += stride) {
    TI x[EUNROLL], y[EUNROLL];
#pragma unroll
    for (int u = 0; u < EUNROLL; u++) {
      long i = b + (long)u * EBLOCK;
      if (i < n) { x[u] = __ldcs(s1 + i); y[u] = __ldcs(s2 + i); }
    }
#pragma unroll
    for (int u = 0; u < EUNROLL; u++) {
      long i = b + (long)u * EBLOCK;
      if (i < n) d[i] = F::f(x[u], y[u]);
    }
  }
}

template <class T>
__global__ void __launch_bounds__(EBLOCK) k_select(T *__restrict__ d, const int *__restrict__ c,
                                                  const T *__restrict__ a, const T *__restrict__ b,
                                                  long n) {
  const long stride = (long)gridDim.x * EBLOCK * EUNROLL;
  for (long q = (long)blockIdx.x * EBLOCK * EUNROLL + threadIdx.x; q < n; q += stride) {
    int cc[EUNROLL];
    T x[EUNROLL], y[EUNROLL];
#pragma unroll
    for (int u = 0; u < EUNROLL; u++) {
      long i = q + (long)u * EBLOCK;
      if (i < n) { cc[u] = __ldcs(c + i); x[u] = __ldcs(a + i); y[u] = __ldcs(b + i); }
    }
#pragma unroll
    for (int u = 0; u < EUNROLL; u++) {
      long i = q + (long)u * EBLOCK;
      if (i < n) d[i] = cc[u] ? x[u] : y[u];
    }
  }
}

template <class T>
__global__ void __launch_bounds__(EBLOCK) k_fillv(T *__restrict__ d, T v, long n) {
  const long stride = (long)gridDim.x * EBLOCK;
  for (long i = (long)blockIdx.x * EBLOCK + threadIdx.x; i < n; i += stride) d[i] = v;
}

// ---- RAND: bit-exact lrand48 stream.  X' = (a X + c) mod 2^48 is affine,
// so element i's state is reached directly by composing the map i+1 times
// (binary powering); the host advances the state by len afterwards.
struct Affine48 { unsigned long long a, c; };
__host__ __device__ inline Affine48 compose48(Affine48 f, Affine48 g) {  // f after g
  const unsigned long long M = 0xFFFFFFFFFFFFULL;
  return Affine48{(f.a * g.a) & M, (f.a * g.c + f.c) & M};
}
__host__ __device__ inline Affine48 power48(unsigned long long e) {
  Affine48 r{1, 0}, b{0x5DEECE66DULL, 0xBULL};
  while (e) {
    if (e & 1) r = compose48(b, r);
    b = compose48(b, b);
    e >>= 1;
  }
  return r;
}
__global__ void k_rand(int *__restrict__ d, const int *__restrict__ s, long n,
                       unsigned long long x0) {
  const long stride = (long)gridDim.x * EBLOCK;
  for (long i = (long)blockIdx.x * EBLOCK + threadIdx.x; i < n; i += stride) {
    Affine48 f = power48((unsigned long long)i + 1);
    unsigned long long x = (f.a * x0 + f.c) & 0xFFFFFFFFFFFFULL;
    int r = (int)(x >> 17);
    d[i] = r % __ldg(s + i);
  }
}

// The element functions (f_<op>_<type>) live in elt_ops.cuh, shared with
// generated fused kernels so that both compute exactly the same thing.

template <class F, class TO, class TI>
void map1(vec_p d, vec_p s, int len, const char *name) {
  ensure_init();
  if (len <= 0) return;
  k_map1<F, TO, TI><<<ew_grid(len), EBLOCK, 0, stream()>>>((TO *)d, (const TI *)s, len);
  launch_check(name);
}
template <class F, class TO, class TI>
void map2(vec_p d, vec_p s1, vec_p s2, int len, const char *name) {
  ensure_init();
  if (len <= 0) return;
  k_map2<F, TO, TI><<<ew_grid(len), EBLOCK, 0, stream()>>>((TO *)d, (const TI *)s1, (const TI *)s2, len);
  launch_check(name);
}

}  // namespace gcvl

using namespace gcvl;

#define EW_META(NAME, INPL)                                                   \
  GCVL_EXPORT int NAME##_scratch(int len) { (void)len; return 0; }           \
  GCVL_EXPORT unsigned NAME##_inplace(void) { return INPL; }
#define EW2X(NAME, F, TO, TI)                                                  \
  GCVL_EXPORT void NAME(vec_p d, vec_p s1, vec_p s2, int len, vec_p scratch) { \
    (void)scratch; map2<F, TO, TI>(d, s1, s2, len, #NAME);                     \
  }                                                                            \
  EW_META(NAME, INPLACE_1 | INPLACE_2)
#define EW1X(NAME, F, TO, TI)                                                  \
  GCVL_EXPORT void NAME(vec_p d, vec_p s, int len, vec_p scratch) {            \
    (void)scratch; map1<F, TO, TI>(d, s, len, #NAME);                          \
  }                                                                            \
  EW_META(NAME, INPLACE_1)

EW2X(max_wuz, f_max_z, int, int)
EW2X(max_wud, f_max_d, double, double)
EW2X(min_wuz, f_min_z, int, int)
EW2X(min_wud, f_min_d, double, double)
EW2X(add_wuz, f_add_z, int, int)
EW2X(add_wud, f_add_d, double, double)
EW2X(sub_wuz, f_sub_z, int, int)
EW2X(sub_wud, f_sub_d, double, double)
EW2X(mul_wuz, f_mul_z, int, int)
EW2X(mul_wud, f_mul_d, double, double)
EW2X(div_wuz, f_div_z, int, int)
EW2X(div_wud, f_div_d, double, double)
EW2X(grt_wuz, f_grt_z, int, int)
EW2X(grt_wud, f_grt_d, int, double)
EW2X(les_wuz, f_les_z, int, int)
EW2X(les_wud, f_les_d, int, double)
EW2X(geq_wuz, f_geq_z, int, int)
EW2X(geq_wud, f_geq_d, int, double)
EW2X(leq_wuz, f_leq_z, int, int)
EW2X(leq_wud, f_leq_d, int, double)
EW2X(lsh_wuz, f_lsh_z, int, int)
EW2X(rsh_wuz, f_rsh_z, int, int)
EW2X(mod_wuz, f_mod_z, int, int)
EW2X(eql_wub, f_eql_z, int, int)
EW2X(eql_wuz, f_eql_z, int, int)
EW2X(eql_wud, f_eql_d, int, double)
EW2X(neq_wub, f_neq_z, int, int)
EW2X(neq_wuz, f_neq_z, int, int)
EW2X(neq_wud, f_neq_d, int, double)
EW2X(xor_wub, f_xor_b, int, int)
EW2X(ior_wub, f_ior_b, int, int)
EW2X(and_wub, f_and_b, int, int)
EW2X(ior_wuz, f_ior_z, int, int)
EW2X(and_wuz, f_and_z, int, int)
EW2X(xor_wuz, f_xor_z, int, int)
EW1X(not_wub, f_not_b, int, int)
EW1X(not_wuz, f_not_z, int, int)
EW1X(int_wud, f_int_d, int, double)
EW1X(int_wub, f_int_b, int, int)
EW1X(dbl_wuz, f_dbl_z, double, int)
EW1X(boo_wuz, f_boo_z, int, int)
EW1X(flr_wud, f_flr_d, int, double)
EW1X(cei_wud, f_cei_d, int, double)
EW1X(trn_wud, f_trn_d, int, double)
EW1X(rou_wud, f_rou_d, int, double)
EW1X(exp_wud, f_exp_d, double, double)
EW1X(log_wud, f_log_d, double, double)
EW1X(sqt_wud, f_sqt_d, double, double)
EW1X(sin_wud, f_sin_d, double, double)
EW1X(cos_wud, f_cos_d, double, double)
EW1X(tan_wud, f_tan_d, double, double)
EW1X(asn_wud, f_asn_d, double, double)
EW1X(acs_wud, f_acs_d, double, double)
EW1X(atn_wud, f_atn_d, double, double)
EW1X(snh_wud, f_snh_d, double, double)
EW1X(csh_wud, f_csh_d, double, double)
EW1X(tnh_wud, f_tnh_d, double, double)

// Copies are device-to-device memcpys (elwise.c:278-298).
#define CPYX(NAME, T)                                                         \
  GCVL_EXPORT void NAME(vec_p d, vec_p s, int len, vec_p scratch) {           \
    (void)scratch; ensure_init();                                             \
    if (len <= 0 || d == s) return;                                           \
    GCVL_CK(cudaMemcpyAsync(d, s, (size_t)len * sizeof(T),                    \
                            cudaMemcpyDeviceToDevice, stream()));             \
  }                                                                           \
  EW_META(NAME, INPLACE_1)
CPYX(cpy_wuz, int)
CPYX(cpy_wub, cvl_bool)
CPYX(cpy_wud, double)

// cpy_wus copies a whole segment descriptor (elwise.c:286-298 copies the m
// lengths, which is the whole serial descriptor).
GCVL_EXPORT void cpy_wus(vec_p d, vec_p s, int n, int m, vec_p scratch) {
  (void)scratch; ensure_init();
  if (d == s) return;
  GCVL_CK(cudaMemcpyAsync(d, s, (size_t)siz_fos(n, m) * 8, cudaMemcpyDeviceToDevice, stream()));
}
GCVL_EXPORT int cpy_wus_scratch(int n, int m) { (void)n; (void)m; return 0; }
GCVL_EXPORT unsigned cpy_wus_inplace(void) { return INPLACE_1; }

#define SELX(NAME, T)                                                                   \
  GCVL_EXPORT void NAME(vec_p d, vec_p s1, vec_p s2, vec_p s3, int len, vec_p scratch) { \
    (void)scratch; ensure_init();                                                       \
    if (len <= 0) return;                                                               \
    k_select<T><<<ew_grid(len), EBLOCK, 0, stream()>>>((T *)d, (const int *)s1,         \
                                                      (const T *)s2, (const T *)s3, len); \
    launch_check(#NAME);                                                                \
  }                                                                                     \
  EW_META(NAME, INPLACE_1 | INPLACE_2 | INPLACE_3)
SELX(sel_wuz, int)
SELX(sel_wub, cvl_bool)
SELX(sel_wud, double)

GCVL_EXPORT void rnd_wuz(vec_p d, vec_p s, int len, vec_p scratch) {
  (void)scratch; ensure_init();
  if (len <= 0) return;
  State &S = st();
  k_rand<<<ew_grid(len), EBLOCK, 0, S.stream>>>((int *)d, (const int *)s, len, S.rand48);
  launch_check("rnd_wuz");
  Affine48 f = power48((unsigned long long)len);
  S.rand48 = (f.a * S.rand48 + f.c) & 0xFFFFFFFFFFFFULL;
}
EW_META(rnd_wuz, INPLACE_1)

// Distribute (vprims.c:297-344, unsegmented part).
#define DISX(L, T)                                                                 \
  GCVL_EXPORT void dis_vu##L(vec_p d, T v, int len, vec_p scratch) {               \
    (void)scratch; ensure_init();                                                  \
    if (len <= 0) return;                                                          \
    k_fillv<T><<<ew_grid(len), EBLOCK, 0, stream()>>>((T *)d, v, len);             \
    launch_check("dis_vu" #L);                                                     \
  }                                                                                \
  EW_META(dis_vu##L, INPLACE_NONE)
DISX(z, int)
DISX(d, double)
GCVL_EXPORT void dis_vub(vec_p d, cvl_bool v, int len, vec_p scratch) {
  (void)scratch; ensure_init();
  if (len <= 0) return;
  k_fillv<int><<<ew_grid(len), EBLOCK, 0, stream()>>>((int *)d, v, len);
  launch_check("dis_vub");
}
EW_META(dis_vub, INPLACE_NONE)

// Index (library.c:12-49, unsegmented part): d[i] = init + i*stride with
// the serial CVL's wrapping int arithmetic.
__global__ void k_iota(int *__restrict__ d, int init, int stride, long n) {
  const long step = (long)gridDim.x * EBLOCK;
  for (long i = (long)blockIdx.x * EBLOCK + threadIdx.x; i < n; i += step)
    d[i] = (int)((unsigned)init + (unsigned)stride * (unsigned)i);
}
GCVL_EXPORT void ind_luz(vec_p d, int init, int stride, int count, vec_p scratch) {
  (void)scratch; ensure_init();
  if (count <= 0) return;
  k_iota<<<ew_grid(count), EBLOCK, 0, stream()>>>((int *)d, init, stride, count);
  launch_check("ind_luz");
}
EW_META(ind_luz, INPLACE_NONE)
