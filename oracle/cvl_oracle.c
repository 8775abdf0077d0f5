/*
 * cvl_oracle.c -- CPU oracle for the CVL primitive path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is a plain-C restatement of the
 * semantics of the reference's serial CVL (nesl/cvl/serial/*.c of
 * Nessie-Compiler/neslgpu).  It is the checker for the GPU library: only the
 * tests, __graft_entry__.smoke() and bench.py's CPU-baseline leg load it.
 * Nothing in the product library links it or calls it.
 *
 * Every exported function is named ocvl_<cvl name> and has the C signature of
 * the cvl.h prototype it restates (vec_p = host pointer, sizes in 8-byte
 * CVL_SIZE_UNITs).  Loops run in the same order as the serial CVL so that
 * float64 scans and reductions produce bit-identical sums; this is pinned by
 * comparing against the serial CVL compiled from the reference sources
 * (oracle/Makefile target `ref`) and against the golden fixtures under
 * tests/golden/.
 *
 * Integer arithmetic that may wrap (+, *, -) is done in unsigned 32-bit so
 * that wrapping is defined; the bits equal what the serial CVL computes with
 * gcc on x86-64 and aarch64.
 */
#include <limits.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

typedef void *vec_p;
typedef int cvl_bool;

#define EXPORT __attribute__((visibility("default")))
#define UNIT 8 /* sizeof(MAXALIGN) in the serial CVL, facilt.c:92-93 */

/* Identities: nesl/cvl/serial/defins.h:217-228. The double min/max
 * "infinities" are 1e36 rounded to float and widened back. */
static const double kMaxDouble = (double)(float)1.0e36;
static const double kMinDouble = (double)(float)-1.0e36;

/* ---- binary operators (defins.h:58-115) -------------------------------- */
static inline int op_add_z(int a, int b) { return (int)((uint32_t)a + (uint32_t)b); }
static inline int op_sub_z(int a, int b) { return (int)((uint32_t)a - (uint32_t)b); }
static inline int op_mul_z(int a, int b) { return (int)((uint32_t)a * (uint32_t)b); }
static inline double op_add_d(double a, double b) { return a + b; }
static inline double op_sub_d(double a, double b) { return a - b; }
static inline double op_mul_d(double a, double b) { return a * b; }
/* max(i,j) ((i) > (j) ? (i) : (j)); ties pick the right operand. */
static inline int op_max_z(int a, int b) { return a > b ? a : b; }
static inline int op_min_z(int a, int b) { return a < b ? a : b; }
static inline double op_max_d(double a, double b) { return a > b ? a : b; }
static inline double op_min_d(double a, double b) { return a < b ? a : b; }
static inline int op_land(int a, int b) { return a && b; }
static inline int op_lor(int a, int b) { return a || b; }
static inline int op_lxor(int a, int b) { return (!!a) ^ (!!b); }
static inline int op_band(int a, int b) { return a & b; }
static inline int op_bor(int a, int b) { return a | b; }
static inline int op_bxor(int a, int b) { return a ^ b; }

/* ========================= elementwise (elwise.c:192-298) ================ */
#define EW2(NAME, TI, TO, EXPR)                                                  \
  EXPORT void ocvl_##NAME(vec_p d, vec_p s1, vec_p s2, int len, vec_p scr) {     \
    TO *o = (TO *)d; const TI *a = (const TI *)s1; const TI *b = (const TI *)s2; \
    (void)scr;                                                                   \
    for (int i = 0; i < len; i++) { TI x = a[i], y = b[i]; o[i] = (TO)(EXPR); }  \
  }
#define EW1(NAME, TI, TO, EXPR)                                              \
  EXPORT void ocvl_##NAME(vec_p d, vec_p s, int len, vec_p scr) {            \
    TO *o = (TO *)d; const TI *a = (const TI *)s; (void)scr;                 \
    for (int i = 0; i < len; i++) { TI x = a[i]; o[i] = (TO)(EXPR); }        \
  }

EW2(max_wuz, int, int, op_max_z(x, y))
EW2(max_wud, double, double, op_max_d(x, y))
EW2(min_wuz, int, int, op_min_z(x, y))
EW2(min_wud, double, double, op_min_d(x, y))
EW2(add_wuz, int, int, op_add_z(x, y))
EW2(add_wud, double, double, x + y)
EW2(sub_wuz, int, int, op_sub_z(x, y))
EW2(sub_wud, double, double, x - y)
EW2(mul_wuz, int, int, op_mul_z(x, y))
EW2(mul_wud, double, double, x * y)
/* C division truncates toward zero; zero divisors are undefined in C and
 * are never passed by the tests. */
EW2(div_wuz, int, int, x / y)
EW2(div_wud, double, double, x / y)
EW2(grt_wuz, int, cvl_bool, x > y)
EW2(grt_wud, double, cvl_bool, x > y)
EW2(les_wuz, int, cvl_bool, x < y)
EW2(les_wud, double, cvl_bool, x < y)
EW2(geq_wuz, int, cvl_bool, x >= y)
EW2(geq_wud, double, cvl_bool, x >= y)
EW2(leq_wuz, int, cvl_bool, x <= y)
EW2(leq_wud, double, cvl_bool, x <= y)
/* Shift counts: x86-64 and aarch64 both take the count modulo 32 for a
 * variable 32-bit shift, which is what the serial CVL computes there. */
EW2(lsh_wuz, int, int, (int)((uint32_t)x << (y & 31)))
EW2(rsh_wuz, int, int, x >> (y & 31))
EW2(mod_wuz, int, int, x % y)
EW2(eql_wub, cvl_bool, cvl_bool, x == y)
EW2(eql_wuz, int, cvl_bool, x == y)
EW2(eql_wud, double, cvl_bool, x == y)
EW2(neq_wub, cvl_bool, cvl_bool, x != y)
EW2(neq_wuz, int, cvl_bool, x != y)
EW2(neq_wud, double, cvl_bool, x != y)
EW2(xor_wub, cvl_bool, cvl_bool, x ^ y)
EW2(ior_wub, cvl_bool, cvl_bool, x || y)
EW2(and_wub, cvl_bool, cvl_bool, x && y)
EW2(ior_wuz, int, int, x | y)
EW2(and_wuz, int, int, x & y)
EW2(xor_wuz, int, int, x ^ y)
EW1(not_wub, cvl_bool, cvl_bool, !x)
EW1(not_wuz, int, int, ~x)
EW1(int_wud, double, int, (int)x)
EW1(int_wub, cvl_bool, int, (int)x)
EW1(dbl_wuz, int, double, (double)x)
EW1(boo_wuz, int, cvl_bool, !!x)
EW1(flr_wud, double, int, (int)floor(x))
EW1(cei_wud, double, int, (int)ceil(x))
EW1(trn_wud, double, int, (int)x)
EW1(rou_wud, double, int, (int)(x + 0.5))
EW1(exp_wud, double, double, exp(x))
EW1(log_wud, double, double, log(x))
EW1(sqt_wud, double, double, sqrt(x))
EW1(sin_wud, double, double, sin(x))
EW1(cos_wud, double, double, cos(x))
EW1(tan_wud, double, double, tan(x))
EW1(asn_wud, double, double, asin(x))
EW1(acs_wud, double, double, acos(x))
EW1(atn_wud, double, double, atan(x))
EW1(snh_wud, double, double, sinh(x))
EW1(csh_wud, double, double, cosh(x))
EW1(tnh_wud, double, double, tanh(x))
EW1(cpy_wuz, int, int, x)
EW1(cpy_wub, cvl_bool, cvl_bool, x)
EW1(cpy_wud, double, double, x)

#define SEL(NAME, T)                                                             \
  EXPORT void ocvl_##NAME(vec_p d, vec_p f, vec_p s2, vec_p s3, int len,         \
                          vec_p scr) {                                           \
    T *o = (T *)d; const cvl_bool *c = (const cvl_bool *)f;                      \
    const T *a = (const T *)s2; const T *b = (const T *)s3; (void)scr;           \
    for (int i = 0; i < len; i++) o[i] = c[i] ? a[i] : b[i];                     \
  }
SEL(sel_wuz, int)
SEL(sel_wub, cvl_bool)
SEL(sel_wud, double)

/* cpy_wus copies the m lengths of a segment descriptor (elwise.c:286-298). */
EXPORT void ocvl_cpy_wus(vec_p d, vec_p s, int n, int m, vec_p scr) {
  (void)n; (void)scr; memmove(d, s, (size_t)m * sizeof(int));
}

/* ---- RAND: rnd_wuz (elwise.c:211-236) draws (int)lrand48() % s[i] in
 * order.  The oracle keeps its own 48-bit lrand48 state so that runs do not
 * depend on libc state; rnd_foz seeds it as srand48(seed) does.  Before any
 * seeding the state is 0: glibc's lrand48, which the serial CVL calls on
 * Linux, starts there (POSIX leaves the unseeded state to the C library). */
static uint64_t g_rand48 = 0;
EXPORT void ocvl_rnd_foz(int seed) {
  g_rand48 = (((uint64_t)(uint32_t)seed) << 16 | 0x330EULL) & 0xFFFFFFFFFFFFULL;
}
static inline int next_lrand48(void) {
  g_rand48 = (0x5DEECE66DULL * g_rand48 + 0xBULL) & 0xFFFFFFFFFFFFULL;
  return (int)(g_rand48 >> 17);
}
EXPORT void ocvl_rnd_wuz(vec_p d, vec_p s, int len, vec_p scr) {
  int *o = (int *)d; const int *a = (const int *)s; (void)scr;
  for (int i = 0; i < len; i++) o[i] = next_lrand48() % a[i];
}
EXPORT void ocvl_rnd_state(uint64_t *get, const uint64_t *set) {
  if (get) *get = g_rand48;
  if (set) g_rand48 = *set & 0xFFFFFFFFFFFFULL;
}

/* ============================ scans (vprims.c:17-109) ==================== */
/* Exclusive scan: out[k] = init (op) s[seg_start] (op) ... s[k-1], folded
 * left to right starting from init, restarting at every segment. */
#define SCAN(OPN, L, T, OP, INIT)                                                \
  EXPORT void ocvl_##OPN##_su##L(vec_p d, vec_p s, int len, vec_p scr) {         \
    T *o = (T *)d; const T *a = (const T *)s; T acc = (INIT); (void)scr;         \
    for (int i = 0; i < len; i++) { T x = a[i]; o[i] = acc; acc = OP(acc, x); }  \
  }                                                                              \
  EXPORT void ocvl_##OPN##_se##L(vec_p d, vec_p s, vec_p sd, int n, int m,       \
                                 vec_p scr) {                                    \
    T *o = (T *)d; const T *a = (const T *)s; const int *ln = (const int *)sd;   \
    int k = 0; (void)n; (void)scr;                                               \
    for (int g = 0; g < m; g++) {                                                \
      T acc = (INIT);                                                            \
      for (int e = k + ln[g]; k < e; k++) { T x = a[k]; o[k] = acc; acc = OP(acc, x); } \
    }                                                                            \
  }

SCAN(add, z, int, op_add_z, 0)
SCAN(add, d, double, op_add_d, 0.0)
SCAN(mul, z, int, op_mul_z, 1)
SCAN(mul, d, double, op_mul_d, 1.0)
SCAN(min, z, int, op_min_z, INT_MAX)
SCAN(min, d, double, op_min_d, kMaxDouble)
SCAN(max, z, int, op_max_z, INT_MIN)
SCAN(max, d, double, op_max_d, kMinDouble)
SCAN(and, b, cvl_bool, op_land, 1)
SCAN(and, z, int, op_band, ~0)
SCAN(ior, b, cvl_bool, op_lor, 0)
SCAN(ior, z, int, op_bor, 0)
SCAN(xor, b, cvl_bool, op_lxor, 0)
SCAN(xor, z, int, op_bxor, 0)

/* ============================ reduces (vprims.c:114-201) ================= */
#define RED(OPN, L, T, OP, INIT)                                                 \
  EXPORT T ocvl_##OPN##_ru##L(vec_p s, int len, vec_p scr) {                     \
    const T *a = (const T *)s; T acc = (INIT); (void)scr;                        \
    for (int i = 0; i < len; i++) acc = OP(acc, a[i]);                           \
    return acc;                                                                  \
  }                                                                              \
  EXPORT void ocvl_##OPN##_re##L(vec_p d, vec_p s, vec_p sd, int n, int m,       \
                                 vec_p scr) {                                    \
    T *o = (T *)d; const T *a = (const T *)s; const int *ln = (const int *)sd;   \
    int k = 0; (void)n; (void)scr;                                               \
    for (int g = 0; g < m; g++) {                                                \
      T acc = (INIT);                                                            \
      for (int e = k + ln[g]; k < e; k++) acc = OP(acc, a[k]);                   \
      o[g] = acc;                                                                \
    }                                                                            \
  }

RED(add, z, int, op_add_z, 0)
RED(add, d, double, op_add_d, 0.0)
RED(mul, z, int, op_mul_z, 1)
RED(mul, d, double, op_mul_d, 1.0)
RED(min, z, int, op_min_z, INT_MAX)
RED(min, d, double, op_min_d, kMaxDouble)
RED(max, z, int, op_max_z, INT_MIN)
RED(max, d, double, op_max_d, kMinDouble)
RED(and, b, cvl_bool, op_land, 1)
RED(and, z, int, op_band, ~0)
RED(ior, b, cvl_bool, op_lor, 0)
RED(ior, z, int, op_bor, 0)
RED(xor, b, cvl_bool, op_lxor, 0)
RED(xor, z, int, op_bxor, 0)

/* ============== extract / replace / distribute (vprims.c:207-344) ======== */
#define EXT(L, T)                                                                \
  EXPORT T ocvl_ext_vu##L(vec_p v, int i, int len, vec_p scr) {                  \
    (void)len; (void)scr; return ((const T *)v)[i];                              \
  }                                                                              \
  EXPORT void ocvl_ext_ve##L(vec_p d, vec_p s, vec_p idx, vec_p sd, int n,       \
                             int m, vec_p scr) {                                 \
    T *o = (T *)d; const T *a = (const T *)s; const int *ix = (const int *)idx;  \
    const int *ln = (const int *)sd; long base = 0; (void)n; (void)scr;          \
    for (int g = 0; g < m; g++) { o[g] = a[base + ix[g]]; base += ln[g]; }       \
  }
EXT(z, int)
EXT(b, cvl_bool)
EXT(d, double)

EXPORT void ocvl_rep_vuz(vec_p v, int i, int val, int len, vec_p scr) {
  (void)len; (void)scr; ((int *)v)[i] = val;
}
EXPORT void ocvl_rep_vub(vec_p v, int i, cvl_bool val, int len, vec_p scr) {
  (void)len; (void)scr; ((cvl_bool *)v)[i] = !!val;
}
EXPORT void ocvl_rep_vud(vec_p v, int i, double val, int len, vec_p scr) {
  (void)len; (void)scr; ((double *)v)[i] = val;
}
#define REPSEG(L, T)                                                             \
  EXPORT void ocvl_rep_ve##L(vec_p d, vec_p idx, vec_p val, vec_p sd, int n,     \
                             int m, vec_p scr) {                                 \
    T *o = (T *)d; const int *ix = (const int *)idx; const T *v = (const T *)val;\
    const int *ln = (const int *)sd; long base = 0; (void)n; (void)scr;          \
    for (int g = 0; g < m; g++) { o[base + ix[g]] = v[g]; base += ln[g]; }       \
  }
REPSEG(z, int)
REPSEG(b, cvl_bool)
REPSEG(d, double)

#define DIS(L, T)                                                                \
  EXPORT void ocvl_dis_vu##L(vec_p d, T v, int len, vec_p scr) {                 \
    T *o = (T *)d; (void)scr; for (int i = 0; i < len; i++) o[i] = v;            \
  }                                                                              \
  EXPORT void ocvl_dis_ve##L(vec_p d, vec_p v, vec_p sd, int n, int m,           \
                             vec_p scr) {                                        \
    T *o = (T *)d; const T *val = (const T *)v; const int *ln = (const int *)sd; \
    int k = 0; (void)n; (void)scr;                                               \
    for (int g = 0; g < m; g++) for (int e = k + ln[g]; k < e; k++) o[k] = val[g];\
  }
DIS(z, int)
DIS(b, cvl_bool)
DIS(d, double)

/* ===================== permutes (vprims.c:356-467) ====================== */
#define PERM(L, T)                                                               \
  EXPORT void ocvl_smp_pu##L(vec_p d, vec_p s, vec_p idx, int len, vec_p scr) {  \
    T *o = (T *)d; const T *a = (const T *)s; const int *ix = (const int *)idx;  \
    (void)scr; for (int k = 0; k < len; k++) o[ix[k]] = a[k];                    \
  }                                                                              \
  EXPORT void ocvl_smp_pe##L(vec_p d, vec_p s, vec_p idx, vec_p sd, int n,       \
                             int m, vec_p scr) {                                 \
    T *o = (T *)d; const T *a = (const T *)s; const int *ix = (const int *)idx;  \
    const int *ln = (const int *)sd; int k = 0; (void)n; (void)scr;              \
    for (int g = 0; g < m; g++) {                                                \
      int base = k;                                                              \
      for (int e = k + ln[g]; k < e; k++) o[base + ix[k]] = a[k];                \
    }                                                                            \
  }                                                                              \
  EXPORT void ocvl_bck_pu##L(vec_p d, vec_p s, vec_p idx, int s_len, int d_len,  \
                             vec_p scr) {                                        \
    T *o = (T *)d; const T *a = (const T *)s; const int *ix = (const int *)idx;  \
    (void)s_len; (void)scr; for (int k = 0; k < d_len; k++) o[k] = a[ix[k]];     \
  }                                                                              \
  EXPORT void ocvl_bck_pe##L(vec_p d, vec_p s, vec_p idx, vec_p sd_s, int n_s,   \
                             int m_s, vec_p sd_d, int n_d, int m_d, vec_p scr) { \
    T *o = (T *)d; const T *a = (const T *)s; const int *ix = (const int *)idx;  \
    const int *ls = (const int *)sd_s; const int *ld = (const int *)sd_d;        \
    long sbase = 0; int k = 0; (void)m_s; (void)scr;                             \
    if (m_s == 1) { ocvl_bck_pu##L(d, s, idx, n_s, n_d, scr); return; }          \
    for (int g = 0; g < m_d; g++) {                                              \
      for (int e = k + ld[g]; k < e; k++) o[k] = a[sbase + ix[k]];               \
      sbase += ls[g];                                                            \
    }                                                                            \
  }
PERM(z, int)
PERM(b, cvl_bool)
PERM(d, double)

/* ====================== flag permutes (vecops.c:22-286) ================= */
#define FPERM(L, T)                                                              \
  EXPORT void ocvl_fpm_pu##L(vec_p d, vec_p s, vec_p idx, vec_p f, int len_src,  \
                             int len_dest, vec_p scr) {                          \
    T *o = (T *)d; const T *a = (const T *)s; const int *ix = (const int *)idx;  \
    const cvl_bool *fl = (const cvl_bool *)f; (void)len_dest; (void)scr;         \
    for (int k = 0; k < len_src; k++) if (fl[k]) o[ix[k]] = a[k];                \
  }                                                                              \
  EXPORT void ocvl_fpm_pe##L(vec_p d, vec_p s, vec_p idx, vec_p f, vec_p sd_s,   \
                             int n_s, int m_s, vec_p sd_d, int n_d, int m_d,     \
                             vec_p scr) {                                        \
    T *o = (T *)d; const T *a = (const T *)s; const int *ix = (const int *)idx;  \
    const cvl_bool *fl = (const cvl_bool *)f; const int *ls = (const int *)sd_s; \
    const int *ld = (const int *)sd_d; long dbase = 0; int k = 0;                \
    (void)n_s; (void)n_d; (void)m_d; (void)scr;                                  \
    for (int g = 0; g < m_s; g++) {                                              \
      for (int e = k + ls[g]; k < e; k++) if (fl[k]) o[dbase + ix[k]] = a[k];    \
      dbase += ld[g];                                                            \
    }                                                                            \
  }                                                                              \
  EXPORT void ocvl_bfp_pu##L(vec_p d, vec_p s, vec_p idx, vec_p f, int len_src,  \
                             int len_dest, vec_p scr) {                          \
    T *o = (T *)d; const T *a = (const T *)s; const int *ix = (const int *)idx;  \
    const cvl_bool *fl = (const cvl_bool *)f; (void)len_src; (void)scr;         \
    for (int k = 0; k < len_dest; k++) o[k] = fl[k] ? a[ix[k]] : (T)0;          \
  }                                                                              \
  EXPORT void ocvl_bfp_pe##L(vec_p d, vec_p s, vec_p idx, vec_p f, vec_p sd_s,   \
                             int n_s, int m_s, vec_p sd_d, int n_d, int m_d,     \
                             vec_p scr) {                                        \
    T *o = (T *)d; const T *a = (const T *)s; const int *ix = (const int *)idx;  \
    const cvl_bool *fl = (const cvl_bool *)f; const int *ls = (const int *)sd_s; \
    const int *ld = (const int *)sd_d; long sbase = 0; int k = 0;                \
    (void)m_d; (void)scr;                                                        \
    if (m_s == 1) { ocvl_bfp_pu##L(d, s, idx, f, n_s, n_d, scr); return; }       \
    memset(d, 0, (size_t)n_d * sizeof(T));                                       \
    for (int g = 0; g < m_s; g++) {                                              \
      for (int e = k + ld[g]; k < e; k++) if (fl[k]) o[k] = a[sbase + ix[k]];    \
      sbase += ls[g];                                                            \
    }                                                                            \
  }                                                                              \
  EXPORT void ocvl_dpe_pu##L(vec_p d, vec_p s, vec_p idx, vec_p v, int len_src,  \
                             int len_dest, vec_p scr) {                          \
    if (d != v) memmove(d, v, (size_t)len_dest * sizeof(T));                     \
    ocvl_smp_pu##L(d, s, idx, len_src, scr);                                     \
  }                                                                              \
  EXPORT void ocvl_dpe_pe##L(vec_p d, vec_p s, vec_p idx, vec_p v, vec_p sd_s,   \
                             int n_s, int m_s, vec_p sd_d, int n_d, int m_d,     \
                             vec_p scr) {                                        \
    T *o = (T *)d; const T *a = (const T *)s; const int *ix = (const int *)idx;  \
    const int *ls = (const int *)sd_s; const int *ld = (const int *)sd_d;        \
    long dbase = 0; int k = 0; (void)m_d;                                        \
    if (m_s == 1) { ocvl_dpe_pu##L(d, s, idx, v, n_s, n_d, scr); return; }       \
    if (d != v) memmove(d, v, (size_t)n_d * sizeof(T));                          \
    for (int g = 0; g < m_s; g++) {                                              \
      for (int e = k + ls[g]; k < e; k++) o[dbase + ix[k]] = a[k];               \
      dbase += ld[g];                                                            \
    }                                                                            \
  }                                                                              \
  EXPORT void ocvl_dfp_pu##L(vec_p d, vec_p s, vec_p idx, vec_p f, vec_p v,      \
                             int len_src, int len_dest, vec_p scr) {             \
    if (d != v) memmove(d, v, (size_t)len_dest * sizeof(T));                     \
    ocvl_fpm_pu##L(d, s, idx, f, len_src, len_dest, scr);                        \
  }                                                                              \
  EXPORT void ocvl_dfp_pe##L(vec_p d, vec_p s, vec_p idx, vec_p f, vec_p v,      \
                             vec_p sd_s, int n_s, int m_s, vec_p sd_d, int n_d,  \
                             int m_d, vec_p scr) {                               \
    if (d != v) memmove(d, v, (size_t)n_d * sizeof(T));                          \
    if (m_s == 1) ocvl_fpm_pu##L(d, s, idx, f, n_s, n_d, scr);                   \
    else ocvl_fpm_pe##L(d, s, idx, f, sd_s, n_s, m_s, sd_d, n_d, m_d, scr);      \
  }
FPERM(z, int)
FPERM(b, cvl_bool)
FPERM(d, double)

/* ============================ facilities (facilt.c) ===================== */
EXPORT int ocvl_siz_fob(int n) { return (int)(((size_t)n * sizeof(cvl_bool) + UNIT - 1) / UNIT); }
EXPORT int ocvl_siz_foz(int n) { return (int)(((size_t)n * sizeof(int) + UNIT - 1) / UNIT); }
EXPORT int ocvl_siz_fod(int n) { return (int)(((size_t)n * sizeof(double) + UNIT - 1) / UNIT); }
/* Serial segment descriptor = the m segment lengths (facilt.c:112-144). */
EXPORT int ocvl_siz_fos(int n, int m) { (void)n; return (int)(((size_t)m * sizeof(int) + UNIT - 1) / UNIT); }
EXPORT void ocvl_mke_fov(vec_p sd, vec_p l, int n, int m, vec_p scr) {
  (void)n; (void)scr; if (sd != l) memmove(sd, l, (size_t)m * sizeof(int));
}
EXPORT void ocvl_len_fos(vec_p l, vec_p sd, int n, int m, vec_p scr) {
  (void)n; (void)scr; if (sd != l) memmove(l, sd, (size_t)m * sizeof(int));
}

/* Vector memory and host transfers (facilt.c:149-160, 252-283): malloc'd
 * units of UNIT bytes, and element copies to and from host arrays.  Used by
 * the VCODE interpreter when it runs on the oracle. */
EXPORT vec_p ocvl_alo_foz(int size) { return malloc((size_t)(size > 0 ? size : 1) * UNIT); }
EXPORT void ocvl_fre_fov(vec_p p) { free(p); }
/* mov_fov (facilt.c:160-183): move `size` units that may overlap, one unit
 * at a time, front to back when moving down and back to front when moving
 * up, so every unit is read before it is overwritten. */
EXPORT void ocvl_mov_fov(vec_p d, vec_p s, int size, vec_p scr) {
  uint64_t *dst = (uint64_t *)d;
  const uint64_t *src = (const uint64_t *)s;
  (void)scr;
  if (dst == src) return;
  if (dst < src) {
    for (int i = 0; i < size; i++) dst[i] = src[i];
  } else {
    for (int i = size - 1; i >= 0; i--) dst[i] = src[i];
  }
}
#define XFER(L, T)                                                                      \
  EXPORT void ocvl_v2c_fu##L(void *d, vec_p s, int len, vec_p scr) {                    \
    (void)scr; if (len > 0) memcpy(d, s, (size_t)len * sizeof(T));                      \
  }                                                                                     \
  EXPORT void ocvl_c2v_fu##L(vec_p d, void *s, int len, vec_p scr) {                    \
    (void)scr; if (len > 0) memcpy(d, s, (size_t)len * sizeof(T));                      \
  }
XFER(z, int)
XFER(b, cvl_bool)
XFER(d, double)

/* ============================ library (library.c) ======================= */
EXPORT void ocvl_ind_luz(vec_p d, int init, int stride, int count, vec_p scr) {
  int *o = (int *)d; int cur = init; (void)scr;
  for (int i = 0; i < count; i++) { o[i] = cur; cur = op_add_z(cur, stride); }
}
EXPORT void ocvl_ind_lez(vec_p d, vec_p init, vec_p stride, vec_p sd, int n,
                         int m, vec_p scr) {
  int *o = (int *)d; const int *in = (const int *)init;
  const int *st = (const int *)stride; const int *ln = (const int *)sd;
  int k = 0; (void)n; (void)scr;
  for (int g = 0; g < m; g++) {
    int cur = in[g];
    for (int e = k + ln[g]; k < e; k++) { o[k] = cur; cur = op_add_z(cur, st[g]); }
  }
}
EXPORT int ocvl_pk1_luv(vec_p f, int len, vec_p scr) {
  const cvl_bool *fl = (const cvl_bool *)f; int c = 0; (void)scr;
  for (int i = 0; i < len; i++) if (fl[i]) c++;
  return c;
}
EXPORT void ocvl_pk1_lev(vec_p ds, vec_p f, vec_p sd, int n, int m, vec_p scr) {
  int *o = (int *)ds; const cvl_bool *fl = (const cvl_bool *)f;
  const int *ln = (const int *)sd; int k = 0; (void)n; (void)scr;
  for (int g = 0; g < m; g++) {
    int c = 0;
    for (int e = k + ln[g]; k < e; k++) if (fl[k]) c++;
    o[g] = c;
  }
}
#define PACK(L, T)                                                               \
  EXPORT void ocvl_pk2_lu##L(vec_p d, vec_p s, vec_p f, int src_len,             \
                             int dest_len, vec_p scr) {                          \
    T *o = (T *)d; const T *a = (const T *)s; const cvl_bool *fl = (const cvl_bool *)f; \
    int j = 0; (void)dest_len; (void)scr;                                        \
    for (int k = 0; k < src_len; k++) if (fl[k]) o[j++] = a[k];                  \
  }                                                                              \
  EXPORT void ocvl_pk2_le##L(vec_p d, vec_p s, vec_p f, vec_p sd_s, int n_s,     \
                             int m_s, vec_p sd_d, int n_d, int m_d, vec_p scr) { \
    (void)sd_s; (void)m_s; (void)sd_d; (void)m_d;                                \
    ocvl_pk2_lu##L(d, s, f, n_s, n_d, scr);                                      \
  }
PACK(z, int)
PACK(b, cvl_bool)
PACK(d, double)

/* ============================== rank (rank.c) =========================== */
/* Stable LSD rank with 8-bit digits of one 32-bit field (rank.c:49-73):
 * perm holds the current order and is re-sorted stably by key[perm[i]]. */
static void rank_field(uint32_t *tmp, const uint32_t *key, int *perm, int n) {
  for (int shift = 0; shift < 32; shift += 8) {
    int count[256];
    memset(count, 0, sizeof(count));
    for (int i = 0; i < n; i++) count[(key[perm[i]] >> shift) & 0xFF]++;
    int run = 0;
    for (int b = 0; b < 256; b++) { int c = count[b]; count[b] = run; run += c; }
    for (int i = 0; i < n; i++) tmp[count[(key[perm[i]] >> shift) & 0xFF]++] = (uint32_t)perm[i];
    memcpy(perm, tmp, (size_t)n * sizeof(int));
  }
}

/* Segmented ranks: after the key passes, one more stable pass on the segment
 * number, then rank within the segment (rank.c:118-149). */
static void rank_finish(int *out, int *perm, uint32_t *tmp, const int *ln,
                        int n, int m, int seg) {
  uint32_t *segno = NULL;
  if (seg && m > 1) {
    segno = (uint32_t *)malloc((size_t)n * sizeof(uint32_t) + 1);
    int k = 0;
    for (int g = 0; g < m; g++) for (int e = k + ln[g]; k < e; k++) segno[k] = (uint32_t)g;
    rank_field(tmp, segno, perm, n);
    free(segno);
  }
  for (int i = 0; i < n; i++) out[perm[i]] = i;
  if (seg && m > 1) {
    int k = 0, base = 0;
    for (int g = 0; g < m; g++) {
      for (int e = k + ln[g]; k < e; k++) out[k] -= base;
      base += ln[g];
    }
  }
}

/* Integer keys: up flips the sign bit, down flips every other bit
 * (rank.c:94-99), so ascending unsigned order gives the wanted order. */
static void rank_int(vec_p d, vec_p s, vec_p sd, int n, int m, int seg, int up) {
  uint32_t mask = up ? 0x80000000u : 0x7FFFFFFFu;
  const uint32_t *a = (const uint32_t *)s;
  uint32_t *key = (uint32_t *)malloc((size_t)n * sizeof(uint32_t) + 1);
  uint32_t *tmp = (uint32_t *)malloc((size_t)n * sizeof(uint32_t) + 1);
  int *perm = (int *)malloc((size_t)n * sizeof(int) + 1);
  for (int i = 0; i < n; i++) { key[i] = a[i] ^ mask; perm[i] = i; }
  rank_field(tmp, key, perm, n);
  rank_finish((int *)d, perm, tmp, (const int *)sd, n, m, seg);
  free(key); free(tmp); free(perm);
}

/* Double keys: two 32-bit fields, low word first; negative numbers have all
 * bits flipped, others the sign bit; down ranks complement the field
 * (rank.c:234-280, little-endian word order). */
static void rank_dbl(vec_p d, vec_p s, vec_p sd, int n, int m, int seg, int up) {
  const uint64_t *a = (const uint64_t *)s;
  uint32_t *key = (uint32_t *)malloc((size_t)n * sizeof(uint32_t) + 1);
  uint32_t *tmp = (uint32_t *)malloc((size_t)n * sizeof(uint32_t) + 1);
  int *perm = (int *)malloc((size_t)n * sizeof(int) + 1);
  for (int i = 0; i < n; i++) perm[i] = i;
  for (int w = 0; w < 2; w++) {
    for (int i = 0; i < n; i++) {
      uint64_t bits = a[i];
      uint32_t t = w == 0 ? (uint32_t)bits : (uint32_t)(bits >> 32);
      int neg = (int)(bits >> 63);
      uint32_t f = neg ? ~t : (w == 1 ? t ^ 0x80000000u : t);
      key[i] = up ? f : ~f;
    }
    rank_field(tmp, key, perm, n);
  }
  rank_finish((int *)d, perm, tmp, (const int *)sd, n, m, seg);
  free(key); free(tmp); free(perm);
}

EXPORT void ocvl_rku_luz(vec_p d, vec_p s, int len, vec_p scr) { (void)scr; rank_int(d, s, NULL, len, 1, 0, 1); }
EXPORT void ocvl_rkd_luz(vec_p d, vec_p s, int len, vec_p scr) { (void)scr; rank_int(d, s, NULL, len, 1, 0, 0); }
EXPORT void ocvl_rku_lez(vec_p d, vec_p s, vec_p sd, int n, int m, vec_p scr) { (void)scr; rank_int(d, s, sd, n, m, 1, 1); }
EXPORT void ocvl_rkd_lez(vec_p d, vec_p s, vec_p sd, int n, int m, vec_p scr) { (void)scr; rank_int(d, s, sd, n, m, 1, 0); }
EXPORT void ocvl_rku_lud(vec_p d, vec_p s, int len, vec_p scr) { (void)scr; rank_dbl(d, s, NULL, len, 1, 0, 1); }
EXPORT void ocvl_rkd_lud(vec_p d, vec_p s, int len, vec_p scr) { (void)scr; rank_dbl(d, s, NULL, len, 1, 0, 0); }
EXPORT void ocvl_rku_led(vec_p d, vec_p s, vec_p sd, int n, int m, vec_p scr) { (void)scr; rank_dbl(d, s, sd, n, m, 1, 1); }
EXPORT void ocvl_rkd_led(vec_p d, vec_p s, vec_p sd, int n, int m, vec_p scr) { (void)scr; rank_dbl(d, s, sd, n, m, 1, 0); }

/* ============================ timing helper ============================= */
EXPORT double ocvl_now(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}
