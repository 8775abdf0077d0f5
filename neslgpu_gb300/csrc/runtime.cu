// runtime.cu -- library state, errors and the CVL facility functions
// (memory, transfers, sizes, timers, RAND seed) of libcvl_gb300.so.
//
// Facility semantics follow the serial CVL (nesl/cvl/serial/facilt.c); the
// memory model follows the reference's CUDA CVL in spirit (one device heap
// the caller sub-allocates, nesl/cvl/cuda/facilities.c:196-237) but vec_p is
// a device pointer rather than an int offset.
#include "gcvl.cuh"

#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <time.h>
#include <dlfcn.h>

namespace gcvl {

static State g_state;
State &st() { return g_state; }

void set_error(int code, const char *fmt, ...) {
  State &s = g_state;
  if (s.err != 0) return;  // sticky: keep the first error
  s.err = code;
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(s.msg, sizeof(s.msg), fmt, ap);
  va_end(ap);
  if (getenv("GCVL_VERBOSE")) fprintf(stderr, "gcvl: error %d: %s\n", code, s.msg);
}

bool check_cuda(cudaError_t e, const char *what) {
  if (e == cudaSuccess) return true;
  set_error(GCVL_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
  return false;
}

static unsigned long long g_launches = 0;
void launch_check(const char *what) {
  ++g_launches;
  cudaError_t e = cudaPeekAtLastError();
  if (e != cudaSuccess) {
    cudaGetLastError();
    set_error(GCVL_ERR_CUDA, "launch of %s: %s", what, cudaGetErrorString(e));
  }
}

void ensure_init() {
  State &s = g_state;
  if (s.ready) return;
  const char *dev = getenv("GCVL_DEVICE");
  if (dev) {
    s.device = atoi(dev);
    if (!GCVL_CK(cudaSetDevice(s.device))) return;
  } else {
    if (!GCVL_CK(cudaGetDevice(&s.device))) return;
  }
  if (!GCVL_CK(cudaDeviceGetAttribute(&s.sm_count, cudaDevAttrMultiProcessorCount, s.device))) return;
  if (!s.stream) {
    if (!GCVL_CK(cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking))) return;
    s.own_stream = true;
  }
  if (!GCVL_CK(cudaMalloc(&s.d_small, 4096))) return;
  if (!GCVL_CK(cudaMallocHost(&s.h_small, 4096))) return;
  s.d_status = (unsigned *)s.d_small;  // word 0 of the small buffer
  if (!GCVL_CK(cudaMemset(s.d_small, 0, 4096))) return;
  const char *spin = getenv("GCVL_SPIN_LIMIT");
  if (spin) s.spin_limit = atoi(spin);
  s.ready = true;
}

void *scratch_or_work(vec_p scratch, size_t bytes) {
  if (scratch) return scratch;
  State &s = g_state;
  if (bytes <= s.work_bytes) return s.work;
  if (s.work) {
    cudaStreamSynchronize(s.stream);
    cudaFree(s.work);
    s.work = nullptr;
    s.work_bytes = 0;
  }
  size_t want = align_up(bytes < ((size_t)1 << 20) ? ((size_t)1 << 20) : bytes, (size_t)1 << 20);
  if (!GCVL_CK(cudaMalloc(&s.work, want))) return nullptr;
  s.work_bytes = want;
  return s.work;
}

}  // namespace gcvl

using namespace gcvl;

// ===================================================== library extensions ==
// Error reporting.  The CVL ABI has no error returns (the serial CVL and the
// CUDA CVL abort); this library records the first error and keeps going.
GCVL_EXPORT int gcvl_last_error(void) { return st().err; }
GCVL_EXPORT const char *gcvl_error_string(void) { return st().msg; }
GCVL_EXPORT void gcvl_clear_error(void) { st().err = 0; st().msg[0] = 0; }

// Synchronise the library stream, fold the device status words into the
// error state and return the error code (0 when all is well).
GCVL_EXPORT int gcvl_sync(void) {
  State &s = st();
  if (!s.ready && noalloc_used()) {
    // Only gcvl_add_sed_noalloc has run, on the legacy default stream: wait
    // for it and read its status word without the library's set-up, which
    // allocates.
    if (GCVL_CK(cudaStreamSynchronize(0))) noalloc_fold_status();
    return s.err;
  }
  ensure_init();
  if (!s.ready) return s.err ? s.err : GCVL_ERR_CUDA;
  if (!GCVL_CK(cudaStreamSynchronize(s.stream))) return s.err;
  unsigned word = 0;
  if (!GCVL_CK(cudaMemcpy(&word, s.d_status, 4, cudaMemcpyDeviceToHost))) return s.err;
  if (word & DEV_TIMEOUT) set_error(GCVL_ERR_TIMEOUT, "a bounded device wait gave up (status 0x%x)", word);
  if (word & DEV_RANGE) set_error(GCVL_ERR_RANGE, "a kernel was given input outside its range and skipped it (status 0x%x)", word);
  if (word) {
    unsigned zero = 0;
    cudaMemcpy(s.d_status, &zero, 4, cudaMemcpyHostToDevice);
  }
  noalloc_fold_status();
  return s.err;
}

GCVL_EXPORT void *gcvl_get_stream(void) { ensure_init(); return (void *)st().stream; }
// Run every later call on `stream` (a cudaStream_t); NULL restores the
// library's own stream.
GCVL_EXPORT void gcvl_set_stream(void *stream) {
  ensure_init();
  State &s = st();
  static cudaStream_t own = nullptr;
  if (s.own_stream) own = s.stream;
  if (stream) { s.stream = (cudaStream_t)stream; s.own_stream = false; }
  else if (own) { s.stream = own; s.own_stream = true; }
}
// A new non-blocking stream on the library's device, for gcvl_set_stream
// (copies on one stream overlapping kernels on another); NULL on failure.
GCVL_EXPORT void *gcvl_stream_create(void) {
  ensure_init();
  cudaStream_t q = nullptr;
  if (!GCVL_CK(cudaStreamCreateWithFlags(&q, cudaStreamNonBlocking))) return nullptr;
  return (void *)q;
}
GCVL_EXPORT void gcvl_stream_destroy(void *stream) {
  if (stream) GCVL_CK(cudaStreamDestroy((cudaStream_t)stream));
}
// Number of kernels this library has launched (all entry points).
GCVL_EXPORT unsigned long long gcvl_launch_count(void) { return gcvl::g_launches; }

// Seeded synthetic vectors generated on the device (benchmark inputs):
// element i depends only on (seed, i) through splitmix64.
//   kind 0: int32 uniform over all values      kind 1: float64 N(0,1)
//   kind 2: cvl_bool Bernoulli(p = a)           kind 3: int32 uniform [0, b)
__device__ __forceinline__ unsigned long long splitmix64(unsigned long long x) {
  x += 0x9E3779B97F4A7C15ULL;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ULL;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBULL;
  return x ^ (x >> 31);
}
__global__ void k_fill_random(void *d, long n, int kind, unsigned long long seed, double a, int b) {
  const long stride = (long)gridDim.x * blockDim.x;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    unsigned long long h = splitmix64(seed * 0x632BE59BD9B4E019ULL + (unsigned long long)i);
    if (kind == 0) {
      ((int *)d)[i] = (int)(unsigned)(h >> 32);
    } else if (kind == 1) {
      // Box-Muller on two 53-bit uniforms
      unsigned long long h2 = splitmix64(h);
      double u1 = ((h >> 11) + 1) * 0x1.0p-53, u2 = (h2 >> 11) * 0x1.0p-53;
      ((double *)d)[i] = sqrt(-2.0 * log(u1)) * cospi(2.0 * u2);
    } else if (kind == 2) {
      ((int *)d)[i] = ((h >> 11) * 0x1.0p-53) < a ? 1 : 0;
    } else {
      ((int *)d)[i] = (int)((h >> 32) % (unsigned long long)(b > 0 ? b : 1));
    }
  }
}
GCVL_EXPORT void gcvl_fill_random(vec_p d, long n, int kind, unsigned long long seed, double a, int b) {
  ensure_init();
  if (n <= 0) return;
  long g = (n + 255) / 256, cap = (long)st().sm_count * 32;
  k_fill_random<<<(int)(g < cap ? g : cap), 256, 0, st().stream>>>(d, n, kind, seed, a, b);
  launch_check("k_fill_random");
}

GCVL_EXPORT int gcvl_sm_count(void) { ensure_init(); return st().sm_count; }
GCVL_EXPORT int gcvl_device(void) { ensure_init(); return st().device; }
// Iteration limit of every bounded device wait; a small value makes waits
// give up early (used by the failure-detection tests).
GCVL_EXPORT void gcvl_set_spin_limit(int iters) { st().spin_limit = iters < 1 ? 1 : iters; }
GCVL_EXPORT int gcvl_get_spin_limit(void) { return st().spin_limit; }

// CUDA-event timing on the library stream (for benchmarks).
GCVL_EXPORT void *gcvl_event_create(void) {
  ensure_init();
  cudaEvent_t e = nullptr;
  GCVL_CK(cudaEventCreate(&e));
  return (void *)e;
}
GCVL_EXPORT void gcvl_event_record(void *e) { GCVL_CK(cudaEventRecord((cudaEvent_t)e, st().stream)); }
GCVL_EXPORT float gcvl_event_elapsed_ms(void *a, void *b) {
  float ms = -1.0f;
  GCVL_CK(cudaEventSynchronize((cudaEvent_t)b));
  GCVL_CK(cudaEventElapsedTime(&ms, (cudaEvent_t)a, (cudaEvent_t)b));
  return ms;
}
GCVL_EXPORT void gcvl_event_destroy(void *e) { cudaEventDestroy((cudaEvent_t)e); }
// Later work on the library stream waits for the event's last record (on
// any stream): orders a pipeline whose stages run on different streams.
GCVL_EXPORT void gcvl_stream_wait_event(void *e) {
  ensure_init();
  GCVL_CK(cudaStreamWaitEvent(st().stream, (cudaEvent_t)e, 0));
}

// Pinned host memory for callers that time host<->device transfers.
GCVL_EXPORT void *gcvl_host_alloc(size_t bytes) {
  ensure_init();
  void *p = nullptr;
  if (!GCVL_CK(cudaMallocHost(&p, bytes))) return nullptr;
  return p;
}
GCVL_EXPORT void gcvl_host_free(void *p) { if (p) cudaFreeHost(p); }

// A wait on a flag that nothing sets: returns the status word the kernel
// wrote (DEV_TIMEOUT once the bounded wait gave up).  Exercises the
// failure-detection path without hanging the GPU.
__global__ void k_selftest_wait(const unsigned *flag, unsigned *status, int limit, unsigned *out) {
  int i = 0;
  while (ld_acquire(flag) == 0u) {
    if (++i >= limit) { atomicOr(status, DEV_TIMEOUT); break; }
    __nanosleep(64);
  }
  *out = i;
}
GCVL_EXPORT int gcvl_selftest_timeout(int limit) {
  ensure_init();
  State &s = st();
  unsigned *flag = (unsigned *)s.d_small + 8;
  unsigned *out = (unsigned *)s.d_small + 9;
  GCVL_CK(cudaMemsetAsync(flag, 0, 8, s.stream));
  k_selftest_wait<<<1, 1, 0, s.stream>>>(flag, s.d_status, limit < 1 ? 1 : limit, out);
  launch_check("k_selftest_wait");
  return gcvl_sync();
}

// =================================================== CVL facility functions
// CVL_init (cvl.h:121-123, CUDA build): records the fused super-op library
// named by vinterp's -l flag and brings the device up.  The serial CVL_init
// calls rnd_foz(0) (facilt.c:316-319), which on Linux is srandom(0) and leaves
// lrand48 unseeded: RAND then draws glibc's unseeded stream, from state 0.
GCVL_EXPORT void CVL_init(char *lib) {
  if (lib) {
    strncpy(st().fused_lib, lib, sizeof(st().fused_lib) - 1);
    st().fused_init_done = false;
  }
  ensure_init();
  st().rand48 = 0;
}

// Timers (facilt.c:43-99).  tgt_fos drains the library stream first so that
// VCODE's START_TIMER/STOP_TIMER bracket finished GPU work.
GCVL_EXPORT void tgt_fos(struct timespec *t) {
  if (st().ready) cudaStreamSynchronize(st().stream);
  clock_gettime(CLOCK_REALTIME, t);
}
GCVL_EXPORT double tdf_fos(struct timespec *t1, struct timespec *t2) {
  return (double)(t1->tv_sec - t2->tv_sec) + 1.0e-9 * (double)(t1->tv_nsec - t2->tv_nsec);
}

// Sizes in 8-byte units (facilt.c:101-146), rounded up to an even number
// of units.  vinterp places every vector of its one heap right after the
// previous block, at the sizes these functions return (vstack.c:405-468,
// 603-606); even sizes keep every vector 16-byte aligned, which the TMA
// kernels need (an 8-byte aligned float64 vector takes the generic kernels:
// 2.3x slower for a segmented scan, 4.3x for a segmented reduction).
static inline int units16(size_t bytes) { return (int)(((bytes + 15) / 16) * 2); }
GCVL_EXPORT int siz_fob(int n) { return units16((size_t)n * 4); }
GCVL_EXPORT int siz_foz(int n) { return units16((size_t)n * 4); }
GCVL_EXPORT int siz_fod(int n) { return units16((size_t)n * 8); }
// The device segment descriptor holds lengths, offsets and the granule
// table (layout in gcvl.cuh), so it is larger than the serial m lengths.
GCVL_EXPORT int siz_fos(int n, int m) {
  if (n < 0 || m < 0) return 0;
  return units16(segdes_total_words(n, m) * 4);
}

// Memory (facilt.c:148-234).  alo_foz returns NULL when the device is out
// of memory, as the serial CVL returns NULL from malloc.  The first
// allocation after CVL_init named a fused library passes its base to that
// library's init(), as the reference's CUDA CVL does with its heap
// (nesl/cvl/cuda/facilities.c:206-221); a library that cannot be opened or
// has no init makes that allocation fail, as there.
static bool call_fused_init(void *base) {
  State &s = st();
  void *h = dlopen(s.fused_lib, RTLD_NOW);
  if (!h) { set_error(GCVL_ERR_ARG, "alo_foz: cannot load fused library %s: %s", s.fused_lib, dlerror()); return false; }
  void (*init_fn)(void *) = (void (*)(void *))dlsym(h, "init");
  if (!init_fn) {
    set_error(GCVL_ERR_ARG, "alo_foz: fused library %s has no init", s.fused_lib);
    dlclose(h);
    return false;
  }
  init_fn(base);
  dlclose(h);
  return true;
}
GCVL_EXPORT vec_p alo_foz(int size) {
  ensure_init();
  if (size < 0) { set_error(GCVL_ERR_ARG, "alo_foz: negative size %d", size); return nullptr; }
  void *p = nullptr;
  size_t bytes = (size_t)(size > 0 ? size : 1) * 8;
  cudaError_t e = cudaMalloc(&p, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    set_error(GCVL_ERR_NOMEM, "alo_foz(%d units): %s", size, cudaGetErrorString(e));
    return nullptr;
  }
  State &s = st();
  if (s.fused_lib[0] && !s.fused_init_done) {
    s.fused_init_done = true;
    if (!call_fused_init(p)) {
      cudaFree(p);
      return nullptr;
    }
  }
  return p;
}
GCVL_EXPORT void fre_fov(vec_p p) {
  if (!p) return;
  cudaStreamSynchronize(st().stream);
  GCVL_CK(cudaFree(p));
}

// mov_fov must handle overlapping regions (facilt.c:162-183).  Disjoint
// regions take one device copy.  Overlapping ones take one cooperative
// kernel that moves the region in rounds and allocates nothing: in each
// round every CTA loads its part of the round's source units into
// registers, all CTAs meet at a grid barrier, then store.  Moving down
// (d < s) the rounds run from the front, moving up from the back; a round's
// stores only overwrite source units that this or an earlier round has
// already loaded, and the next round's loads do not touch what it stored,
// so one barrier per round is enough.  The barrier's waits are bounded: a
// round whose barrier gave up stores nothing and the timeout is reported.
constexpr int MV_BLOCK = 256, MV_ITEMS = 16, MV_CHUNK = MV_BLOCK * MV_ITEMS;  // 8-byte units per CTA per round
__device__ __forceinline__ bool grid_meet(unsigned *count, unsigned *gen, unsigned nblocks, unsigned *status,
                                          int limit) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    const unsigned g = *(volatile unsigned *)gen;
    __threadfence();
    if (atomicAdd(count, 1u) == nblocks - 1) {
      *(volatile unsigned *)count = 0;
      __threadfence();
      atomicAdd(gen, 1u);
    } else {
      int it = 0;
      while (*(volatile unsigned *)gen == g) {
        if (++it >= limit) { ok = 0; atomicOr(status, DEV_TIMEOUT); break; }
        __nanosleep(64);
      }
    }
    __threadfence();
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}
__global__ void __launch_bounds__(MV_BLOCK) k_move_overlap(unsigned long long *d, const unsigned long long *s,
                                                           long units, int up, unsigned *bar, unsigned *status,
                                                           int limit) {
  const long per_round = (long)gridDim.x * MV_CHUNK;
  for (long r0 = 0; r0 < units; r0 += per_round) {
    // this round covers [lo, lo + len) of the units, counted from the front
    // (moving down) or from the back (moving up)
    const long len = units - r0 < per_round ? units - r0 : per_round;
    const long lo = up ? units - r0 - len : r0;
    const long mine = lo + (long)blockIdx.x * MV_CHUNK;
    unsigned long long v[MV_ITEMS];
#pragma unroll
    for (int c = 0; c < MV_ITEMS; c++) {
      const long k = mine + c * MV_BLOCK + threadIdx.x;
      if (k < lo + len) v[c] = s[k];
    }
    if (!grid_meet(bar, bar + 1, gridDim.x, status, limit)) return;
#pragma unroll
    for (int c = 0; c < MV_ITEMS; c++) {
      const long k = mine + c * MV_BLOCK + threadIdx.x;
      if (k < lo + len) d[k] = v[c];
    }
  }
}

GCVL_EXPORT void mov_fov(vec_p d, vec_p s, int size, vec_p scratch) {
  (void)scratch;
  ensure_init();
  if (d == s || size <= 0) return;
  State &S = st();
  char *dst = (char *)d, *src = (char *)s;
  size_t bytes = (size_t)size * 8;
  bool overlap = dst < src + bytes && src < dst + bytes;
  if (!overlap) {
    GCVL_CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, S.stream));
    return;
  }
  // every CTA of a cooperative launch is resident at once, so the grid
  // barrier's waits end
  static int per_sm = -1;
  if (per_sm < 0) {
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_move_overlap, MV_BLOCK, 0) != cudaSuccess ||
        per_sm < 1) {
      cudaGetLastError();
      per_sm = 1;
    }
  }
  const long need = ((long)size + MV_CHUNK - 1) / MV_CHUNK;
  const long cap = (long)per_sm * S.sm_count;
  int grid = (int)(need < cap ? need : cap);
  unsigned *bar = (unsigned *)((char *)S.d_small + 512);  // count, generation
  if (!GCVL_CK(cudaMemsetAsync(bar, 0, 8, S.stream))) return;
  unsigned long long *dp = (unsigned long long *)d;
  const unsigned long long *sp = (const unsigned long long *)s;
  long units = size;
  int up = dst > src;
  unsigned *status = S.d_status;
  int limit = S.spin_limit;
  void *args[] = {&dp, &sp, &units, &up, &bar, &status, &limit};
  GCVL_CK(cudaLaunchCooperativeKernel((const void *)k_move_overlap, dim3(grid), dim3(MV_BLOCK), args, 0, S.stream));
  launch_check("k_move_overlap");
}
GCVL_EXPORT int mov_fov_scratch(int size) { (void)size; return 0; }

// Pointer arithmetic in 8-byte units (facilt.c:186-234).
GCVL_EXPORT vec_p add_fov(vec_p v, int a) { return (vec_p)((char *)v + (long)a * 8); }
GCVL_EXPORT int sub_fov(vec_p v1, vec_p v2) {
  long d = ((char *)v1 - (char *)v2) / 8;
  return (int)(d < 0 ? -d : d);
}
GCVL_EXPORT cvl_bool eql_fov(vec_p v1, vec_p v2) { return v1 == v2; }
GCVL_EXPORT int cmp_fov(vec_p v1, vec_p v2) { return (int)(((char *)v1 - (char *)v2) / 8); }

// CVL <-> C transfers (facilt.c:236-275).  Both block until the copy is
// done, so the caller may reuse or read its host buffer on return.
#define GCVL_XFER(L, T)                                                                   \
  GCVL_EXPORT void v2c_fu##L(T *d, vec_p s, int len, vec_p scratch) {                     \
    (void)scratch; ensure_init();                                                          \
    if (len <= 0) return;                                                                  \
    GCVL_CK(cudaMemcpyAsync(d, s, (size_t)len * sizeof(T), cudaMemcpyDeviceToHost,         \
                            st().stream));                                                 \
    GCVL_CK(cudaStreamSynchronize(st().stream));                                           \
  }                                                                                        \
  GCVL_EXPORT int v2c_fu##L##_scratch(int len) { (void)len; return 0; }                   \
  GCVL_EXPORT unsigned v2c_fu##L##_inplace(void) { return INPLACE_NONE; }                 \
  GCVL_EXPORT void c2v_fu##L(vec_p d, T *s, int len, vec_p scratch) {                     \
    (void)scratch; ensure_init();                                                          \
    if (len <= 0) return;                                                                  \
    GCVL_CK(cudaMemcpyAsync(d, s, (size_t)len * sizeof(T), cudaMemcpyHostToDevice,         \
                            st().stream));                                                 \
    GCVL_CK(cudaStreamSynchronize(st().stream));                                           \
  }                                                                                        \
  GCVL_EXPORT int c2v_fu##L##_scratch(int len) { (void)len; return 0; }                   \
  GCVL_EXPORT unsigned c2v_fu##L##_inplace(void) { return INPLACE_NONE; }
GCVL_XFER(z, int)
GCVL_XFER(b, cvl_bool)
GCVL_XFER(d, double)

// Asynchronous transfer variants for callers that manage their own host
// buffers (pinned memory) and synchronise with gcvl_sync().
GCVL_EXPORT void gcvl_h2d_async(vec_p d, const void *s, size_t bytes) {
  ensure_init();
  GCVL_CK(cudaMemcpyAsync(d, s, bytes, cudaMemcpyHostToDevice, st().stream));
}
GCVL_EXPORT void gcvl_d2h_async(void *d, vec_p s, size_t bytes) {
  ensure_init();
  GCVL_CK(cudaMemcpyAsync(d, s, bytes, cudaMemcpyDeviceToHost, st().stream));
}

// RAND seed.  The serial CVL on Linux seeds srandom() (facilt.c:292-311)
// although RAND draws from lrand48(); this library seeds the lrand48 stream
// as srand48(seed) does, so that rand_seed makes RAND reproducible.
GCVL_EXPORT void rnd_foz(int seed) {
  st().rand48 = ((((uint64_t)(uint32_t)seed) << 16) | 0x330EULL) & 0xFFFFFFFFFFFFULL;
}
GCVL_EXPORT unsigned long long gcvl_rand_state(void) { return st().rand48; }
GCVL_EXPORT void gcvl_set_rand_state(unsigned long long s) { st().rand48 = s & 0xFFFFFFFFFFFFULL; }
