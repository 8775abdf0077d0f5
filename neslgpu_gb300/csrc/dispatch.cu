// dispatch.cu -- the learned dispatcher: features of a segment descriptor,
// a small FP32 MLP (16 features -> 64 -> 64 -> softmax over the kernel
// variants of variants.cu) with hand-written training and inference
// kernels, and an entry point that runs whichever variant the model picks.
//
// The model is trained on timings the library itself produces (the
// autotuner in neslgpu_gb300/dispatch.py times every valid variant of each
// instance); targets are soft (variants within a few percent of the best
// share the probability mass), invalid variants are masked out of the
// softmax.  A choice only selects among variants that compute the same CVL
// function, so it never changes what is computed -- only how fast.
#include "gcvl.cuh"

#include <math.h>
#include <string.h>

#include <map>
#include <string>
#include <tuple>

namespace gcvl {

constexpr int MF = 16, MH = 64, MK = 8;  // features, hidden width, classes
constexpr int P_W1 = 0, P_B1 = P_W1 + MF * MH, P_W2 = P_B1 + MH, P_B2 = P_W2 + MH * MH, P_W3 = P_B2 + MH,
              P_B3 = P_W3 + MH * MK, P_COUNT = P_B3 + MK;
constexpr int FEAT_STRIDE = MF + MK;  // a features row: 16 features, then the 8-entry validity mask
constexpr int RB_MAXLEN = 2048;       // the per-segment rank variant's limit (variants.cu)

// ---------------------------------------------------------- features ---
struct FeatAcc {
  double sumsq;
  unsigned long long bucket[6];  // segments with length in [0,4) [4,32) [32,256) [256,2048) [2048,65536) [65536,)
  unsigned long long long_elems; // elements in segments of length >= 65536
  int maxlen;
};
__device__ __forceinline__ int len_bucket(int L) {
  return L < 4 ? 0 : L < 32 ? 1 : L < 256 ? 2 : L < 2048 ? 3 : L < 65536 ? 4 : 5;
}
__global__ void __launch_bounds__(256) k_seg_stats(const int *__restrict__ len, int m, FeatAcc *acc) {
  __shared__ unsigned long long s_b[6], s_long;
  __shared__ double s_sq;
  __shared__ int s_max;
  if (threadIdx.x < 6) s_b[threadIdx.x] = 0;
  if (threadIdx.x == 0) { s_long = 0; s_sq = 0.0; s_max = 0; }
  __syncthreads();
  unsigned long long b[6] = {0, 0, 0, 0, 0, 0}, lg = 0;
  double sq = 0.0;
  int mx = 0;
  for (long i = (long)blockIdx.x * 256 + threadIdx.x; i < m; i += (long)gridDim.x * 256) {
    const int L = __ldg(len + i);
    const int bk = len_bucket(L);
#pragma unroll
    for (int k = 0; k < 6; k++) b[k] += bk == k;
    if (L >= 65536) lg += (unsigned long long)L;
    sq += (double)L * (double)L;
    mx = max(mx, L);
  }
  for (int k = 0; k < 6; k++) if (b[k]) atomicAdd(&s_b[k], b[k]);
  if (lg) atomicAdd(&s_long, lg);
  if (sq != 0.0) atomicAdd(&s_sq, sq);
  atomicMax(&s_max, mx);
  __syncthreads();
  if (threadIdx.x < 6 && s_b[threadIdx.x]) atomicAdd(&acc->bucket[threadIdx.x], s_b[threadIdx.x]);
  if (threadIdx.x == 0) {
    if (s_long) atomicAdd(&acc->long_elems, s_long);
    if (s_sq != 0.0) atomicAdd(&acc->sumsq, s_sq);
    atomicMax(&acc->maxlen, s_max);
  }
}
// kind: 0 scan, 1 reduce, 2 rank
__global__ void k_seg_features(const FeatAcc *acc, int n, int m, int kind, int is_double, float *out) {
  if (threadIdx.x != 0) return;
  const double mm = m > 0 ? (double)m : 1.0;
  const double mean = (double)n / mm;
  double var = acc->sumsq / mm - mean * mean;
  if (var < 0) var = 0;
  float f[MF];
  f[0] = (float)(log2((double)n + 1.0) / 32.0);
  f[1] = (float)(log2((double)m + 1.0) / 32.0);
  f[2] = (float)(log2(mean + 1.0) / 24.0);
  f[3] = (float)(log2(sqrt(var) + 1.0) / 24.0);
  f[4] = (float)(log2((double)acc->maxlen + 1.0) / 24.0);
  f[5] = n > 0 ? (float)((double)acc->long_elems / (double)n) : 0.f;
  for (int k = 0; k < 6; k++) f[6 + k] = (float)((double)acc->bucket[k] / mm);
  f[12] = kind == 0; f[13] = kind == 1; f[14] = kind == 2; f[15] = (float)is_double;
  for (int k = 0; k < MF; k++) out[k] = f[k];
  // validity mask over the classes (variants.cu: 0 flat, 1-4 segment owners, 5 per-segment rank)
  for (int k = 0; k < MK; k++) {
    float v = 0.f;
    if (k == 0) v = 1.f;
    else if (k <= 4) v = kind != 2;
    else if (k == 5) v = kind == 2 && acc->maxlen <= RB_MAXLEN;
    out[MF + k] = v;
  }
}

// ---------------------------------------------------------- the MLP ----
// One warp evaluates one sample; lane j holds hidden units j and j + 32.
struct Fwd {
  float x, h1a, h1b, h2a, h2b, logit;  // x: feature (lane & 15); logit: class lane & 7
};
__device__ __forceinline__ float relu(float v) { return v > 0.f ? v : 0.f; }
__device__ __forceinline__ Fwd mlp_forward(const float *p, const float *xrow, const float *mask, int lane) {
  Fwd r;
  r.x = xrow[lane & 15];
  float a = p[P_B1 + lane], b = p[P_B1 + lane + 32];
#pragma unroll
  for (int i = 0; i < MF; i++) {
    const float xi = __shfl_sync(0xffffffffu, r.x, i);
    a = fmaf(xi, p[P_W1 + i * MH + lane], a);
    b = fmaf(xi, p[P_W1 + i * MH + lane + 32], b);
  }
  r.h1a = relu(a); r.h1b = relu(b);
  a = p[P_B2 + lane]; b = p[P_B2 + lane + 32];
#pragma unroll 8
  for (int i = 0; i < MH; i++) {
    const float hi = __shfl_sync(0xffffffffu, i < 32 ? r.h1a : r.h1b, i & 31);
    a = fmaf(hi, p[P_W2 + i * MH + lane], a);
    b = fmaf(hi, p[P_W2 + i * MH + lane + 32], b);
  }
  r.h2a = relu(a); r.h2b = relu(b);
  const int k = lane & 7;
  float z = p[P_B3 + k];
#pragma unroll 8
  for (int i = 0; i < MH; i++) {
    const float hi = __shfl_sync(0xffffffffu, i < 32 ? r.h2a : r.h2b, i & 31);
    z = fmaf(hi, p[P_W3 + i * MK + k], z);
  }
  r.logit = mask[k] > 0.f ? z : -INFINITY;
  return r;
}

// Training: one CTA of 32 warps, parameters, gradients and Adam moments in
// shared memory; `epochs` passes over the N samples in minibatches of
// `batch`, the order a fresh affine permutation each epoch.  loss[e] gets
// the epoch's mean cross-entropy.
__global__ void __launch_bounds__(1024) k_mlp_train(float *params, float *moments, const float *X, const float *T,
                                                    int N, int epochs, int batch, float lr, unsigned perm_a,
                                                    unsigned seed, int step0, float *loss) {
  extern __shared__ float sm[];
  float *p = sm, *g = sm + P_COUNT, *m1 = g + P_COUNT, *m2 = m1 + P_COUNT;
  __shared__ float s_loss;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int i = tid; i < P_COUNT; i += 1024) {
    p[i] = params[i]; g[i] = 0.f; m1[i] = moments[i]; m2[i] = moments[P_COUNT + i];
  }
  __syncthreads();
  if (tid == 0) s_loss = 0.f;
  __syncthreads();
  int step = step0;
  for (int e = 0; e < epochs; e++) {
    const unsigned off = (seed * 2654435761u + (unsigned)e * 40503u) % (unsigned)N;
    for (int b0 = 0; b0 < N; b0 += batch) {
      const int bn = min(batch, N - b0);
      for (int j = warp; j < bn; j += 32) {
        const int sidx = (int)(((unsigned long long)(b0 + j) * perm_a + off) % (unsigned)N);
        const float *xrow = X + (long)sidx * FEAT_STRIDE;
        const float *trow = T + (long)sidx * MK;
        const Fwd f = mlp_forward(p, xrow, xrow + MF, lane);
        // softmax over the valid classes (lanes 0..7 hold them)
        float mx = lane < MK ? f.logit : -INFINITY;
        for (int o = 4; o; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        float ex = (lane < MK && f.logit != -INFINITY) ? expf(f.logit - mx) : 0.f;
        float sum = ex;
        for (int o = 4; o; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
        const float pk = sum > 0.f ? ex / sum : 0.f;
        const float tk = lane < MK ? trow[lane & 7] : 0.f;
        const float dl = lane < MK ? pk - tk : 0.f;  // d(cross-entropy)/d(logit)
        if (lane < MK && tk > 0.f) atomicAdd(&s_loss, -tk * logf(fmaxf(pk, 1e-30f)));
        // layer 3
        if (lane < MK) atomicAdd(&g[P_B3 + lane], dl);
        float d2a = 0.f, d2b = 0.f;
#pragma unroll
        for (int k = 0; k < MK; k++) {
          const float dk = __shfl_sync(0xffffffffu, dl, k);
          atomicAdd(&g[P_W3 + lane * MK + k], f.h2a * dk);
          atomicAdd(&g[P_W3 + (lane + 32) * MK + k], f.h2b * dk);
          d2a = fmaf(p[P_W3 + lane * MK + k], dk, d2a);
          d2b = fmaf(p[P_W3 + (lane + 32) * MK + k], dk, d2b);
        }
        d2a = f.h2a > 0.f ? d2a : 0.f;
        d2b = f.h2b > 0.f ? d2b : 0.f;
        // layer 2
        atomicAdd(&g[P_B2 + lane], d2a);
        atomicAdd(&g[P_B2 + lane + 32], d2b);
        float d1a = 0.f, d1b = 0.f;
#pragma unroll 8
        for (int i = 0; i < MH; i++) {
          const float hi = __shfl_sync(0xffffffffu, i < 32 ? f.h1a : f.h1b, i & 31);
          atomicAdd(&g[P_W2 + i * MH + lane], hi * d2a);
          atomicAdd(&g[P_W2 + i * MH + lane + 32], hi * d2b);
        }
#pragma unroll 8
        for (int j2 = 0; j2 < MH; j2++) {
          const float dj = __shfl_sync(0xffffffffu, j2 < 32 ? d2a : d2b, j2 & 31);
          d1a = fmaf(p[P_W2 + lane * MH + j2], dj, d1a);
          d1b = fmaf(p[P_W2 + (lane + 32) * MH + j2], dj, d1b);
        }
        d1a = f.h1a > 0.f ? d1a : 0.f;
        d1b = f.h1b > 0.f ? d1b : 0.f;
        // layer 1
        atomicAdd(&g[P_B1 + lane], d1a);
        atomicAdd(&g[P_B1 + lane + 32], d1b);
#pragma unroll
        for (int i = 0; i < MF; i++) {
          const float xi = __shfl_sync(0xffffffffu, f.x, i);
          atomicAdd(&g[P_W1 + i * MH + lane], xi * d1a);
          atomicAdd(&g[P_W1 + i * MH + lane + 32], xi * d1b);
        }
      }
      __syncthreads();
      // Adam (beta1 0.9, beta2 0.999)
      step++;
      const float c1 = 1.f - powf(0.9f, (float)step), c2 = 1.f - powf(0.999f, (float)step);
      for (int i = tid; i < P_COUNT; i += 1024) {
        const float gi = g[i] / (float)bn;
        m1[i] = 0.9f * m1[i] + 0.1f * gi;
        m2[i] = 0.999f * m2[i] + 0.001f * gi * gi;
        p[i] -= lr * (m1[i] / c1) / (sqrtf(m2[i] / c2) + 1e-8f);
        g[i] = 0.f;
      }
      __syncthreads();
    }
    if (tid == 0) {
      if (loss) loss[e] = s_loss / (float)N;
      s_loss = 0.f;
    }
    __syncthreads();
  }
  for (int i = tid; i < P_COUNT; i += 1024) {
    params[i] = p[i]; moments[i] = m1[i]; moments[P_COUNT + i] = m2[i];
  }
}

// Inference: one warp per sample; cls[s] = the valid class of largest logit.
__global__ void __launch_bounds__(256) k_mlp_infer(const float *__restrict__ params, const float *__restrict__ X,
                                                   int N, int *cls) {
  const int lane = threadIdx.x & 31;
  const int s = blockIdx.x * 8 + (threadIdx.x >> 5);
  if (s >= N) return;
  const float *xrow = X + (long)s * FEAT_STRIDE;
  const Fwd f = mlp_forward(params, xrow, xrow + MF, lane);
  float best = lane < MK ? f.logit : -INFINITY;
  int arg = lane < MK ? lane : MK;
  for (int o = 4; o; o >>= 1) {
    const float ob = __shfl_xor_sync(0xffffffffu, best, o);
    const int oa = __shfl_xor_sync(0xffffffffu, arg, o);
    if (ob > best || (ob == best && oa < arg)) { best = ob; arg = oa; }
  }
  if (lane == 0) cls[s] = best == -INFINITY ? 0 : arg;
}

// ------------------------------------------------------ auto dispatch ---
struct DispatchState {
  float *model = nullptr;   // device copy of the parameters (null: always the default kernel)
  float *feat = nullptr;    // device features row
  FeatAcc *acc = nullptr;
  int *cls_dev = nullptr;
  int *cls_host = nullptr;  // pinned
  std::map<std::tuple<std::string, const void *, int, int>, int> cache;
};
static DispatchState &ds() { static DispatchState d; return d; }

static int prim_kind(const char *prim, int *is_double) {
  const size_t L = strlen(prim);
  *is_double = L > 0 && prim[L - 1] == 'd';
  if (L >= 6 && prim[0] == 'r' && prim[1] == 'k') return 2;
  if (L >= 6 && prim[4] == 'r') return 1;
  return 0;
}

static bool features_into(const char *prim, vec_p sd, int n, int m, float *out) {
  DispatchState &D = ds();
  if (!D.acc && !GCVL_CK(cudaMalloc(&D.acc, sizeof(FeatAcc)))) return false;
  int is_double;
  const int kind = prim_kind(prim, &is_double);
  GCVL_CK(cudaMemsetAsync(D.acc, 0, sizeof(FeatAcc), stream()));
  if (m > 0) {
    SegView sv = seg_view(sd, n, m);
    long g = ((long)m + 255) / 256;
    if (g > (long)st().sm_count * 8) g = (long)st().sm_count * 8;
    k_seg_stats<<<(int)g, 256, 0, stream()>>>(sv.len, m, D.acc);
    launch_check("k_seg_stats");
  }
  k_seg_features<<<1, 32, 0, stream()>>>(D.acc, n, m, kind, is_double, out);
  launch_check("k_seg_features");
  return true;
}

}  // namespace gcvl

using namespace gcvl;

GCVL_EXPORT int gcvl_mlp_param_count(void) { return P_COUNT; }
GCVL_EXPORT int gcvl_mlp_feature_stride(void) { return FEAT_STRIDE; }
GCVL_EXPORT int gcvl_mlp_classes(void) { return MK; }

// Features (16 floats) and the validity mask (8 floats) of calling `prim`
// on the descriptor sd, written to out_dev (device memory, 24 floats).
GCVL_EXPORT int gcvl_seg_features(const char *prim, vec_p sd, int n, int m, float *out_dev) {
  ensure_init();
  features_into(prim, sd, n, m, out_dev);
  return st().err;
}

// Trains the model in place: params (P floats) and moments (2P floats,
// zero at the start), N samples of X (N x 24: features and mask) against
// soft targets T (N x 8); all device pointers.  loss_dev: epochs floats or
// NULL.
GCVL_EXPORT int gcvl_mlp_train(float *params, float *moments, const float *X, const float *T, int N, int epochs,
                               int batch, float lr, unsigned seed, int step0, float *loss_dev) {
  ensure_init();
  if (N <= 0 || batch <= 0 || epochs <= 0) return 0;
  // an odd multiplier coprime to N gives a permutation of [0, N)
  unsigned a = 2654435761u % (unsigned)N;
  auto gcd = [](unsigned x, unsigned y) { while (y) { unsigned t = x % y; x = y; y = t; } return x; };
  if (a == 0) a = 1;
  while (gcd(a, (unsigned)N) != 1) a++;
  const size_t smem = (size_t)4 * P_COUNT * sizeof(float);
  static bool attr = false;
  if (!attr) {
    GCVL_CK(cudaFuncSetAttribute(k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr = true;
  }
  k_mlp_train<<<1, 1024, smem, stream()>>>(params, moments, X, T, N, epochs, batch, lr, a, seed, step0, loss_dev);
  launch_check("k_mlp_train");
  return st().err;
}

GCVL_EXPORT int gcvl_mlp_infer(const float *params, const float *X, int N, int *cls_dev) {
  ensure_init();
  if (N <= 0) return 0;
  k_mlp_infer<<<(N + 7) / 8, 256, 0, stream()>>>(params, X, N, cls_dev);
  launch_check("k_mlp_infer");
  return st().err;
}

// Installs a trained model (P floats, host memory) for gcvl_auto_run; NULL
// removes it.  Clears the decision cache.
GCVL_EXPORT int gcvl_dispatch_set_model(const float *params_host) {
  ensure_init();
  DispatchState &D = ds();
  D.cache.clear();
  if (!params_host) {
    if (D.model) cudaFree(D.model);
    D.model = nullptr;
    return 0;
  }
  if (!D.model && !GCVL_CK(cudaMalloc(&D.model, P_COUNT * sizeof(float)))) return st().err;
  GCVL_CK(cudaMemcpy(D.model, params_host, P_COUNT * sizeof(float), cudaMemcpyHostToDevice));
  return st().err;
}

// The class the installed model picks for prim on this descriptor (0, the
// default kernel, when no model is installed).  Synchronises to read the
// choice; choices are cached per (prim, descriptor address, n, m).
GCVL_EXPORT int gcvl_dispatch_choice(const char *prim, vec_p sd, int n, int m) {
  ensure_init();
  DispatchState &D = ds();
  if (!D.model || n <= 0 || m <= 0) return 0;
  auto key = std::make_tuple(std::string(prim), (const void *)sd, n, m);
  auto it = D.cache.find(key);
  if (it != D.cache.end()) return it->second;
  if (!D.feat && !GCVL_CK(cudaMalloc(&D.feat, FEAT_STRIDE * sizeof(float)))) return 0;
  if (!D.cls_dev && !GCVL_CK(cudaMalloc(&D.cls_dev, sizeof(int)))) return 0;
  if (!D.cls_host && !GCVL_CK(cudaMallocHost(&D.cls_host, sizeof(int)))) return 0;
  if (!features_into(prim, sd, n, m, D.feat)) return 0;
  k_mlp_infer<<<1, 256, 0, stream()>>>(D.model, D.feat, 1, D.cls_dev);
  launch_check("k_mlp_infer");
  GCVL_CK(cudaMemcpyAsync(D.cls_host, D.cls_dev, sizeof(int), cudaMemcpyDeviceToHost, stream()));
  GCVL_CK(cudaStreamSynchronize(stream()));
  const int c = *D.cls_host;
  D.cache[key] = c;
  return c;
}

// prim (a CVL segmented scan, reduction or rank name) run by the variant
// the installed model picks; CVL argument order, scratch of
// gcvl_variant_scratch.  Returns 0 or a GCVL error code.
GCVL_EXPORT int gcvl_auto_run(const char *prim, vec_p d, vec_p s, vec_p sd, int n, int m, vec_p scratch) {
  const int c = gcvl_dispatch_choice(prim, sd, n, m);
  return gcvl_run_variant(prim, c, d, s, sd, n, m, scratch);
}
