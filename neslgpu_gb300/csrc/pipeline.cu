// pipeline.cu -- CUDA graphs over library calls, a device-resident reduction
// for graph-captured sequences, and the per-vector call loop that a caller
// issuing one CVL sequence per vector (as vinterp does per VCODE basic block)
// would run.  Used by the batched form (neslgpu_gb300/batch.py).
#include "gcvl.cuh"

#include <stdlib.h>

using namespace gcvl;

// ------------------------------------------------------------ CUDA graphs
// Every library call issued between gcvl_graph_begin() and gcvl_graph_end()
// is captured from the library stream into one executable graph instead of
// running.  Captured calls must not synchronise (no *_ru*, ext_vu*, pk1_luv,
// c2v/v2c) and must be given scratch vectors (the library workspace may need
// to grow, which cannot happen during capture).
GCVL_EXPORT int gcvl_graph_begin(void) {
  ensure_init();
  return GCVL_CK(cudaStreamBeginCapture(stream(), cudaStreamCaptureModeThreadLocal)) ? 0 : st().err;
}
GCVL_EXPORT void *gcvl_graph_end(void) {
  cudaGraph_t g = nullptr;
  if (!GCVL_CK(cudaStreamEndCapture(stream(), &g))) return nullptr;
  cudaGraphExec_t e = nullptr;
  cudaError_t r = cudaGraphInstantiate(&e, g, 0);
  cudaGraphDestroy(g);
  if (!GCVL_CK(r)) return nullptr;
  return (void *)e;
}
GCVL_EXPORT int gcvl_graph_launch(void *exec) {
  return GCVL_CK(cudaGraphLaunch((cudaGraphExec_t)exec, stream())) ? 0 : st().err;
}
GCVL_EXPORT void gcvl_graph_destroy(void *exec) {
  if (exec) cudaGraphExecDestroy((cudaGraphExec_t)exec);
}

// --------------------------------------------------- per-vector call loop
// For each of nvec vectors (concatenated in x, inner segment lengths in
// seg_lens, vector v owning nseg_of[v] segments), the sequence a VCODE
// basic block issues through the CVL ABI:
//   MAKE_SEGDES, +_SCAN of x, DIST 0, x > 0, PACK of the scan by those flags (pk1_lev, +_REDUCE -> host,
//   MAKE_SEGDES, pk2_le), DIST of the new lengths, RAND, BPERMUTE
// all on device vectors, one vector at a time.  Results land at the same
// places as the batched form's, so the two can be compared.
//   work: scratch vec_p of gcvl_pipeline_scratch(...) units
//   y, f, p, bnd, idx, g: outputs (scan, flags, packed, bounds, indices, gathered)
//   newlens: packed segment lengths (sum(nseg_of) entries)
//   sd_work / sd2_work: segment descriptor storage, siz_fos(n_max, m_max)
template <class T>
static int percall(T *x, const int *seg_lens_host, const int *nseg_of, const int *len_of, int nvec, T *y,
                   int *f, T *p, int *newlens, int *bnd, int *idx, T *g, vec_p zeros, vec_p lens_dev,
                   vec_p sd, vec_p sd2, vec_p work, unsigned seed);

#define PC_CALLS(L, T)                                                                                 \
  static void pc_scan(T *d, T *s, vec_p sd, int n, int m, vec_p w) { add_se##L(d, s, sd, n, m, w); }   \
  static void pc_dis(T *d, int n) { dis_vu##L(d, (T)0, n, nullptr); }                                  \
  static void pc_grt(int *f, T *a, T *b, int n) { grt_wu##L(f, a, b, n, nullptr); }                      \
  static void pc_pack(T *d, T *s, int *f, vec_p sd, int n, int m, vec_p sd2, int n2, vec_p w) {           \
    pk2_le##L(d, s, f, sd, n, m, sd2, n2, m, w);                                                        \
  }                                                                                                      \
  static void pc_gather(T *d, T *s, int *i, vec_p sd, int n, int m, vec_p w) {                         \
    bck_pe##L(d, s, i, sd, n, m, sd, n, m, w);                                                          \
  }
PC_CALLS(z, int)
PC_CALLS(d, double)

template <class T>
static int percall(T *x, const int *seg_lens_host, const int *nseg_of, const int *len_of, int nvec, T *y,
                   int *f, T *p, int *newlens, int *bnd, int *idx, T *g, vec_p zeros, vec_p lens_dev,
                   vec_p sd, vec_p sd2, vec_p work, unsigned seed) {
  long eoff = 0, soff = 0, poff = 0;
  rnd_foz((int)seed);
  for (int v = 0; v < nvec; v++) {
    const int n = len_of[v], m = nseg_of[v];
    // MAKE_SEGDES: lengths come from the program (here: the host copy)
    c2v_fuz(lens_dev, (int *)(seg_lens_host + soff), m, nullptr);
    mke_fov(sd, lens_dev, n, m, work);
    pc_scan(y + eoff, x + eoff, sd, n, m, work);
    pc_dis((T *)zeros, n);
    pc_grt(f + eoff, x + eoff, (T *)zeros, n);
    pk1_lev(newlens + soff, f + eoff, sd, n, m, work);
    const int n2 = add_ruz(newlens + soff, m, work);  // host synchronisation, as in vinterp
    mke_fov(sd2, newlens + soff, n2, m, work);
    pc_pack(p + poff, y + eoff, f + eoff, sd, n, m, sd2, n2, work);
    dis_vez(bnd + poff, newlens + soff, sd2, n2, m, nullptr);
    rnd_wuz(idx + poff, bnd + poff, n2, nullptr);
    pc_gather(g + poff, p + poff, idx + poff, sd2, n2, m, work);
    eoff += n;
    soff += m;
    poff += n2;
  }
  return gcvl_sync();
}

GCVL_EXPORT int gcvl_pipeline_percall(int is_double, vec_p x, const int *seg_lens_host, const int *nseg_of,
                                      const int *len_of, int nvec, vec_p y, vec_p f, vec_p p, vec_p newlens,
                                      vec_p bnd, vec_p idx, vec_p g, vec_p zeros, vec_p lens_dev, vec_p sd,
                                      vec_p sd2, vec_p work, unsigned seed) {
  ensure_init();
  if (is_double)
    return percall<double>((double *)x, seg_lens_host, nseg_of, len_of, nvec, (double *)y, (int *)f,
                           (double *)p, (int *)newlens, (int *)bnd, (int *)idx, (double *)g, zeros, lens_dev,
                           sd, sd2, work, seed);
  return percall<int>((int *)x, seg_lens_host, nseg_of, len_of, nvec, (int *)y, (int *)f, (int *)p,
                      (int *)newlens, (int *)bnd, (int *)idx, (int *)g, zeros, lens_dev, sd, sd2, work, seed);
}
