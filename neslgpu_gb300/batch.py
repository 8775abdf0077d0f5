"""The batched form: many segmented vectors of uneven lengths at once.

Workload (per vector, inner segments geometric with mean 32):
    y = add_se(x)            segmented exclusive +-scan
    f = grt_wu(x, 0)         flags x > 0
    p = pack(y, f)           PACK: pk1_lev, +_REDUCE, MAKE_SEGDES, pk2_le
    i = rand % len(seg)      RAND of a per-segment bound
    g = bck_pe(p, i)         gather within each packed segment

Three ways to run it, all through the C ABI of libcvl_gb300.so:

* ``percall``  -- one CVL call sequence per vector (a C loop inside the
  library: ``gcvl_pipeline_percall``), reading the PACK length back to the
  host for every vector, as an interpreter executing one vector per basic
  block does;
* ``batched``  -- NESL's flattening: the vectors' inner segments are
  concatenated into one segmented vector, so each primitive is one launch
  over all vectors (segments never cross vector boundaries, so results are
  the same);
* ``graph``    -- the batched sequence replayed from two CUDA graphs, split
  at the one host read PACK needs (the packed length); the second graph is
  captured once per packed length.

Float64 scans of the flattened vector may differ from per-vector scans by
reassociation only; integer results are identical in all three modes.
"""
from __future__ import annotations

import ctypes as C
import time
from dataclasses import dataclass, field

import numpy as np

from . import workloads as W
from .cvl import CVL, check, load


@dataclass
class BatchData:
    nvec: int
    vec_len: np.ndarray        # elements per vector
    nseg: np.ndarray           # inner segments per vector
    seg_lens: np.ndarray       # all inner segment lengths, vector after vector
    n: int
    m: int


def make_batch(nvec: int, total: int, seed: int = 3, lo: int = 10, hi: int = 10 ** 6,
               inner_mean: float = 32.0) -> BatchData:
    """nvec vector lengths, log-normal clipped to [lo, hi] and rescaled so
    they sum to about `total`; inner segments geometric with `inner_mean`."""
    r = W.rng(seed)
    raw = np.clip(np.exp(r.normal(np.log(np.sqrt(lo * hi)), 1.6, size=nvec)), lo, hi)
    vl = np.clip(np.rint(raw * (total / raw.sum())), lo, hi).astype(np.int64)
    return batch_from_lengths(vl, r, inner_mean)


def make_skewed_batch(huge: int = 4, huge_len: int = 1 << 24, tiny: int = 8188, tiny_hi: int = 100,
                      seed: int = 5, inner_mean: float = 32.0) -> BatchData:
    """The flattened form's worst case: a few huge vectors beside thousands
    of tiny ones (lengths log-uniform in [1, tiny_hi]), the huge ones spread
    among the tiny."""
    r = W.rng(seed)
    small = np.rint(np.exp(r.uniform(0.0, np.log(tiny_hi), size=tiny))).astype(np.int64)
    vl = np.concatenate([np.full(huge, huge_len, dtype=np.int64), np.maximum(small, 1)])
    return batch_from_lengths(vl[r.permutation(vl.size)], r, inner_mean)


def single_vector_batch(total: int, seed: int = 6, inner_mean: float = 32.0) -> BatchData:
    """One vector of `total` elements: the same work with no vector
    boundaries, which no launch scheme over the same bytes can beat."""
    return batch_from_lengths(np.array([total], dtype=np.int64), W.rng(seed), inner_mean)


def batch_from_lengths(vl: np.ndarray, r, inner_mean: float = 32.0) -> BatchData:
    """Vectors of the given lengths, inner segments geometric with `inner_mean`."""
    nvec = int(vl.size)
    segs, nseg = [], []
    for L in vl:
        s = W.geometric_lengths(r, int(L), inner_mean)
        segs.append(s)
        nseg.append(len(s))
    seg_lens = np.concatenate(segs).astype(np.int32)
    return BatchData(nvec, vl.astype(np.int32), np.array(nseg, dtype=np.int32), seg_lens,
                     int(vl.sum()), int(seg_lens.size))


class BatchRun:
    """Device buffers for one element type of the batch and the three modes."""

    def __init__(self, b: BatchData, is_double: bool, seed: int = 11, cvl: CVL | None = None):
        self.c = c = cvl or load()
        self.b = b
        self.dbl = is_double
        self.L = "d" if is_double else "z"
        n, m = b.n, b.m
        esz = c.siz_fod(n) if is_double else c.siz_foz(n)
        al = lambda u: self._alloc(u)
        self.x, self.y, self.p, self.g = al(esz), al(esz), al(esz), al(esz)
        self.zeros = al(esz)
        self.f, self.bnd, self.idx = al(c.siz_foz(n)), al(c.siz_foz(n)), al(c.siz_foz(n))
        self.newlens = al(c.siz_foz(m))
        self.lens = al(c.siz_foz(m))
        self.sd, self.sd2 = al(c.siz_fos(n, m)), al(c.siz_fos(n, m))
        self.count = al(1)
        L = self.L
        self.work = al(max(c.mke_fov_scratch(n, m), getattr(c, f"add_se{L}_scratch")(n, m),
                           c.pk1_lev_scratch(n, m), getattr(c, f"pk2_le{L}_scratch")(n, m, n, m),
                           c.gcvl_add_ruz_dev_scratch(m), c.add_ruz_scratch(m)))
        c.gcvl_fill_random(self.x, n, 1 if is_double else 3, seed, 0.0, 2001)
        if not is_double:  # ints in [-1000, 1000]
            self._shift_ints(n)
        c.c2v_fuz(self.lens, b.seg_lens.ctypes.data, m, None)
        self.host_count = c.gcvl_host_alloc(8)
        self.graphs = {}
        self.seed = 12345
        check(c)

    def _alloc(self, units):
        p = self.c.alo_foz(int(max(units, 1)))
        if not p:
            raise MemoryError(self.c.gcvl_error_string().decode())
        return p

    def _shift_ints(self, n):
        # x in [0, 2001) -> [-1000, 1000]: x + (-1000) with a distributed constant
        c = self.c
        c.dis_vuz(self.zeros, -1000, n, None)
        c.add_wuz(self.x, self.x, self.zeros, n, None)

    # ------------------------------------------------------------ modes
    def percall(self):
        c, b = self.c, self.b
        rc = c.gcvl_pipeline_percall(int(self.dbl), self.x, b.seg_lens.ctypes.data, b.nseg.ctypes.data,
                                     b.vec_len.ctypes.data, b.nvec, self.y, self.f, self.p, self.newlens,
                                     self.bnd, self.idx, self.g, self.zeros, self.lens, self.sd, self.sd2,
                                     self.work, self.seed)
        if rc:
            check(c)
        return self._packed_len_host()

    def _front(self, dev_count: bool):
        c, b, L = self.c, self.b, self.L
        n, m = b.n, b.m
        c.mke_fov(self.sd, self.lens, n, m, self.work)
        getattr(c, f"add_se{L}")(self.y, self.x, self.sd, n, m, self.work)
        if self.dbl:
            c.dis_vud(self.zeros, 0.0, n, None)
        else:
            c.dis_vuz(self.zeros, 0, n, None)
        getattr(c, f"grt_wu{L}")(self.f, self.x, self.zeros, n, None)
        c.pk1_lev(self.newlens, self.f, self.sd, n, m, self.work)
        if dev_count:
            c.gcvl_add_ruz_dev(self.count, self.newlens, m, self.work)

    def _back(self, n2: int):
        c, b, L = self.c, self.b, self.L
        n, m = b.n, b.m
        c.mke_fov(self.sd2, self.newlens, n2, m, self.work)
        getattr(c, f"pk2_le{L}")(self.p, self.y, self.f, self.sd, n, m, self.sd2, n2, m, self.work)
        c.dis_vez(self.bnd, self.newlens, self.sd2, n2, m, None)
        c.rnd_wuz(self.idx, self.bnd, n2, None)
        getattr(c, f"bck_pe{L}")(self.g, self.p, self.idx, self.sd2, n2, m, self.sd2, n2, m, self.work)

    def batched(self):
        c = self.c
        c.rnd_foz(self.seed)
        self._front(False)
        n2 = c.add_ruz(self.newlens, self.b.m, self.work)  # the one host read
        self._back(n2)
        c.gcvl_sync()
        return n2

    def graph(self):
        c = self.c
        c.rnd_foz(self.seed)
        if "front" not in self.graphs:
            c.gcvl_graph_begin()
            self._front(True)
            self.graphs["front"] = c.gcvl_graph_end()
            check(c, sync=False)
        c.gcvl_graph_launch(self.graphs["front"])
        c.gcvl_d2h_async(self.host_count, self.count, 4)
        c.gcvl_sync()
        n2 = C.cast(self.host_count, C.POINTER(C.c_int))[0]
        key = ("back", n2)
        if key not in self.graphs:
            c.gcvl_graph_begin()
            self._back(n2)
            self.graphs[key] = c.gcvl_graph_end()
            check(c, sync=False)
        c.gcvl_graph_launch(self.graphs[key])
        c.gcvl_sync()
        return n2

    def _packed_len_host(self):
        nl = np.empty(self.b.m, dtype=np.int32)
        self.c.v2c_fuz(nl.ctypes.data, self.newlens, self.b.m, None)
        return int(nl.sum(dtype=np.int64))

    def results(self, n2: int) -> dict:
        c, b = self.c, self.b
        dt = np.float64 if self.dbl else np.int32
        get = lambda ptr, k, d=dt: self._get(ptr, k, d)  # noqa: E731
        return {"y": get(self.y, b.n), "f": get(self.f, b.n, np.int32), "newlens": get(self.newlens, b.m, np.int32),
                "p": get(self.p, n2), "idx": get(self.idx, n2, np.int32), "g": get(self.g, n2)}

    def _get(self, ptr, k, dt):
        out = np.empty(k, dtype=dt)
        fn = self.c.v2c_fud if dt == np.float64 else self.c.v2c_fuz
        if k:
            fn(out.ctypes.data, ptr, k, None)
        return out

    def timeit(self, mode: str, reps: int = 3) -> float:
        fn = getattr(self, mode)
        fn()  # warm-up (and graph capture)
        ts = []
        for _ in range(reps):
            self.c.gcvl_sync()
            t0 = time.perf_counter()
            fn()
            ts.append(time.perf_counter() - t0)
        return float(np.median(ts))

    def free(self):
        for g in self.graphs.values():
            self.c.gcvl_graph_destroy(g)
        for ptr in (self.x, self.y, self.p, self.g, self.zeros, self.f, self.bnd, self.idx, self.newlens,
                    self.lens, self.sd, self.sd2, self.count, self.work):
            self.c.fre_fov(ptr)
        self.c.gcvl_host_free(self.host_count)
