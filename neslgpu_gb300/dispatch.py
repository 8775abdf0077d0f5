"""Kernel-variant autotuner and the learned dispatcher's training loop.

The library has several kernels for the same segmented scan, reduction or
rank (``gcvl_run_variant``; variants.cu): the default tile kernel with a
decoupled look-back, one CTA per segment (two chunk sizes), one warp per
segment (two chunk sizes) and, for ranks, a per-segment shared-memory rank.
Which one is fastest depends on the segment-length distribution.

* ``autotune`` times every valid variant of one call and returns the
  fastest -- the dispatcher's fallback, and the optimum its regret is
  measured against.
* ``sweep`` builds the training set: seeded synthetic descriptors
  (uniform, geometric, power-law and bimodal length distributions, totals
  log-uniform in [2^lo, 2^hi], int32 / uint32 / float64, scan / reduce /
  rank), the device-computed features of each (``gcvl_seg_features``) and
  the measured time of every valid variant.
* ``train`` fits the FP32 MLP with the library's own CUDA training kernel
  (``gcvl_mlp_train``) on 80 % of the instances and evaluates it with the
  inference kernel (``gcvl_mlp_infer``) on the other 20 %: regret against
  the autotuned optimum and speed-up against plain dispatch (always the
  default kernel).

All timings come from CUDA events on the library stream around the variant
call alone; inputs are device-resident.
"""
from __future__ import annotations

import ctypes as C
import math
import time
from dataclasses import dataclass, field

import numpy as np

from . import workloads as W
from .cvl import CVL, check, load

VARIANTS = ["flat", "cta-2048", "cta-512", "warp-256", "warp-64", "rank-smem"]
PRIM = {("scan", "int32"): "add_sez", ("scan", "uint32"): "add_sez", ("scan", "float64"): "add_sed",
        ("reduce", "int32"): "add_rez", ("reduce", "uint32"): "add_rez", ("reduce", "float64"): "add_red",
        ("rank", "int32"): "rku_lez", ("rank", "uint32"): "rku_lez", ("rank", "float64"): "rku_led"}
DISTS = ["uniform", "geometric", "powerlaw", "bimodal"]


# ----------------------------------------------------------- descriptors --
def lengths_for(r: np.random.Generator, dist: str, n: int, max_m: int) -> np.ndarray:
    """Segment lengths of one synthetic descriptor, summing to n, at most
    max_m segments (the mean is raised when the draw would exceed it)."""
    floor_mean = max(1.0, 1.5 * n / max_m)  # keeps every draw below max_m segments
    if dist == "uniform":
        L = max(2 ** r.uniform(0, 14), floor_mean)
        hi = max(1, int(round(2 * L)) - 1)
        k = int(n / ((1 + hi) / 2) * 1.1) + 16
        lens = r.integers(1, hi + 1, size=k)
    elif dist == "geometric":
        mean = max(2 ** r.uniform(0, 16), floor_mean)
        k = int(n / mean * 1.2) + 16
        lens = r.geometric(min(1.0, 1.0 / mean), size=k)
    elif dist == "powerlaw":
        alpha = r.uniform(1.5, 3.0)
        xmax = 2 ** 20
        k = max(16, int(n / max(floor_mean, 1.0)))
        u = r.random(size=min(k, int(max_m / 1.25)))
        # inverse CDF of a continuous power law on [1, xmax], rounded down
        a1 = 1.0 - alpha
        lens = np.floor((1.0 + u * (xmax ** a1 - 1.0)) ** (1.0 / a1)).astype(np.int64)
        if lens.sum() < n:  # heavy tails may fall short: scale up
            lens = np.maximum(1, np.round(lens * (n / max(1, lens.sum())) + 0.5)).astype(np.int64)
    elif dist == "bimodal":
        big = int(r.integers(1, 17))
        frac = r.uniform(0.3, 0.95)
        n_big = int(n * frac)
        small_mean = max(2.5, floor_mean)
        k_small = int((n - n_big) / small_mean * 1.2) + 16
        small = r.integers(1, 5, size=k_small) if small_mean <= 2.5 else \
            r.geometric(1.0 / small_mean, size=k_small)
        bigs = np.full(big, max(1, n_big // big), dtype=np.int64)
        lens = np.concatenate([bigs, small])
        r.shuffle(lens)
    else:
        raise ValueError(dist)
    lens = np.asarray(lens, dtype=np.int64)
    c = np.cumsum(lens)
    k = int(np.searchsorted(c, n))
    lens = lens[: k + 1].copy()
    if len(lens) == 0:
        lens = np.array([n], dtype=np.int64)
    lens[-1] -= int(lens.sum()) - n  # the cut segment keeps what is left (> 0)
    assert lens.sum() == n and lens.min() >= 0 and len(lens) <= max_m
    return lens.astype(np.int32)


@dataclass
class Instance:
    dist: str
    kind: str
    dtype: str
    n: int
    m: int
    max_len: int
    prim: str
    times: np.ndarray = field(default_factory=lambda: np.full(len(VARIANTS), np.inf))
    feat: np.ndarray | None = None

    @property
    def valid(self):
        return np.isfinite(self.times)

    @property
    def best(self):
        return int(np.argmin(self.times))


# ------------------------------------------------------------- timing -----
class Bench:
    """Device buffers sized for the largest instance, reused for all."""

    def __init__(self, max_n: int, max_m: int, cvl: CVL | None = None):
        self.c = c = cvl or load()
        self.max_n, self.max_m = max_n, max_m
        al = lambda u: self._alloc(u)  # noqa: E731
        self.x = al(c.siz_fod(max_n))
        self.d = al(c.siz_fod(max_n))
        self.lens = al(c.siz_foz(max_m))
        self.sd = al(c.siz_fos(max_n, max_m))
        scr = 0
        for prim in set(PRIM.values()):
            scr = max(scr, c.gcvl_variant_scratch(prim.encode(), max_n, max_m))
        self.scr = al(max(scr, c.mke_fov_scratch(max_n, max_m)))
        self.ev = [c.gcvl_event_create() for _ in range(2)]
        c.gcvl_fill_random(self.x, max_n, 1, 7, 0.0, 0)  # float64 N(0,1); ints reuse the bits
        check(c)

    def _alloc(self, units):
        p = self.c.alo_foz(int(max(units, 1)))
        if not p:
            raise MemoryError(self.c.gcvl_error_string().decode())
        return p

    def set_descriptor(self, lens: np.ndarray):
        c = self.c
        m = len(lens)
        n = int(lens.sum(dtype=np.int64))
        c.c2v_fuz(self.lens, lens.ctypes.data, m, None)
        c.mke_fov(self.sd, self.lens, n, m, self.scr)
        return n, m

    def fill(self, dtype: str, n: int, seed: int):
        kind = {"int32": 3, "uint32": 0, "float64": 1}[dtype]
        self.c.gcvl_fill_random(self.x, n, kind, seed, 0.0, 2001)

    def time_variant(self, prim: str, v: int, n: int, m: int, reps: int = 3, limit_ms: float | None = None):
        c = self.c
        p = prim.encode()
        t = []
        for i in range(reps + 1):
            c.gcvl_event_record(self.ev[0])
            rc = c.gcvl_run_variant(p, v, self.d, self.x, self.sd, n, m, self.scr)
            c.gcvl_event_record(self.ev[1])
            ms = c.gcvl_event_elapsed_ms(self.ev[0], self.ev[1])
            if rc:
                check(c)
            if i > 0:
                t.append(ms)
            elif limit_ms is not None and ms > limit_ms:
                return ms  # far off the pace: one run is enough to rank it last
        return float(np.median(t))

    def free(self):
        for p in (self.x, self.d, self.lens, self.sd, self.scr):
            self.c.fre_fov(p)
        for e in self.ev:
            self.c.gcvl_event_destroy(e)


def autotune(bench: Bench, prim: str, n: int, m: int, max_len: int, reps: int = 3) -> np.ndarray:
    """Times of every variant of prim on the current descriptor (inf where
    the variant is not valid).  The default kernel is timed first; a variant
    more than 20x slower after one run is not run again."""
    c = bench.c
    t = np.full(len(VARIANTS), np.inf)
    t[0] = bench.time_variant(prim, 0, n, m, reps)
    for v in range(1, len(VARIANTS)):
        if c.gcvl_variant_valid(prim.encode(), v, max_len):
            t[v] = bench.time_variant(prim, v, n, m, reps, limit_ms=20 * t[0] + 0.05)
    return t


def sweep(count: int, seed: int = 2024, lo: int = 16, hi: int = 28, max_m: int = 1 << 22,
          reps: int = 3, cvl: CVL | None = None, log=None, workers: int = 8) -> tuple[list[Instance], np.ndarray]:
    """count instances; returns them and X (count x 24 float32 features and
    validity masks, computed on the device).  Segment lengths are drawn on
    host threads ahead of the GPU timing (each instance has its own seeded
    generator, so the set does not depend on the thread count)."""
    from concurrent.futures import ThreadPoolExecutor

    c = cvl or load()
    r = W.rng(seed)
    specs = []
    for i in range(count):
        dist = DISTS[int(r.integers(0, len(DISTS)))]
        kind = ["scan", "reduce", "rank"][int(r.integers(0, 3))]
        dtype = ["int32", "uint32", "float64"][int(r.integers(0, 3))]
        n = int(2 ** r.uniform(lo, hi))
        specs.append((dist, kind, dtype, n))

    def gen(i):
        dist, _, _, n = specs[i]
        return lengths_for(W.rng(seed * 100_003 + i), dist, n, max_m)

    bench = Bench(1 << hi, max_m, cvl=c)
    stride = c.gcvl_mlp_feature_stride()
    fx = c.alo_foz(max(1, count * stride // 2 + 1))
    insts = []
    t0 = time.time()
    pool = ThreadPoolExecutor(max_workers=workers)
    try:
        ahead = 2 * workers
        futs = {i: pool.submit(gen, i) for i in range(min(ahead, count))}
        for i in range(count):
            lens = futs.pop(i).result()
            if i + ahead < count:
                futs[i + ahead] = pool.submit(gen, i + ahead)
            dist, kind, dtype, _ = specs[i]
            n, m = bench.set_descriptor(lens)
            prim = PRIM[(kind, dtype)]
            bench.fill(dtype, n, seed + i)
            c.gcvl_seg_features(prim.encode(), bench.sd, n, m, fx + i * stride * 4)
            inst = Instance(dist, kind, dtype, n, m, int(lens.max()), prim)
            inst.times = autotune(bench, prim, n, m, inst.max_len, reps)
            insts.append(inst)
            if log and (i + 1) % 256 == 0:
                log(f"sweep {i + 1}/{count} ({time.time() - t0:.0f} s)")
        X = np.empty(count * stride, dtype=np.float32)
        c.v2c_fuz(X.ctypes.data, fx, count * stride, None)  # 4-byte words
        check(c)
    finally:
        pool.shutdown(wait=True, cancel_futures=True)
        bench.free()
        c.fre_fov(fx)
    X = X.reshape(count, stride)
    for i, inst in enumerate(insts):
        inst.feat = X[i]
    return insts, X


# ------------------------------------------------------------- training ---
def soft_targets(times: np.ndarray, tau: float = 0.05) -> np.ndarray:
    """Probability over the variants: exp(-(t/t_best - 1)/tau) over the
    valid ones, normalised -- near-ties share the mass."""
    T = np.zeros((len(times), 8), dtype=np.float32)
    for i, t in enumerate(times):
        ok = np.isfinite(t)
        rel = np.where(ok, t / t[ok].min() - 1.0, np.inf)
        w = np.where(ok, np.exp(-rel / tau), 0.0)
        T[i, : len(t)] = w / w.sum()
    return T


def init_params(c: CVL, seed: int) -> np.ndarray:
    """He-initialised weights, zero biases, in the kernel's layout
    (W1 16x64, b1, W2 64x64, b2, W3 64x8, b3)."""
    r = np.random.default_rng(seed)
    F, H, K = 16, 64, 8
    parts = [r.normal(0, math.sqrt(2 / F), F * H), np.zeros(H), r.normal(0, math.sqrt(2 / H), H * H),
             np.zeros(H), r.normal(0, math.sqrt(1 / H), H * K), np.zeros(K)]
    p = np.concatenate(parts).astype(np.float32)
    assert p.size == c.gcvl_mlp_param_count()
    return p


class DevF32:
    """A float32 array in the library's device heap."""

    def __init__(self, c: CVL, arr: np.ndarray | None = None, size: int | None = None):
        self.c = c
        self.size = int(arr.size if arr is not None else size)
        self.ptr = c.alo_foz(max(1, (self.size + 1) // 2))
        if arr is not None and self.size:
            a = np.ascontiguousarray(arr, dtype=np.float32)
            c.c2v_fuz(self.ptr, a.ctypes.data, self.size, None)

    def get(self, dtype=np.float32) -> np.ndarray:
        out = np.empty(self.size, dtype=dtype)
        if self.size:
            self.c.v2c_fuz(out.ctypes.data, self.ptr, self.size, None)
        return out

    def free(self):
        self.c.fre_fov(self.ptr)


def split(count: int, seed: int, frac: float = 0.8):
    idx = np.random.default_rng(seed).permutation(count)
    k = int(round(frac * count))
    return idx[:k], idx[k:]


def train(insts: list[Instance], X: np.ndarray, seed: int = 7, epochs: int = 400, batch: int = 128,
          lr: float = 3e-3, cvl: CVL | None = None) -> dict:
    c = cvl or load()
    times = np.stack([i.times for i in insts])
    tr, te = split(len(insts), seed)
    T = soft_targets(times)
    params = DevF32(c, init_params(c, seed))
    moments = DevF32(c, np.zeros(2 * params.size, dtype=np.float32))
    Xtr, Ttr = DevF32(c, X[tr]), DevF32(c, T[tr])
    Xte = DevF32(c, X[te])
    loss = DevF32(c, size=epochs)
    cls = DevF32(c, size=len(te))
    try:
        t0 = time.perf_counter()
        c.gcvl_mlp_train(params.ptr, moments.ptr, Xtr.ptr, Ttr.ptr, len(tr), epochs, batch, lr, seed, 0, loss.ptr)
        check(c)
        train_s = time.perf_counter() - t0
        c.gcvl_mlp_infer(params.ptr, Xte.ptr, len(te), cls.ptr)
        check(c)
        choice = cls.get(np.int32)
        # the training set's own fit
        cls_tr = DevF32(c, size=len(tr))
        c.gcvl_mlp_infer(params.ptr, Xtr.ptr, len(tr), cls_tr.ptr)
        check(c)
        choice_tr = cls_tr.get(np.int32)
        cls_tr.free()
        p = params.get()
        losses = loss.get()
    finally:
        for a in (params, moments, Xtr, Ttr, Xte, loss, cls):
            a.free()
    return {"params": p, "test": te, "train": tr, "choice": choice, "choice_train": choice_tr,
            "loss_first": float(losses[0]), "loss_last": float(losses[-1]), "train_seconds": train_s,
            **evaluate(times[te], choice)}


def evaluate(times: np.ndarray, choice: np.ndarray) -> dict:
    """Regret of the choices against the autotuned optimum and speed-up of
    dispatch against always running the default kernel."""
    n = len(times)
    best = times.min(axis=1)
    picked = times[np.arange(n), choice]
    flat = times[:, 0]
    assert np.all(np.isfinite(picked)), "a choice fell on an invalid variant"
    return {
        "instances": int(n),
        "regret_mean": float(np.mean(picked / best - 1.0)),
        "regret_p90": float(np.quantile(picked / best - 1.0, 0.9)),
        "regret_total": float(picked.sum() / best.sum() - 1.0),
        "accuracy": float(np.mean(choice == times.argmin(axis=1))),
        "speedup_vs_plain": float(flat.sum() / picked.sum()),
        "speedup_autotuned_vs_plain": float(flat.sum() / best.sum()),
        "speedup_vs_plain_geomean": float(np.exp(np.mean(np.log(flat / picked)))),
    }


def choice_counts(insts: list[Instance]) -> dict:
    out = {}
    for i in insts:
        k = f"{i.kind}/{i.dist}"
        out.setdefault(k, [0] * len(VARIANTS))
        out[k][i.best] += 1
    return out


def dispatch_overhead_ms(c: CVL, params: np.ndarray, reps: int = 20) -> float:
    """Host-side cost of one uncached dispatch decision (features, inference,
    read-back) on a mid-sized descriptor."""
    lens = np.full(1 << 14, 64, dtype=np.int32)
    n, m = int(lens.sum()), len(lens)
    lv = c.alo_foz(c.siz_foz(m))
    sd = c.alo_foz(c.siz_fos(n, m))
    scr = c.alo_foz(c.mke_fov_scratch(n, m))
    c.c2v_fuz(lv, lens.ctypes.data, m, None)
    c.mke_fov(sd, lv, n, m, scr)
    c.gcvl_dispatch_set_model(params.ctypes.data)
    ts = []
    for _ in range(reps):
        c.gcvl_dispatch_set_model(params.ctypes.data)  # clears the cache
        c.gcvl_sync()
        t0 = time.perf_counter()
        c.gcvl_dispatch_choice(b"add_sez", sd, n, m)
        ts.append((time.perf_counter() - t0) * 1e3)
    c.gcvl_dispatch_set_model(None)
    for p in (lv, sd, scr):
        c.fre_fov(p)
    check(c)
    return float(np.median(ts))
