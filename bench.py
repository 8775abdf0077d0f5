#!/usr/bin/env python3
"""Benchmark of the GB300 CVL library on the segmented float64 workload.

Workload (one step): the segmented exclusive +-scan (add_sed) and the
segmented +-reduce (add_red) of 2^28 float64 N(0,1) values whose segment
lengths are round(LogNormal(mu=5, sigma=2)) clipped to [1, 2^24] -- the
primitive part of the "plain GPU drop-in at scale" configuration.  Each step
processes 2 x 2^28 elements; value = elements / second (Gelem/s).

Printed as one JSON line (rank 0).  Besides the headline it carries:
  roofline     -- the add_sed scan kernel: algorithmic bytes per launch
                  (16 B/element + 4 B/segment) / its CUDA-event time, against
                  the measured HBM copy bandwidth of MEASURED_PEAKS.json
  e2e          -- the same step through the C ABI with pinned host buffers,
                  every step uploading the values and downloading both
                  results: the vector cut at segment starts into 8 pieces,
                  pipelined on three streams (uploads, kernels, downloads)
                  so that transfers in both directions and kernels overlap
                  ("sequential": whole-vector c2v_fud, both primitives,
                  v2c_fud x2)
  cpu_baseline -- the CPU oracle (plain-C restatement of the serial CVL)
                  on one host core over the same workload
  parity       -- the timed GPU results against that CPU run under the
                  float64 rule |gpu - cpu| <= 1e-12 * max(|cpu|, S)
  primitives   -- Gelem/s and roofline fraction of the other CVL primitives
                  at 2^28 elements (int32 unless named)
  clocks       -- SM clock and throttle reasons sampled (NVML, every
                  millisecond) during the timed region

``--impl reference`` times the CPU implementation of the same step (the
oracle restatement of the serial CVL; the reference sources are not on this
machine) on all host cores, splitting the segments across threads.

Multi-GPU: the workload does not exchange data between GPUs, so N GPUs run
N independent replicas (one process per GPU under torchrun); value is the
total over replicas divided by the slowest replica's time.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

LOG2N = 28
SEED = 0x5EED + 1
METRIC = "CVL primitive Gelem/s (segmented +_scan and +_reduce, float64)"
NCU_SCAN_DRAM_BYTES_PER_ELEM = 488.69e6 / (1 << 25)  # add_sed's DRAM traffic per element, ncu at 2^25
UNIT = "Gelem/s"


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def segment_lengths(n):
    from neslgpu_gb300 import workloads as W
    return W.lognormal_lengths(W.rng(SEED), n, 5.0, 2.0, 1 << 24)


class Clocks:
    """SM clock and throttle reasons sampled during the timed region.

    NVML (libnvidia-ml, read-only queries) is polled every millisecond from a
    thread, so that a timed region of a few tens of milliseconds still holds
    tens of samples; where NVML cannot be loaded, nvidia-smi's own 100 ms
    loop stands in."""

    Q = ("timestamp,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")
    # nvmlClocksEventReason* bits (nvml.h)
    REASONS = {0x8: "hw_slowdown", 0x40: "hw_thermal_slowdown", 0x20: "sw_thermal_slowdown",
               0x4: "sw_power_cap"}

    def __init__(self, device, period_s=0.001):
        self.device = device
        self.period = period_s
        self.proc = None
        self.thread = None
        self.samples = []  # (host time, sm MHz, max MHz, reason bits)

    def _nvml(self):
        try:
            nv = C.CDLL("libnvidia-ml.so.1")
        except OSError:
            return None
        if nv.nvmlInit_v2() != 0:
            return None
        count = C.c_uint(0)
        if nv.nvmlDeviceGetCount_v2(C.byref(count)) != 0 or count.value == 0:
            return None
        h = C.c_void_p()
        idx = self.device if count.value > self.device else 0
        if nv.nvmlDeviceGetHandleByIndex_v2(C.c_uint(idx), C.byref(h)) != 0:
            return None
        return nv, h

    def _poll(self, nv, h):
        clk, mx, rs = C.c_uint(0), C.c_uint(0), C.c_ulonglong(0)
        nv.nvmlDeviceGetMaxClockInfo(h, 1, C.byref(mx))  # NVML_CLOCK_SM
        get_reasons = getattr(nv, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            nv.nvmlDeviceGetCurrentClocksThrottleReasons
        while not self.stop:
            t = time.time()
            if nv.nvmlDeviceGetClockInfo(h, 1, C.byref(clk)) == 0 and get_reasons(h, C.byref(rs)) == 0:
                self.samples.append((t, float(clk.value), float(mx.value), int(rs.value)))
            time.sleep(self.period)

    def __enter__(self):
        self.stop = False
        got = self._nvml()
        if got is not None:
            self.thread = threading.Thread(target=self._poll, args=got, daemon=True)
            self.thread.start()
            return self
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.stop = True
        if self.thread:
            self.thread.join(timeout=5)
        self.out = ""
        if self.proc:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.out, _ = self.proc.communicate()

    def _smi_samples(self):
        import datetime as dt
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        bits = {v: k for k, v in self.REASONS.items()}
        for line in (getattr(self, "out", "") or "").splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 8:
                continue
            try:
                ts = dt.datetime.strptime(f[0], "%Y/%m/%d %H:%M:%S.%f").timestamp()
                clk, cmax = float(f[1]), float(f[2])
            except ValueError:
                continue
            rs = sum(bits[nm] for nm, v in zip(names, f[4:8]) if v.lower() == "active")
            yield ts, clk, cmax, rs

    def summary(self, t0=None, t1=None):
        """Median SM clock and active throttle reasons over the samples whose
        timestamps fall inside [t0, t1] (host wall-clock seconds)."""
        samples = self.samples if self.thread else list(self._smi_samples())
        sm, mx, reasons = [], 0.0, set()
        for ts, clk, cmax, rs in samples:
            if t0 is not None and not (t0 - 0.002 <= ts <= t1 + 0.002):
                continue
            sm.append(clk)
            mx = max(mx, cmax)
            reasons.update(nm for b, nm in self.REASONS.items() if rs & b)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples_in_window": len(sm), "samples": len(samples),
                "source": "nvml, 1 ms" if self.thread else "nvidia-smi, 100 ms"}


def sum_err_over_tol(got, want, x, lens, kind, chunk=1 << 24):
    """max |got - want| / (1e-12 * max(|want|, S)) over a segmented float64
    +-scan (S = sum of |x| before the element in its segment) or
    +-reduction (S = sum of |x| over the segment), over groups of whole
    segments of about `chunk` elements."""
    lens = np.asarray(lens, dtype=np.int64)
    ends = np.cumsum(lens)
    starts = ends - lens
    worst, a, m = 0.0, 0, len(lens)
    while a < m:
        b = min(m, max(a + 1, int(np.searchsorted(ends, starts[a] + chunk, side="right"))))
        e0, e1 = int(starts[a]), int(ends[b - 1])
        ln = lens[a:b]
        ax = np.abs(x[e0:e1])
        cs = np.concatenate([[0.0], np.cumsum(ax)])
        ls = np.cumsum(ln) - ln
        if kind == "scan":
            S = cs[np.arange(e1 - e0)] - cs[np.repeat(ls, ln)]
            g, w = got[e0:e1], want[e0:e1]
        else:
            S = cs[ls + ln] - cs[ls]
            g, w = got[a:b], want[a:b]
        if len(w):
            tol = 1e-12 * np.maximum(np.abs(w), S) + 1e-300
            same = (g == w) | (np.isnan(g) & np.isnan(w))
            worst = max(worst, float(np.max(np.where(same, 0.0, np.abs(g - w) / tol))))
        a = b
    return worst


def dist():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as td
        td.init_process_group("gloo")
        pg = td
    return world, rank, local, pg


def allmax(pg, v):
    if pg is None:
        return v
    import torch
    t = torch.tensor([float(v)], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def barrier(pg):
    if pg is not None:
        pg.barrier()


# ------------------------------------------------------------ GPU arm ---
class Gpu:
    def __init__(self):
        from neslgpu_gb300.cvl import load, check
        self.c = load()
        self.check = check

    def alloc(self, units):
        p = self.c.alo_foz(int(units))
        if not p:
            raise RuntimeError(self.c.gcvl_error_string().decode())
        return p

    def events(self, k):
        return [self.c.gcvl_event_create() for _ in range(k)]

    def ms(self, a, b):
        return self.c.gcvl_event_elapsed_ms(a, b)


def timed(g, fn, reps=10):
    """Median CUDA-event time (ms) of fn() after one warm-up call."""
    fn()
    e = g.events(2)
    ts = []
    for _ in range(reps):
        g.c.gcvl_event_record(e[0])
        fn()
        g.c.gcvl_event_record(e[1])
        ts.append(g.ms(e[0], e[1]))
    return statistics.median(ts)


def primitive_suite(g, n, hbm, only=None):
    """Gelem/s and roofline fraction of the other CVL primitives at n.
    only: names to run (a name is an entry's first word, e.g. "rku_luz")."""
    from neslgpu_gb300 import workloads as W
    c = g.c
    out = {}
    xi, yi, dz = g.alloc(c.siz_foz(n)), g.alloc(c.siz_foz(n)), g.alloc(c.siz_foz(n))
    fl, ix = g.alloc(c.siz_foz(n)), g.alloc(c.siz_foz(n))
    c.gcvl_fill_random(xi, n, 0, 11, 0.0, 0)
    c.gcvl_fill_random(yi, n, 0, 12, 0.0, 0)
    c.gcvl_fill_random(fl, n, 2, 13, 0.5, 0)
    lens = W.geometric_lengths(W.rng(SEED), n, 64).astype(np.int32)
    m = len(lens)
    lv = g.alloc(c.siz_foz(m))
    c.c2v_fuz(lv, lens.ctypes.data, m, None)
    sd = g.alloc(c.siz_fos(n, m))
    scr = g.alloc(max(c.mke_fov_scratch(n, m), c.add_sez_scratch(n, m), c.max_rez_scratch(n, m),
                      c.pk2_luz_scratch(n), c.rku_luz_scratch(n), c.rku_lez_scratch(n, m),
                      c.pk1_lev_scratch(n, m)))
    c.mke_fov(sd, lv, n, m, scr)
    # a uniform random permutation: the rank of uniform random keys
    c.rku_luz(ix, yi, n, scr)
    red = g.alloc(c.siz_foz(m))
    cnt = c.pk1_luv(fl, n, scr)
    # indices local to each segment for the segmented gather: rank of random
    # keys within segments (a random permutation of every segment)
    ix_seg = g.alloc(c.siz_foz(n))
    c.rku_lez(ix_seg, yi, sd, n, m, scr)

    def wanted(name):
        return only is None or name.split(" ")[0] in only

    # the set-up above leaves the GPU idle for seconds of host work: bring it
    # back to speed (about 100 ms of streaming) before the first timing
    for _ in range(200):
        c.add_wuz(dz, xi, yi, n, None)
    c.gcvl_sync()

    def rec(name, fn, bytes_per_elem, extra=0.0):
        if not wanted(name):
            return
        t = timed(g, fn)
        gb = (bytes_per_elem * n + extra) / (t * 1e-3) / 1e9
        out[name] = {"gelem_s": round(n / (t * 1e-3) / 1e9, 2), "ms": round(t, 4),
                     "achieved_gbs": round(gb, 1), "frac": round(gb / hbm, 3)}

    rec("add_sez", lambda: c.add_sez(dz, xi, sd, n, m, scr), 8, 4.0 * m)
    rec("add_sez+add_wuz (inclusive)", lambda: (c.add_sez(dz, xi, sd, n, m, scr),
                                                c.add_wuz(dz, dz, xi, n, None)), 20, 4.0 * m)
    rec("max_rez", lambda: c.max_rez(red, xi, sd, n, m, scr), 4, 8.0 * m)
    rec("pk1_lev+pk2_lez (pack)", lambda: (c.pk1_lev(red, fl, sd, n, m, scr),
                                           c.pk2_lez(dz, xi, fl, sd, n, m, sd, cnt, m, scr)), 8, 4.0 * cnt + 8.0 * m)
    rec("pk1_lev", lambda: c.pk1_lev(red, fl, sd, n, m, scr), 4, 8.0 * m)
    rec("pk2_lez", lambda: c.pk2_lez(dz, xi, fl, sd, n, m, sd, cnt, m, scr), 8, 4.0 * cnt)
    rec("dis_vez", lambda: c.dis_vez(dz, red, sd, n, m, None), 4, 8.0 * m)
    rec("bck_pez (segmented gather)", lambda: c.bck_pez(dz, xi, ix_seg, sd, n, m, sd, n, m, None), 12, 8.0 * m)
    rec("smp_puz (permute)", lambda: c.smp_puz(dz, xi, ix, n, None), 12)
    rec("bck_puz (back-permute)", lambda: c.bck_puz(dz, xi, ix, n, n, None), 12)
    rec("add_wuz", lambda: c.add_wuz(dz, xi, yi, n, None), 12)
    t = timed(g, lambda: c.rku_luz(dz, xi, n, scr), reps=3) if wanted("rku_luz") else None
    # declared pass traffic of this design above 2^23 elements: histograms 4,
    # first pass 4 + 8, two middle passes 16 each, last pass 8 + 8 (index,
    # position pairs written grouped by output window), window scatter 8 + 4
    io, passes = 8.0, 76.0
    if t is not None:
        out["rku_luz (rank)"] = {"gelem_s": round(n / (t * 1e-3) / 1e9, 2), "ms": round(t, 4),
                                 "achieved_gbs_io_floor": round(io * n / (t * 1e-3) / 1e9, 1),
                                 "frac_io_floor": round(io * n / (t * 1e-3) / 1e9 / hbm, 3),
                                 "frac_pass_traffic_76B": round(passes * n / (t * 1e-3) / 1e9 / hbm, 3)}
    g.check(c)
    for p in (xi, yi, dz, fl, ix, ix_seg, lv, sd, scr, red):
        c.fre_fov(p)
    return out


def batched_suite(g, nvec=8192, total=1 << 27, seed=3):
    """The batched workload: nvec segmented vectors of log-normal lengths in
    [10, 10^6] (about `total` elements), half int32 and half float64, each
    running +_scan, PACK by x > 0 and a random in-segment gather; per-vector
    call loop against the flattened sequence and its CUDA-graph replay.
    Wall-clock times of whole synchronised runs (the per-call loop reads a
    count back to the host per vector)."""
    from neslgpu_gb300 import batch as B
    res = {"vectors": nvec, "elements": 0, "percall_ms": 0.0, "batched_ms": 0.0, "graph_ms": 0.0}
    for half, dbl in ((0, False), (1, True)):
        b = B.make_batch(nvec // 2, total // 2, seed=seed + half)
        run = B.BatchRun(b, dbl, cvl=g.c)
        try:
            for mode in ("percall", "batched", "graph"):
                res[f"{mode}_ms"] += run.timeit(mode, reps=3 if mode == "percall" else 10) * 1e3
            res["elements"] += b.n
        finally:
            run.free()
    for k in ("percall_ms", "batched_ms", "graph_ms"):
        res[k] = round(res[k], 3)
    res["graph_gelem_s"] = round(res["elements"] / (res["graph_ms"] * 1e-3) / 1e9, 2)
    res["speedup_batched_vs_percall"] = round(res["percall_ms"] / res["batched_ms"], 2)
    res["speedup_graph_vs_percall"] = round(res["percall_ms"] / res["graph_ms"], 2)
    res["skewed"] = skewed_batch_suite(g)
    return res


def skewed_batch_suite(g):
    """Flattening's worst case: 4 vectors of 2^24 elements beside 8188 of
    1-100 elements, against one vector of the same total length (the same
    bytes with no vector boundaries: the bound for any launch scheme,
    a persistent (vector, op) queue included).  int32 and float64."""
    from neslgpu_gb300 import batch as B
    out = {}
    for dbl in (False, True):
        sk = B.make_skewed_batch()
        row = {"vectors": sk.nvec, "elements": sk.n}
        for name, b, modes in (("skewed", sk, ("percall", "batched", "graph")),
                               ("one_vector", B.single_vector_batch(sk.n), ("batched", "graph"))):
            run = B.BatchRun(b, dbl, cvl=g.c)
            try:
                for mode in modes:
                    row[f"{name}_{mode}_ms"] = round(run.timeit(mode, reps=3 if mode == "percall" else 10) * 1e3, 3)
            finally:
                run.free()
        row["batched_vs_one_vector"] = round(row["skewed_batched_ms"] / row["one_vector_batched_ms"], 3)
        row["graph_vs_one_vector"] = round(row["skewed_graph_ms"] / row["one_vector_graph_ms"], 3)
        out["float64" if dbl else "int32"] = row
    return out


def dispatch_suite(g, count=512, hi=24, seed=2024):
    """The learned dispatcher on a seeded sweep of synthetic descriptors
    (uniform / geometric / power-law / bimodal lengths, totals 2^16..2^hi,
    int32 / uint32 / float64, segmented scan / reduce / rank): every valid
    kernel variant timed, the MLP trained on 80 % with the library's CUDA
    training kernel, its picks on the other 20 % scored against the
    autotuned optimum (regret) and against always running the default
    kernel (speed-up)."""
    from neslgpu_gb300 import dispatch as D
    t0 = time.time()
    insts, X = D.sweep(count, seed=seed, lo=16, hi=hi, cvl=g.c)
    res = D.train(insts, X, seed=7, epochs=400, batch=128, cvl=g.c)
    out = {"instances": count, "log2_total_range": [16, hi], "test_instances": res["instances"]}
    for k in ("regret_mean", "regret_p90", "regret_total", "accuracy", "speedup_vs_plain",
              "speedup_autotuned_vs_plain", "speedup_vs_plain_geomean", "train_seconds"):
        out[k] = round(res[k], 4)
    out["decision_overhead_ms"] = round(D.dispatch_overhead_ms(g.c, res["params"]), 4)
    out["wall_seconds"] = round(time.time() - t0, 1)
    return out


def _vcode_sort(cvl, keys, sync, fused=None):
    """QSORT through the VCODE interpreter: (seconds with the keys on the
    device, seconds end to end from host keys to host result, sorted keys,
    VCODE ops run).  fused: a FusedLib, to run the .fcode form instead."""
    from neslgpu_gb300 import vcode as V, vcode_programs as P
    text = P.qsort_fcode_program()[0] if fused is not None else P.qsort_program()
    it = V.Interpreter(text, cvl, sync=sync, fused=fused)
    try:
        t0 = time.perf_counter()
        lv = it.from_host("I", [len(keys)])
        sd = it.segdes_from_lengths(lv)
        it.drop(lv)
        kv = it.from_host("I", keys)
        sync()
        t1 = time.perf_counter()
        st = it.run("QSORT", [sd, kv])
        sync()
        t2 = time.perf_counter()
        out = it.to_host(st[-1])
        t3 = time.perf_counter()
        return t2 - t1, t3 - t0, out, it.ops_run
    finally:
        it.free_all()


def graph_suite(c, sync, seed=7):
    """VCODE basic blocks as CUDA graphs (vcode.Interpreter(graphs=True))
    against plain launches, on programs that run again in the same state:
    the same quicksort repeated (2^12 to 2^18 keys, where the interpreter's
    and the launches' host time is a large part) and the SpMV program
    repeated (2^14 and 2^22 rows).  Seconds per run: the median of the runs
    after four warm-up runs (by then the heap has settled and every block
    replays); results must equal the plain runs'."""
    from neslgpu_gb300 import vcode as V, vcode_programs as P
    r = np.random.default_rng(seed)
    out = {}

    def timed_runs(fn, reps):
        ts, res = [], None
        for _ in range(reps):
            sync()
            t0 = time.perf_counter()
            res = fn()
            sync()
            ts.append(time.perf_counter() - t0)
        return float(np.median(ts[4:])), res

    for lg in (12, 16, 18):
        keys = r.integers(-2 ** 31, 2 ** 31, size=1 << lg, dtype=np.int64).astype(np.int32)
        row = {}
        for mode in (False, True):
            it = V.Interpreter(P.qsort_program(), c, sync=sync, graphs=mode)

            def one():
                lv = it.from_host("I", [len(keys)])
                sd = it.segdes_from_lengths(lv)
                it.drop(lv)
                st = it.run("QSORT", [sd, it.from_host("I", keys)])
                res = it.to_host(st[-1])
                for v in st:
                    it.drop(v)
                return res
            try:
                t, res = timed_runs(one, 10)
                row["graph" if mode else "plain"] = {"seconds": round(t, 6), "sorted": bool(np.array_equal(res, np.sort(keys)))}
                if mode:
                    row["graph"]["stats"] = dict(it.graph_stats)
            finally:
                it.free_all()
        row["speedup"] = round(row["plain"]["seconds"] / row["graph"]["seconds"], 3)
        out[f"quicksort_2e{lg}"] = row
    for lg in (14, 22):
        rows = 1 << lg
        lens = np.minimum(r.zipf(2.1, size=rows), 1 << 16).astype(np.int32)
        nnz = int(lens.sum(dtype=np.int64))
        cols = r.integers(0, rows, size=nnz).astype(np.int32)
        vals = r.standard_normal(nnz)
        x = r.standard_normal(rows)
        row, ys = {}, {}
        for mode in (False, True):
            it = V.Interpreter(P.spmv_program(), c, sync=sync, graphs=mode)
            try:
                lv = it.from_host("I", lens)
                rsd = it.segdes_from_lengths(lv)
                it.drop(lv)
                args = [rsd, it.from_host("I", cols), it.from_host("F", vals), it.from_host("F", x)]

                def one():
                    for a in args:
                        a.ref += 1  # the inputs stay across runs
                    st = it.run("SPMV", list(args))
                    y = it.to_host(st[0])
                    it.drop(st[0])
                    return y
                t, ys[mode] = timed_runs(one, 12)
                row["graph" if mode else "plain"] = {"seconds": round(t, 6)}
                if mode:
                    row["graph"]["stats"] = dict(it.graph_stats)
                for a in args:
                    it.drop(a)
            finally:
                it.free_all()
        row["same_result"] = bool(np.array_equal(ys[False].view(np.int64), ys[True].view(np.int64)))
        row["speedup"] = round(row["plain"]["seconds"] / row["graph"]["seconds"], 3)
        out[f"spmv_2e{lg}_rows"] = row
    return out


def _spmv_case(g, rows, r, sync):
    """CSR SpMV through the VCODE program and through the fused kernel on
    `rows` rows with power-law row lengths (alpha 2.1 on [1, 2^16]), column
    indices uniform, float64 N(0,1) values and x."""
    from neslgpu_gb300 import vcode as V, vcode_programs as P
    c = g.c
    lens = np.minimum(r.zipf(2.1, size=rows), 1 << 16).astype(np.int32)
    nnz = int(lens.sum(dtype=np.int64))
    cols = r.integers(0, rows, size=nnz).astype(np.int32)
    vals = r.standard_normal(nnz)
    x = r.standard_normal(rows)
    it = V.Interpreter(P.spmv_program(), c, sync=sync)
    try:
        lv = it.from_host("I", lens)
        rsd = it.segdes_from_lengths(lv)
        it.drop(lv)
        args = [rsd, it.from_host("I", cols), it.from_host("F", vals), it.from_host("F", x)]
        times = []
        for rep in range(4):
            for a in args:
                a.ref += 1  # keep the inputs across runs
            sync()
            t0 = time.perf_counter()
            st = it.run("SPMV", list(args))
            sync()
            times.append(time.perf_counter() - t0)
            y = st[0]
            if rep < 3:
                it.drop(y)
        yh = it.to_host(y)
        it.drop(y)
        for a in args:
            it.drop(a)
    finally:
        it.free_all()
    # the same product by the fused kernel (one launch, no intermediates)
    lv_d = g.alloc(c.siz_foz(rows))
    c.c2v_fuz(lv_d, lens.ctypes.data, rows, None)
    sd_d = g.alloc(c.siz_fos(nnz, rows))
    scr = g.alloc(max(c.mke_fov_scratch(nnz, rows), c.gcvl_spmv_csr_scratch(nnz, rows)))
    c.mke_fov(sd_d, lv_d, nnz, rows, scr)
    cols_d, vals_d, x_d, y_d = g.alloc(c.siz_foz(nnz)), g.alloc(c.siz_fod(nnz)), g.alloc(c.siz_fod(rows)), \
        g.alloc(c.siz_fod(rows))
    c.c2v_fuz(cols_d, cols.ctypes.data, nnz, None)
    c.c2v_fud(vals_d, vals.ctypes.data, nnz, None)
    c.c2v_fud(x_d, x.ctypes.data, rows, None)
    ev = g.events(2)
    ft = []
    for rep in range(6):
        c.gcvl_event_record(ev[0])
        c.gcvl_spmv_csr(y_d, vals_d, cols_d, x_d, sd_d, nnz, rows, scr)
        c.gcvl_event_record(ev[1])
        ft.append(g.ms(ev[0], ev[1]) * 1e-3)
    yf = np.empty(rows)
    c.v2c_fud(yf.ctypes.data, y_d, rows, None)
    g.check(c)
    for p in (lv_d, sd_d, scr, cols_d, vals_d, x_d, y_d):
        c.fre_fov(p)
    tf = float(np.median(ft[1:]))
    starts = np.cumsum(lens, dtype=np.int64) - lens
    chk = np.array([np.dot(vals[s:s + l], x[cols[s:s + l]]) for s, l in zip(starts[:2000], lens[:2000])])
    t = float(np.median(times[1:]))
    spmv = {"rows": rows, "nnz": nnz, "row_nnz": "power law alpha 2.1 on [1, 2^16]", "seconds": round(t, 5),
            "gflop_s": round(2 * nnz / t / 1e9, 2),
            "alg_gbs": round((nnz * (4 + 8 + 8) + 8 * rows + 4 * rows) / t / 1e9, 1),
            "first_rows_max_abs_err": float(np.max(np.abs(yh[:2000] - chk))),
            "fused": {"kernel": "gcvl_spmv_csr", "seconds": round(tf, 6), "gflop_s": round(2 * nnz / tf / 1e9, 2),
                      "alg_gbs": round((nnz * (4 + 8 + 8) + 8 * rows + 4 * rows) / tf / 1e9, 1),
                      "speedup_vs_vcode": round(t / tf, 2),
                      "max_abs_diff_vs_vcode": float(np.max(np.abs(yf - yh)))}}
    return spmv


def vinterp_suite(g, log2n=26, log2rows=22, seed=2026, cpu_sample_log2n=20):
    """The plain drop-in at scale through a VCODE interpreter: NESL
    quicksort (this repository's flattened VCODE program) on 2^log2n
    uniform int32 keys, and sparse matrix-vector product as a VCODE
    program on 2^log2rows rows with power-law row lengths (alpha 2.1 on
    [1, 2^16]), float64 values and x -- about 2^24.2 nonzeros at 2^22 rows,
    so the same law on 8x the rows ("row_scaled") brings it to about 2^27."""
    from neslgpu_gb300 import vcode as V, vcode_programs as P
    c = g.c
    sync = lambda: c.gcvl_sync()  # noqa: E731
    r = np.random.default_rng(seed)
    n = 1 << log2n
    keys = r.integers(-2 ** 31, 2 ** 31, size=n, dtype=np.int64).astype(np.int32)
    _vcode_sort(c, keys[: 1 << 16], sync)  # warm-up: kernels loaded, heap classes touched
    dev_s, e2e_s, out, ops = _vcode_sort(c, keys, sync)
    ok = bool(np.all(out[1:] >= out[:-1])) and int(out.astype(np.int64).sum()) == int(keys.astype(np.int64).sum())
    qs = {"n": n, "keys": "uniform int32, seeded", "seconds": round(dev_s, 4),
          "mkeys_s": round(n / dev_s / 1e6, 2), "e2e_seconds": round(e2e_s, 4),
          "e2e_mkeys_s": round(n / e2e_s / 1e6, 2), "vcode_ops": ops, "sorted": ok}
    # the .fcode form: elementwise chains as generated fused kernels
    from neslgpu_gb300 import fcode as F, vcode_programs as P
    lib = F.FusedLib(P.qsort_fcode_program()[1])
    _vcode_sort(c, keys[: 1 << 16], sync, lib)
    fdev, fe2e, fout, fops = _vcode_sort(c, keys, sync, lib)
    qs["fcode"] = {"seconds": round(fdev, 4), "mkeys_s": round(n / fdev / 1e6, 2), "vcode_ops": fops,
                   "same_result": bool(np.array_equal(fout, out)), "speedup_vs_vcode": round(dev_s / fdev, 3)}
    if cpu_sample_log2n:
        # the same interpreter and program on the oracle's serial CVL
        # restatement, one host thread, on a bounded sample
        from oracle.oracle import load_oracle
        ns = 1 << cpu_sample_log2n
        cs, _, cout, _ = _vcode_sort(load_oracle(), keys[:ns], lambda: None)
        qs["cpu_baseline"] = {"mkeys_s": round(ns / cs / 1e6, 3), "n": ns, "cores": 1, "kind": "port",
                              "sample": f"the first 2^{cpu_sample_log2n} keys, same VCODE program, oracle CVL",
                              "sorted": bool(np.all(cout[1:] >= cout[:-1]))}
    # sparse matrix-vector product: the configured 2^log2rows rows (about
    # 2^24.2 nonzeros), and the same row-length law on 8x the rows, which
    # reaches about 2^27 nonzeros
    spmv = _spmv_case(g, 1 << log2rows, r, sync)
    spmv["row_scaled"] = _spmv_case(g, 8 << log2rows, r, sync)
    return {"quicksort": qs, "spmv": spmv, "graph": graph_suite(c, sync)}


def cpu_baseline_port(x, lens, threads=1):
    """The oracle restatement of the serial CVL on this host: add_sed and
    add_red over the same values and segments.  With threads > 1 the
    segments are split into contiguous groups, one per thread (ctypes
    releases the GIL, so the C loops run in parallel)."""
    from oracle.oracle import load_oracle
    o = load_oracle()
    n, m = len(x), len(lens)
    scan = np.empty(n)
    red = np.empty(m)
    cuts = [0]
    if threads > 1:
        c = np.cumsum(lens, dtype=np.int64)
        for t in range(1, threads):
            cuts.append(int(np.searchsorted(c, n * t // threads)))
    cuts.append(m)
    starts = np.concatenate([[0], np.cumsum(lens, dtype=np.int64)])

    def work(a, b):
        if b <= a:
            return
        e0, e1 = int(starts[a]), int(starts[b])
        sd = np.ascontiguousarray(lens[a:b])
        xs = x[e0:e1]
        o.add_sed(scan[e0:].ctypes.data, xs.ctypes.data, sd.ctypes.data, e1 - e0, b - a, None)
        o.add_red(red[a:].ctypes.data, xs.ctypes.data, sd.ctypes.data, e1 - e0, b - a, None)

    t0 = time.perf_counter()
    ths = [threading.Thread(target=work, args=(cuts[i], cuts[i + 1])) for i in range(len(cuts) - 1)]
    for th in ths:
        th.start()
    for th in ths:
        th.join()
    return time.perf_counter() - t0, scan, red


def e2e_pipelined(g, lens, hx, hs, hr, steps, chunks=8):
    """The end-to-end step with the vector cut at segment starts (512-byte
    aligned in the host buffers) into `chunks` pieces of about n / chunks
    elements, each a segmented vector of
    its own (device buffers and segment descriptor built once, outside the
    timed region), as a three-stage pipeline on three library streams --
    uploads, kernels, downloads -- ordered by events, so that the upload of
    one piece, the kernels of another and the download of a third overlap
    (and uploads overlap downloads: the link carries both directions at
    once).  Every element and segment goes up and comes back exactly once
    per step.  Returns (seconds per step, pieces)."""
    c = g.c
    n = int(lens.sum())
    ends = np.cumsum(lens, dtype=np.int64)
    starts = ends - lens
    # cut at segment starts whose host byte offset is a multiple of 512: the
    # copy engines moved 341 GB/s both ways between 512-byte aligned host
    # addresses and 228 GB/s from 8-byte aligned ones
    aligned = np.flatnonzero((starts % 64 == 0) & (lens > 0))
    cuts = [0]
    for k in range(1, chunks):
        target = n * k // chunks
        j = int(np.searchsorted(starts[aligned], target))
        cand = aligned[max(j - 1, 0):j + 1]
        if len(cand) == 0:
            continue
        sc = int(cand[np.argmin(np.abs(starts[cand] - target))])
        if sc > cuts[-1]:
            cuts.append(sc)
    cuts.append(len(lens))
    pieces = []
    for s0, s1 in zip(cuts[:-1], cuts[1:]):
        e0 = int(starts[s0])
        pl = np.ascontiguousarray(lens[s0:s1], dtype=np.int32)
        pn, pm = int(pl.sum()), len(pl)
        p = {"e0": e0, "s0": s0, "n": pn, "m": pm, "x": g.alloc(c.siz_fod(pn)), "y": g.alloc(c.siz_fod(pn)),
             "r": g.alloc(c.siz_fod(pm)), "sd": g.alloc(c.siz_fos(pn, pm))}
        p["scr"] = g.alloc(max(c.mke_fov_scratch(pn, pm), c.add_sed_scratch(pn, pm), c.add_red_scratch(pn, pm), 1))
        lv = g.alloc(c.siz_foz(pm))
        c.c2v_fuz(lv, pl.ctypes.data, pm, None)
        c.mke_fov(p["sd"], lv, pn, pm, p["scr"])
        c.gcvl_sync()
        c.fre_fov(lv)
        pieces.append(p)
    assert sum(p["n"] for p in pieces) == n and sum(p["m"] for p in pieces) == len(lens)
    streams = [c.gcvl_stream_create() for _ in range(3)]
    if not all(streams):
        raise RuntimeError(c.gcvl_error_string().decode())
    up, ker, down = streams
    for p in pieces:
        p["ev"] = {k: c.gcvl_event_create() for k in ("up", "ker", "down")}
        c.gcvl_set_stream(ker)
        c.gcvl_event_record(p["ev"]["ker"])
        c.gcvl_event_record(p["ev"]["down"])
    c.gcvl_set_stream(None)

    def run():
        for p in pieces:
            ev = p["ev"]
            c.gcvl_set_stream(up)
            c.gcvl_stream_wait_event(ev["ker"])  # the previous step's kernels have read x
            c.gcvl_h2d_async(p["x"], hx + 8 * p["e0"], 8 * p["n"])
            c.gcvl_event_record(ev["up"])
            c.gcvl_set_stream(ker)
            c.gcvl_stream_wait_event(ev["up"])
            c.gcvl_stream_wait_event(ev["down"])  # the previous step's downloads have read y, r
            c.add_sed(p["y"], p["x"], p["sd"], p["n"], p["m"], p["scr"])
            c.add_red(p["r"], p["x"], p["sd"], p["n"], p["m"], p["scr"])
            c.gcvl_event_record(ev["ker"])
            c.gcvl_set_stream(down)
            c.gcvl_stream_wait_event(ev["ker"])
            c.gcvl_d2h_async(hs + 8 * p["e0"], p["y"], 8 * p["n"])
            c.gcvl_d2h_async(hr + 8 * p["s0"], p["r"], 8 * p["m"])
            c.gcvl_event_record(ev["down"])
        c.gcvl_set_stream(None)

    def sync_all():
        for q in streams:
            c.gcvl_set_stream(q)
            c.gcvl_sync()
        c.gcvl_set_stream(None)

    try:
        for _ in range(2):
            run()
        sync_all()
        t0 = time.perf_counter()
        for _ in range(steps):
            run()
        sync_all()
        dt = (time.perf_counter() - t0) / steps
    finally:
        c.gcvl_set_stream(None)
        for q in streams:
            c.gcvl_stream_destroy(q)
    g.check(c)
    for p in pieces:
        for k in ("x", "y", "r", "sd", "scr"):
            c.fre_fov(p[k])
        for e in p["ev"].values():
            c.gcvl_event_destroy(e)
    return dt, len(pieces)


def gpu_arm(a):
    world, rank, local, pg = dist()
    os.environ.setdefault("GCVL_DEVICE", str(local))
    g = Gpu()
    c = g.c
    hbm, peak_kind = peaks()
    n = 1 << a.log2n
    lens = segment_lengths(n)
    m = len(lens)

    # device-resident inputs
    x = g.alloc(c.siz_fod(n))
    c.gcvl_fill_random(x, n, 1, SEED, 0.0, 0)
    lv = g.alloc(c.siz_foz(m))
    c.c2v_fuz(lv, lens.ctypes.data, m, None)
    sd = g.alloc(c.siz_fos(n, m))
    scr = g.alloc(max(c.mke_fov_scratch(n, m), c.add_sed_scratch(n, m), c.add_red_scratch(n, m)))
    c.mke_fov(sd, lv, n, m, scr)
    ys = g.alloc(c.siz_fod(n))
    yr = g.alloc(c.siz_fod(m))
    g.check(c)

    e_sed = [g.events(2) for _ in range(a.steps)]
    e_red = [g.events(2) for _ in range(a.steps)]
    e_all = g.events(2)

    def step(i=None):
        if i is not None:
            c.gcvl_event_record(e_sed[i][0])
        c.add_sed(ys, x, sd, n, m, scr)
        if i is not None:
            c.gcvl_event_record(e_sed[i][1])
            c.gcvl_event_record(e_red[i][0])
        c.add_red(yr, x, sd, n, m, scr)
        if i is not None:
            c.gcvl_event_record(e_red[i][1])

    for _ in range(a.warmup):
        step()
    g.check(c)
    barrier(pg)
    clk = Clocks(local)
    with clk:
        time.sleep(1.0)  # let the sampler start
        c.gcvl_sync()
        barrier(pg)
        l0 = c.gcvl_launch_count()
        w0 = time.time()
        c.gcvl_event_record(e_all[0])
        for i in range(a.steps):
            step(i)
        c.gcvl_event_record(e_all[1])
        c.gcvl_sync()
        w1 = time.time()
        launches = c.gcvl_launch_count() - l0
        barrier(pg)
        time.sleep(0.2)
    g.check(c)
    ms_total = allmax(pg, g.ms(e_all[0], e_all[1]))
    ms_step = ms_total / a.steps
    t_sed = statistics.mean(g.ms(*e) for e in e_sed)
    t_red = statistics.mean(g.ms(*e) for e in e_red)
    value = world * 2 * n / (ms_step * 1e-3) / 1e9

    # roofline of the dominant kernel (the add_sed scan)
    alg_bytes = 16.0 * n + 4.0 * m
    achieved = alg_bytes / (t_sed * 1e-3) / 1e9
    # DRAM bytes per launch: dram__bytes_read.sum + dram__bytes_write.sum of
    # one ncu capture of this kernel at 2^25 elements (489 MB), scaled by the
    # elements to this launch (profiles/k_scan_ring_add_sed_k_scan_tma_add_red_2e25.md)
    traffic = round(NCU_SCAN_DRAM_BYTES_PER_ELEM * n)
    roofline = {"bound": "hbm", "kernel": "k_scan_ring<AddD,segmented> (add_sed)",
                "achieved": round(achieved, 1), "peak": hbm, "peak_kind": peak_kind, "unit": "GB/s",
                "frac": round(achieved / hbm, 4), "traffic": traffic,
                "traffic_source": "ncu capture at 2^25 elements, scaled by the elements",
                "alg_bytes_per_launch": alg_bytes,
                "add_red": {"ms": round(t_red, 4),
                            "achieved": round((8.0 * n + 12.0 * m) / (t_red * 1e-3) / 1e9, 1)}}

    # end to end through the C ABI with pinned host buffers
    e2e = None
    if a.e2e_steps > 0:
        hx = c.gcvl_host_alloc(8 * n)
        hs = c.gcvl_host_alloc(8 * n)
        hr = c.gcvl_host_alloc(8 * m)
        c.v2c_fud(hx, x, n, None)  # the same values, now on the host
        for _ in range(2):
            c.c2v_fud(x, hx, n, None)
            step()
            c.v2c_fud(hs, ys, n, None)
            c.v2c_fud(hr, yr, m, None)
        barrier(pg)
        c.gcvl_sync()
        t0 = time.perf_counter()
        for _ in range(a.e2e_steps):
            c.c2v_fud(x, hx, n, None)
            step()
            c.v2c_fud(hs, ys, n, None)
            c.v2c_fud(hr, yr, m, None)
        c.gcvl_sync()
        dt_seq = allmax(pg, (time.perf_counter() - t0) / a.e2e_steps)
        g.check(c)
        # the whole-vector results of the sequential form, to check the pieces against
        ws = np.empty(n)
        wr = np.empty(m)
        C.memmove(ws.ctypes.data, hs, 8 * n)
        C.memmove(wr.ctypes.data, hr, 8 * m)
        C.memset(hs, 0, 8 * n)
        C.memset(hr, 0, 8 * m)
        barrier(pg)
        dt_pipe, npieces = e2e_pipelined(g, lens, hx, hs, hr, a.e2e_steps)
        dt_pipe = allmax(pg, dt_pipe)
        ps = np.ctypeslib.as_array(C.cast(hs, C.POINTER(C.c_double)), shape=(n,))
        pr = np.ctypeslib.as_array(C.cast(hr, C.POINTER(C.c_double)), shape=(m,))
        diff = float(max(np.max(np.abs(ps - ws)), np.max(np.abs(pr - wr))))
        e2e = {"value": round(world * 2 * n / dt_pipe / 1e9, 3), "unit": UNIT,
               "ms_per_step": round(dt_pipe * 1e3, 3),
               "h2d_bytes_per_step": 8 * n, "d2h_bytes_per_step": 8 * n + 8 * m,
               "api": f"gcvl_h2d_async, add_sed, add_red, gcvl_d2h_async x2 per piece; {npieces} pieces cut at "
                      "segment starts, pipelined on three library streams (uploads, kernels, downloads; "
                      "gcvl_stream_create / gcvl_set_stream / gcvl_stream_wait_event), pinned host buffers",
               "max_abs_diff_vs_whole_vector": diff,
               "sequential": {"value": round(world * 2 * n / dt_seq / 1e9, 3), "ms_per_step": round(dt_seq * 1e3, 3),
                              "api": "c2v_fud, add_sed, add_red, v2c_fud x2 on the whole vector"}}

    cpu = parity = None
    if rank == 0 and world == 1 and not a.no_cpu:
        xh = np.empty(n)
        c.v2c_fud(xh.ctypes.data, x, n, None)
        t, scan, red = cpu_baseline_port(xh, lens, threads=1)
        cpu = {"value": round(2 * n / t / 1e9, 4), "unit": UNIT, "cores": 1, "kind": "port",
               "sample": f"the full workload once (add_sed + add_red over 2^{a.log2n} float64, {m} segments), "
                         "oracle restatement of the serial CVL, 1 thread"}
        # the GPU results of the timed steps against the CPU ones
        gs = np.empty(n)
        c.v2c_fud(gs.ctypes.data, ys, n, None)
        gr = np.empty(m)
        c.v2c_fud(gr.ctypes.data, yr, m, None)
        e_scan = sum_err_over_tol(gs, scan, xh, lens, "scan")
        e_red = sum_err_over_tol(gr, red, xh, lens, "reduce")
        parity = {"rule": "|gpu - cpu| <= 1e-12 * max(|cpu|, S), S = sum of |x| over the same prefix "
                          "(add_sed) or segment (add_red); err/tol <= 1 passes",
                  "max_err_over_tol": {"add_sed": e_scan, "add_red": e_red},
                  "ok": bool(e_scan <= 1.0 and e_red <= 1.0),
                  "against": "the oracle (CPU restatement of the serial CVL) on the same values"}

    prims = batched = dispatch = vinterp = None
    if not a.no_suite and rank == 0:
        prims = primitive_suite(g, n, hbm)
        batched = batched_suite(g)
        dispatch = dispatch_suite(g)
        vinterp = vinterp_suite(g)

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world,
            "steps": a.steps, "warmup": a.warmup, "ms_per_step": round(ms_step, 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (device-generated N(0,1) values, seeded; host-generated segment lengths)",
            "config": {"workload": f"add_sed + add_red, 2^{a.log2n} float64 N(0,1), segment lengths "
                                   "round(LogNormal(5,2)) clipped to [1, 2^24]",
                       "n": n, "m": m, "elements_per_step": 2 * n,
                       "l2": "inputs larger than L2 (2 GiB per vector), no flush",
                       "parallelism": f"{world} independent replicas"},
            "roofline": roofline, "cpu_baseline": cpu, "parity": parity, "e2e": e2e,
            "gpu_launches": int(launches),
            "clocks": clk.summary(w0, w1), "primitives": prims, "batched": batched, "dispatch": dispatch,
            "vinterp": vinterp,
        }
        print(json.dumps(line))


# ------------------------------------------------------ reference arm ---
def reference_arm(a):
    # rank 0 alone times the CPU implementation; other ranks exit at once
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from neslgpu_gb300 import workloads as W
    n = 1 << a.log2n
    lens = segment_lengths(n)
    m = len(lens)
    cores = os.cpu_count() or 1
    x = W.float64_normal(W.rng(SEED), n)
    times = []
    for _ in range(a.warmup):
        cpu_baseline_port(x, lens, threads=cores)
    for _ in range(a.steps):
        t, _, _ = cpu_baseline_port(x, lens, threads=cores)
        times.append(t)
    t = statistics.median(times)
    v = round(2 * n / t / 1e9, 4)
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": round(t * 1e3, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (host-generated, seeded)",
        "config": {"workload": f"add_sed + add_red, 2^{a.log2n} float64 N(0,1), segment lengths "
                               "round(LogNormal(5,2)) clipped to [1, 2^24]", "n": n, "m": m,
                   "elements_per_step": 2 * n},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": "the full workload per step; segments split across all host threads; "
                                   "the serial CVL's algorithm as restated by the oracle (the reference "
                                   "sources are not present on this machine)"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=500)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--log2n", type=int, default=LOG2N)
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-suite", action="store_true")
    ap.add_argument("--suite-only", action="store_true",
                    help="only the per-primitive table at 2^log2n (for profiling)")
    ap.add_argument("--prims", default=None,
                    help="with --suite-only: comma-separated primitives to time (e.g. rku_luz,pk2_lez)")
    ap.add_argument("--batched-only", action="store_true", help="only the batched workload")
    ap.add_argument("--dispatch-only", action="store_true", help="only the learned-dispatcher sweep")
    ap.add_argument("--vinterp-only", action="store_true", help="only the VCODE programs")
    ap.add_argument("--graph-only", action="store_true", help="only VCODE basic blocks as CUDA graphs")
    ap.add_argument("--dispatch-count", type=int, default=4096)
    ap.add_argument("--dispatch-hi", type=int, default=28)
    a = ap.parse_args()
    a.warmup = max(a.warmup, 3) if a.impl == "gb300" else a.warmup
    if a.impl == "reference":
        reference_arm(a)
    elif a.suite_only:
        g = Gpu()
        only = set(a.prims.split(",")) if a.prims else None
        print(json.dumps({"primitives": primitive_suite(g, 1 << a.log2n, peaks()[0], only)}))
    elif a.batched_only:
        print(json.dumps({"batched": batched_suite(Gpu())}))
    elif a.graph_only:
        c = Gpu().c
        print(json.dumps({"graph": graph_suite(c, lambda: c.gcvl_sync())}))
    elif a.vinterp_only:
        print(json.dumps({"vinterp": vinterp_suite(Gpu())}))
    elif a.dispatch_only:
        print(json.dumps({"dispatch": dispatch_suite(Gpu(), count=a.dispatch_count, hi=a.dispatch_hi)}))
    else:
        gpu_arm(a)


if __name__ == "__main__":
    main()
