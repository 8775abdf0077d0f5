"""Parity cases shared by the CPU tests (oracle vs the reference's serial CVL)
and the GPU tests (libcvl_gb300.so vs the oracle).

A case is (id, run, cmp): ``run(runner)`` calls one CVL primitive through
``neslgpu_gb300.ops`` and returns its result; ``cmp`` names the comparison:

* ``exact``  -- bit-identical (int, bool, index work; float64 moves, min/max)
* ``sum``    -- float64 sums: |a - b| <= 1e-12 * max(|b|, S), S = sum of |x|
                over the same prefix (scan) or segment (reduce)
* ``prod``   -- float64 products: |a - b| <= 1e-12 * |b| (or identical)
* ``ulp``    -- libm vs CUDA math: |a - b| <= 1e-13 * |b| (or identical)
"""
from __future__ import annotations

import numpy as np

from neslgpu_gb300 import ops
from neslgpu_gb300 import workloads as W

SUM_RTOL = 1e-12


def compare(cmp, got, want, ctx=None):
    got = np.asarray(got)
    want = np.asarray(want)
    if np.ndim(want) == 0:
        got = np.asarray([got]).astype(want.dtype if want.dtype != object else float)
        want = np.asarray([want])
    assert got.shape == want.shape, f"shape {got.shape} != {want.shape}"
    if cmp == "exact":
        if want.dtype == np.float64:
            ok = np.array_equal(got.view(np.int64), want.view(np.int64))
        else:
            ok = np.array_equal(got, want)
        if not ok:
            bad = np.flatnonzero(got != want)[:8]
            raise AssertionError(f"mismatch at {bad}: got {got[bad]} want {want[bad]}")
        return
    if cmp == "sum":
        S = ctx if ctx is not None else np.abs(want)
        tol = SUM_RTOL * np.maximum(np.abs(want), S) + 1e-300
        err = np.abs(got - want)
        if not np.all(err <= tol):
            i = int(np.argmax(err / tol))
            raise AssertionError(f"sum mismatch at {i}: got {got[i]!r} want {want[i]!r} tol {tol[i]:.3g}")
        return
    rtol = 1e-12 if cmp == "prod" else 1e-13
    same = (got == want) | (np.isnan(got) & np.isnan(want))
    close = np.abs(got - want) <= rtol * np.abs(want)
    if not np.all(same | close):
        i = int(np.flatnonzero(~(same | close))[0])
        raise AssertionError(f"{cmp} mismatch at {i}: got {got[i]!r} want {want[i]!r}")


def seg_abs_prefix(x, lengths):
    """S for exclusive segmented scans: sum of |x| before k in its segment."""
    a = np.abs(np.asarray(x, dtype=np.float64))
    c = np.concatenate([[0.0], np.cumsum(a)])
    lengths = np.asarray(lengths, dtype=np.int64)
    starts = np.cumsum(lengths) - lengths
    seg_start = np.repeat(starts, lengths)
    k = np.arange(len(a))
    return c[k] - c[seg_start]


def seg_abs_total(x, lengths):
    a = np.abs(np.asarray(x, dtype=np.float64))
    c = np.concatenate([[0.0], np.cumsum(a)])
    ends = np.cumsum(lengths, dtype=np.int64)
    starts = ends - lengths
    return c[ends] - c[starts]


def sum_err_over_tol(got, want, x, lengths, kind, chunk=1 << 24):
    """max over elements of |got - want| / (1e-12 * max(|want|, S)) for a
    segmented float64 +-scan (kind "scan": S = sum of |x| before the element
    in its segment) or +-reduction ("reduce": S = sum of |x| over the
    segment), computed over groups of whole segments of about `chunk`
    elements so that vectors of 2^28 elements need little extra memory.
    A result passes when the value is <= 1."""
    x = np.asarray(x, dtype=np.float64)
    lengths = np.asarray(lengths, dtype=np.int64)
    ends = np.cumsum(lengths)
    starts = ends - lengths
    worst = 0.0
    a = 0
    m = len(lengths)
    while a < m:
        b = max(a + 1, int(np.searchsorted(ends, starts[a] + chunk, side="right")))
        b = min(b, m)
        e0, e1 = int(starts[a]), int(ends[b - 1])
        ln = lengths[a:b]
        if kind == "scan":
            S = seg_abs_prefix(x[e0:e1], ln)
            g, w = got[e0:e1], want[e0:e1]
        else:
            S = seg_abs_total(x[e0:e1], ln)
            g, w = got[a:b], want[a:b]
        if len(w):
            tol = SUM_RTOL * np.maximum(np.abs(w), S) + 1e-300
            err = np.abs(g - w)
            same = (g == w) | (np.isnan(g) & np.isnan(w))
            worst = max(worst, float(np.max(np.where(same, 0.0, err / tol))))
        a = b
    return worst


SCAN_OPS = [("add", "z"), ("add", "d"), ("mul", "z"), ("mul", "d"), ("min", "z"), ("min", "d"),
            ("max", "z"), ("max", "d"), ("and", "b"), ("and", "z"), ("ior", "b"), ("ior", "z"),
            ("xor", "b"), ("xor", "z")]
EW2_Z = ["max", "min", "add", "sub", "mul", "div", "grt", "les", "geq", "leq", "lsh", "rsh",
         "mod", "eql", "neq", "ior", "and", "xor"]
EW2_D = ["max", "min", "add", "sub", "mul", "div", "grt", "les", "geq", "leq", "eql", "neq"]
EW2_B = ["eql", "neq", "xor", "ior", "and"]
EW1_D_EXACT = ["int", "flr", "cei", "trn", "rou", "sqt", "cpy"]
EW1_D_ULP = ["exp", "log", "sin", "cos", "tan", "asn", "acs", "atn", "snh", "csh", "tnh"]


def _cmp_for(op, t):
    if t != "d":
        return "exact"
    return {"add": "sum", "mul": "prod"}.get(op, "exact")


def make_cases(n=5000, seed=7, lengths_kind="geo", include_ulp=True):
    """Cases over one random workload of n elements."""
    r = W.rng(seed)
    n = int(n)
    xi = W.int32_uniform(r, n)
    yi = W.int32_uniform(r, n)
    yi_nz = np.where(yi == 0, 1, yi).astype(np.int32)
    small = r.integers(-1000, 1000, size=n).astype(np.int32)
    small_nz = np.where(small == 0, 7, small).astype(np.int32)
    shifts = r.integers(0, 40, size=n).astype(np.int32)
    xd = W.float64_normal(r, n)
    yd = W.float64_normal(r, n)
    yd[::97] = xd[::97]  # some equal pairs for comparisons
    bx = r.integers(0, 2, size=n).astype(np.int32)
    by = r.integers(0, 2, size=n).astype(np.int32)
    bz = r.integers(-3, 4, size=n).astype(np.int32)  # cvl_bools that are not 0/1
    if lengths_kind == "geo":
        lens = W.geometric_lengths(r, n, 64)
    elif lengths_kind == "tiny":
        lens = W.geometric_lengths(r, n, 1.5)
    elif lengths_kind == "long":
        lens = W.lognormal_lengths(r, n, 9.0, 2.0, max(n, 1))
    elif lengths_kind == "empty":
        lens = W.with_empty(r, W.geometric_lengths(r, n, 16), 0.5)
    elif lengths_kind == "bimodal":
        lens = W.bimodal_lengths(r, n)
    elif lengths_kind == "one":
        lens = np.array([n], dtype=np.int32)
    else:
        raise ValueError(lengths_kind)
    m = len(lens)
    perm = W.permutation(r, n)
    sperm = W.seg_permutation(r, lens)
    flags = r.integers(0, 2, size=n).astype(np.int32)
    C = []

    def add(cid, fn, cmp="exact", ctx=None):
        C.append((cid, fn, cmp, ctx))

    # elementwise
    for op in EW2_Z:
        a, b = xi, yi
        if op in ("div", "mod"):
            a, b = small, small_nz
        if op in ("lsh", "rsh"):
            b = shifts
        add(f"{op}_wuz", lambda R, op=op, a=a, b=b: ops.ew2(R, f"{op}_wuz", a, b))
    for op in EW2_D:
        add(f"{op}_wud", lambda R, op=op: ops.ew2(R, f"{op}_wud", xd, yd))
    for op in EW2_B:
        add(f"{op}_wub", lambda R, op=op: ops.ew2(R, f"{op}_wub", bx, by))
    add("and_wub_raw", lambda R: ops.ew2(R, "and_wub", bz, by))
    add("not_wub", lambda R: ops.ew1(R, "not_wub", bz))
    add("not_wuz", lambda R: ops.ew1(R, "not_wuz", xi))
    add("int_wub", lambda R: ops.ew1(R, "int_wub", bx))
    add("boo_wuz", lambda R: ops.ew1(R, "boo_wuz", small))
    add("dbl_wuz", lambda R: ops.ew1(R, "dbl_wuz", xi))
    add("cpy_wuz", lambda R: ops.ew1(R, "cpy_wuz", xi))
    add("cpy_wub", lambda R: ops.ew1(R, "cpy_wub", bx))
    scaled = xd * 1000.0
    for op in EW1_D_EXACT:
        src = np.abs(xd) if op == "sqt" else scaled
        add(f"{op}_wud", lambda R, op=op, src=src: ops.ew1(R, f"{op}_wud", src))
    if include_ulp:
        for op in EW1_D_ULP:
            src = {"log": np.abs(xd) + 1e-3, "asn": np.tanh(xd), "acs": np.tanh(xd)}.get(op, xd)
            add(f"{op}_wud", lambda R, op=op, src=src: ops.ew1(R, f"{op}_wud", src), "ulp")
    for t in "zbd":
        a, b = {"z": (xi, yi), "b": (bx, by), "d": (xd, yd)}[t]
        add(f"sel_wu{t}", lambda R, t=t, a=a, b=b: ops.sel(R, f"sel_wu{t}", bz, a, b))

    # scans and reductions
    for op, t in SCAN_OPS:
        x = {"z": xi if op != "mul" else small, "b": bz, "d": xd}[t]
        if op == "mul" and t == "d":
            x = 1.0 + 0.01 * xd
        cmp = _cmp_for(op, t)
        ctx_scan = seg_abs_prefix(x, lens) if cmp == "sum" else None
        ctx_red = seg_abs_total(x, lens) if cmp == "sum" else None
        ctx_uscan = seg_abs_prefix(x, [n]) if cmp == "sum" else None
        add(f"{op}_su{t}", lambda R, op=op, t=t, x=x: ops.scan_u(R, f"{op}_su{t}", x), cmp, ctx_uscan)
        add(f"{op}_se{t}", lambda R, op=op, t=t, x=x: ops.scan_e(R, f"{op}_se{t}", x, lens), cmp, ctx_scan)
        add(f"{op}_re{t}", lambda R, op=op, t=t, x=x: ops.reduce_e(R, f"{op}_re{t}", x, lens), cmp, ctx_red)
        add(f"{op}_ru{t}", lambda R, op=op, t=t, x=x: np.asarray(ops.reduce_u(R, f"{op}_ru{t}", x)),
            cmp, np.asarray(np.sum(np.abs(x))) if cmp == "sum" else None)

    # vector primitives
    seg_idx = W.seg_indices(r, np.maximum(lens, 1), np.ones(m, dtype=np.int32))
    nonempty = lens > 0
    for t in "zbd":
        x = {"z": xi, "b": bx, "d": xd}[t]
        vals_m = {"z": yi[:m] if m <= n else np.resize(yi, m), "b": np.resize(by, m), "d": np.resize(yd, m)}[t]
        if n:
            add(f"ext_vu{t}", lambda R, t=t, x=x: np.asarray(ops.ext_u(R, f"ext_vu{t}", x, n // 3)))
            add(f"rep_vu{t}", lambda R, t=t, x=x, v=vals_m: ops.rep_u(R, f"rep_vu{t}", x, n // 2, v[0].item()))
        if np.all(nonempty):
            add(f"ext_ve{t}", lambda R, t=t, x=x: ops.ext_e(R, f"ext_ve{t}", x, seg_idx, lens))
            add(f"rep_ve{t}", lambda R, t=t, x=x, v=vals_m: ops.rep_e(R, f"rep_ve{t}", x, seg_idx, v, lens))
        add(f"dis_vu{t}", lambda R, t=t, v=vals_m: ops.dis_u(R, f"dis_vu{t}", v[0].item() if m else 1, n))
        add(f"dis_ve{t}", lambda R, t=t, v=vals_m: ops.dis_e(R, f"dis_ve{t}", v, lens))
        add(f"smp_pu{t}", lambda R, t=t, x=x: ops.smp_u(R, f"smp_pu{t}", x, perm))
        add(f"smp_pe{t}", lambda R, t=t, x=x: ops.smp_e(R, f"smp_pe{t}", x, sperm, lens))
        add(f"bck_pu{t}", lambda R, t=t, x=x: ops.bck_u(R, f"bck_pu{t}", x, perm))
        add(f"bck_pe{t}", lambda R, t=t, x=x: ops.bck_e(R, f"bck_pe{t}", x, sperm, lens, lens))
        add(f"fpm_pu{t}", lambda R, t=t, x=x: ops.fpm_u(R, f"fpm_pu{t}", x, perm, flags, n))
        add(f"fpm_pe{t}", lambda R, t=t, x=x: ops.fpm_e(R, f"fpm_pe{t}", x, sperm, flags, lens, lens))
        add(f"bfp_pu{t}", lambda R, t=t, x=x: ops.fpm_u(R, f"bfp_pu{t}", x, perm, flags, n))
        add(f"bfp_pe{t}", lambda R, t=t, x=x: ops.fpm_e(R, f"bfp_pe{t}", x, sperm, flags, lens, lens))
        dflt = {"z": yi, "b": by, "d": yd}[t]
        add(f"dpe_pu{t}", lambda R, t=t, x=x, v=dflt: ops.dpe_u(R, f"dpe_pu{t}", x, perm, v))
        add(f"dpe_pe{t}", lambda R, t=t, x=x, v=dflt: ops.dpe_e(R, f"dpe_pe{t}", x, sperm, v, lens, lens))
        add(f"dfp_pu{t}", lambda R, t=t, x=x, v=dflt: ops.fpm_u(R, f"dfp_pu{t}", x, perm, flags, n, v))
        add(f"dfp_pe{t}", lambda R, t=t, x=x, v=dflt: ops.fpm_e(R, f"dfp_pe{t}", x, sperm, flags, lens, lens, v))
        add(f"pk2_lu{t}", lambda R, t=t, x=x: ops.pack_u(R, f"pk2_lu{t}", x, flags))
        add(f"pack_le{t}", lambda R, t=t, x=x: np.concatenate(
            [np.asarray(a, dtype=np.float64) for a in ops.pack_e(R, f"pk2_le{t}", x, flags, lens)]))
    add("pk1_luv", lambda R: np.asarray(ops.pk1_u(R, bz)))
    add("pk1_lev", lambda R: ops.pk1_e(R, bz, lens))
    add("ind_luz", lambda R: ops.ind_u(R, -5, 3, n))
    add("ind_lez", lambda R: ops.ind_e(R, np.resize(small, m), np.resize(small_nz, m), lens))
    # rank: full-range keys plus keys with many ties
    ties = (small % 13).astype(np.int32)
    tied_d = np.round(xd * 4) / 4
    for ud in "ud":
        add(f"rk{ud}_luz", lambda R, ud=ud: ops.rank_u(R, f"rk{ud}_luz", xi))
        add(f"rk{ud}_luz_ties", lambda R, ud=ud: ops.rank_u(R, f"rk{ud}_luz", ties))
        add(f"rk{ud}_lez", lambda R, ud=ud: ops.rank_e(R, f"rk{ud}_lez", ties, lens))
        add(f"rk{ud}_lud", lambda R, ud=ud: ops.rank_u(R, f"rk{ud}_lud", xd))
        add(f"rk{ud}_lud_ties", lambda R, ud=ud: ops.rank_u(R, f"rk{ud}_lud", tied_d))
        add(f"rk{ud}_led", lambda R, ud=ud: ops.rank_e(R, f"rk{ud}_led", tied_d, lens))
    return C
