"""Every kernel variant of the segmented scans, reductions and ranks
(gcvl_run_variant) against the oracle's serial CVL restatement: integer,
min/max and rank results bit-identical, float64 sums within
|a - b| <= 1e-12 * max(|b|, S), S the sum of |x| over the same prefix or
segment -- the same bar as the default kernels, whichever variant runs."""
import numpy as np
import pytest

from cases import compare, seg_abs_prefix, seg_abs_total
from neslgpu_gb300 import ops
from neslgpu_gb300 import workloads as W

pytestmark = pytest.mark.gpu

PRIMS = ["add_sez", "add_sed", "max_sez", "max_sed", "add_rez", "add_red", "max_rez", "max_red"]
RANKS = ["rku_lez", "rku_led", "rkd_lez", "rkd_led"]


def _lengths(r, kind, n):
    if kind == "geo4":
        return W.geometric_lengths(r, n, 4.0)
    if kind == "geo300":
        return W.with_empty(r, W.geometric_lengths(r, n, 300.0), 0.1)
    if kind == "bimodal":
        return W.bimodal_lengths(r, n)
    if kind == "one":
        return np.array([n], dtype=np.int32)
    raise ValueError(kind)


def _run(R, prim, v, x, lens):
    c = R.cvl
    k = "d" if prim.endswith("d") else "z"
    sd, n, m = R.segd(lens)
    a = R.vec(x, k)
    reduce_ = prim[4] == "r"
    rank = prim.startswith("rk")
    out_n = m if reduce_ else n
    d = R.out(out_n, "z" if rank else k)
    scr = R.units(c.gcvl_variant_scratch(prim.encode(), n, m))
    rc = c.gcvl_run_variant(prim.encode(), v, d.ptr, a.ptr, sd.ptr, n, m, scr.ptr)
    assert rc == 0, c.gcvl_error_string().decode()
    got = R.get(d, out_n)
    R.done()
    return got


@pytest.mark.parametrize("kind", ["geo4", "geo300", "bimodal", "one"])
@pytest.mark.parametrize("prim", PRIMS)
def test_scan_reduce_variants(gpu, oracle, prim, kind):
    r = W.rng(31)
    n = 200_003 if kind != "one" else 70_001
    lens = _lengths(r, kind, n)
    x = W.float64_normal(r, n) if prim.endswith("d") else r.integers(-1000, 1000, size=n).astype(np.int32)
    if prim[4] == "s":
        want = ops.scan_e(oracle, prim, x, lens)
        ctx = seg_abs_prefix(x, lens)
    else:
        want = ops.reduce_e(oracle, prim, x, lens)
        ctx = seg_abs_total(x, lens)
    cmp = "sum" if prim == "add_sed" or prim == "add_red" else "exact"
    nv = gpu.cvl.gcvl_variant_count()
    for v in range(nv):
        if not gpu.cvl.gcvl_variant_valid(prim.encode(), v, int(lens.max(initial=0))):
            continue
        got = _run(gpu, prim, v, x, lens)
        compare(cmp, got, want, ctx if cmp == "sum" else None)


@pytest.mark.parametrize("prim", RANKS)
def test_rank_variants(gpu, oracle, prim):
    r = W.rng(32)
    lens = np.minimum(W.geometric_lengths(r, 150_001, 500.0), 2048).astype(np.int32)
    n = int(lens.sum())
    if prim.endswith("d"):
        x = np.round(W.float64_normal(r, n), 2)  # ties
    else:
        x = r.integers(-300, 300, size=n).astype(np.int32)
    want = ops.rank_e(oracle, prim, x, lens)
    for v in range(gpu.cvl.gcvl_variant_count()):
        if gpu.cvl.gcvl_variant_valid(prim.encode(), v, int(lens.max())):
            compare("exact", _run(gpu, prim, v, x, lens), want)
    assert not gpu.cvl.gcvl_variant_valid(prim.encode(), 5, 2049)
