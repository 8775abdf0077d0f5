"""The batched form (neslgpu_gb300/batch.py): the per-vector call loop, the
flattened sequence and its CUDA-graph replay give the same results, and
those results are the composition of the oracle's primitives on the
flattened vector (segments never cross vector boundaries)."""
import numpy as np
import pytest

from cases import compare, seg_abs_prefix
from neslgpu_gb300 import batch as B
from neslgpu_gb300 import ops

pytestmark = pytest.mark.gpu


def _oracle_pipeline(ora, x, lens, is_double):
    L = "d" if is_double else "z"
    y = ops.scan_e(ora, f"add_se{L}", x, lens)
    f = (x > 0).astype(np.int32)
    p, newlens = ops.pack_e(ora, f"pk2_le{L}", y, f, lens)
    return y, f, newlens, p


@pytest.mark.parametrize("is_double", [False, True])
def test_modes_agree_and_match_oracle(gpu, oracle, is_double):
    b = B.make_batch(nvec=40, total=1 << 16, seed=5, hi=20_000)
    run = B.BatchRun(b, is_double, cvl=gpu.cvl)
    try:
        n2a = run.batched()
        ra = run.results(n2a)
        n2g = run.graph()
        rg = run.results(n2g)
        n2g2 = run.graph()  # a replay of the cached graphs
        rg2 = run.results(n2g2)
        n2p = run.percall()
        rp = run.results(n2p)
        x = run._get(run.x, b.n, np.float64 if is_double else np.int32)
    finally:
        run.free()
    # the graph replays the batched sequence exactly
    assert n2a == n2g == n2g2
    for k in ra:
        compare("exact", rg[k], ra[k])
        compare("exact", rg2[k], ra[k])
    y, f, newlens, p = _oracle_pipeline(oracle, x, b.seg_lens, is_double)
    assert n2a == n2p == int(newlens.sum())
    for r in (ra, rp):
        compare("exact", r["f"], f)
        compare("exact", r["newlens"], newlens)
        if is_double:
            S = seg_abs_prefix(x, b.seg_lens)
            compare("sum", r["y"], y, S)
            compare("sum", r["p"], p, S[f.astype(bool)])
        else:
            compare("exact", r["y"], y)
            compare("exact", r["p"], p)
    # per-call and batched draw the same RAND stream, so gather the same
    compare("exact", rp["idx"], ra["idx"])
    # the gather reads inside each packed segment
    off = np.concatenate([[0], np.cumsum(newlens, dtype=np.int64)])
    seg = np.repeat(np.arange(b.m), newlens)
    assert np.all((ra["idx"] >= 0) & (ra["idx"] < newlens[seg]))
    for r in (ra, rp):
        compare("exact", r["g"], r["p"][off[seg] + r["idx"]])


@pytest.mark.parametrize("is_double", [False, True])
def test_skewed_batch_flattened_matches_percall(gpu, is_double):
    """A few large vectors beside hundreds of tiny ones (the flattened
    form's worst case): the flattened sequence and the per-vector loop give
    the same results."""
    b = B.make_skewed_batch(huge=2, huge_len=1 << 15, tiny=400, tiny_hi=60, seed=8)
    run = B.BatchRun(b, is_double, cvl=gpu.cvl)
    try:
        n2a = run.batched()
        ra = run.results(n2a)
        n2p = run.percall()
        rp = run.results(n2p)
    finally:
        run.free()
    assert n2a == n2p
    for k in ("f", "newlens", "idx"):
        compare("exact", rp[k], ra[k])
    for k in ("y", "p", "g"):
        if is_double:  # float64 scans of the flattened vector reassociate only
            np.testing.assert_allclose(rp[k], ra[k], rtol=1e-12, atol=1e-9)
        else:
            compare("exact", rp[k], ra[k])
