"""gcvl_add_sed_noalloc: the segmented float64 +-scan for callers that may
not allocate device memory (code running during CUDA graph capture,
embedders whose device memory all belongs to their own pool).  It keeps its
scratch in a fixed array inside the library, so it is checked here against
the ordinary add_sed -- same inputs, through the C ABI -- on two calls in a
row (the array keeps the previous call's contents, which each call must
clear), on the TMA and the unaligned path, and for the size limit.

This file is collected last so that a failure here, in a run that stops at
the first failure, comes after every other test."""
import numpy as np
import pytest

from cases import compare, seg_abs_prefix
from neslgpu_gb300 import workloads as W
from neslgpu_gb300.cvl import DeviceVector, load
from neslgpu_gb300.ops import DeviceRunner

pytestmark = pytest.mark.gpu


def _scan_both(R, x, lens):
    """(add_sed result, gcvl_add_sed_noalloc result) for the same inputs."""
    c = R.cvl
    sd, n, m = R.segd(lens)
    xs = R.vec(x, "d")
    want = R.out(n, "d")
    scr = R.units(c.add_sed_scratch(n, m))
    c.add_sed(want.ptr, xs.ptr, sd.ptr, n, m, scr.ptr)
    got = R.out(n, "d")
    rc = c.gcvl_add_sed_noalloc(got.ptr, xs.ptr, sd.ptr, n, m)
    assert rc == 0, c.gcvl_error_string().decode()
    R.done()
    return R.get(got, n), R.get(want, n)


@pytest.mark.parametrize("offset", [0, 1])
def test_noalloc_matches_add_sed_twice(gpu, offset):
    R = DeviceRunner(load(), offset=offset)  # offset 1: not 16-byte aligned
    r = W.rng(77)
    for call, (n, mean) in enumerate([(300_007, 40.0), (1_000_003, 700.0)]):
        x = W.float64_normal(r, n)
        lens = W.with_empty(r, W.geometric_lengths(r, n, mean), 0.1)
        got, want = _scan_both(R, x, lens)
        # both are decoupled look-back scans; float64 sums may differ only by
        # reassociation, within the parity tolerance the other tests use
        compare("sum", got, want, seg_abs_prefix(x, lens))
        assert np.isfinite(got).all(), f"call {call}"


def test_noalloc_single_segment(gpu):
    R = DeviceRunner(load())
    r = W.rng(78)
    x = W.float64_normal(r, 123_457)
    got, want = _scan_both(R, x, np.array([len(x)], dtype=np.int32))
    compare("sum", got, want, seg_abs_prefix(x, [len(x)]))


def test_noalloc_rejects_too_large(gpu):
    c = load()
    limit = c.gcvl_add_sed_noalloc_max_n()
    assert limit == 1 << 28
    d = DeviceVector(c, 1, "d")
    c.gcvl_clear_error()
    rc = c.gcvl_add_sed_noalloc(d.ptr, d.ptr, None, limit + 1, 1)
    assert rc == 5
    assert "outside" in c.gcvl_error_string().decode()
    c.gcvl_clear_error()
