"""gcvl_add_sed_noalloc: the segmented float64 +-scan for callers that may
not allocate device memory -- embedders whose device memory all belongs to
their own pool, runtimes that forbid allocation after start-up.  It keeps its
scratch in a fixed array inside the library (2,097,664 bytes, at most 2^28
elements), shared by every call.

Checked here through the C ABI against the oracle (the CPU restatement of
the serial CVL) with the float64 sum tolerance of every other parity test,
and against the ordinary add_sed, on two calls in a row (the array keeps the
previous call's contents, which each call must clear), on the TMA and the
unaligned path; a bounded wait that gives up must be reported by gcvl_sync;
sizes beyond the maximum are rejected.

This file is collected last so that a failure here, in a run that stops at
the first failure, comes after every other test."""
import numpy as np
import pytest

from cases import compare, seg_abs_prefix
from neslgpu_gb300 import ops, workloads as W
from neslgpu_gb300.cvl import DeviceVector, load
from neslgpu_gb300.ops import DeviceRunner


def _noalloc(R, x, lens):
    """(gcvl_add_sed_noalloc result, add_sed result) for the same inputs."""
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


@pytest.mark.gpu
@pytest.mark.parametrize("offset", [0, 1])
def test_noalloc_matches_oracle_twice(gpu, oracle, offset):
    R = DeviceRunner(load(), offset=offset)  # offset 1: not 16-byte aligned
    r = W.rng(77)
    for call, (n, mean) in enumerate([(300_007, 40.0), (1_000_003, 700.0)]):
        x = W.float64_normal(r, n)
        lens = W.with_empty(r, W.geometric_lengths(r, n, mean), 0.1)
        got, plain = _noalloc(R, x, lens)
        want = ops.scan_e(oracle, "add_sed", x, lens)
        S = seg_abs_prefix(x, lens)
        compare("sum", got, want, S)    # |a-b| <= 1e-12 * max(|b|, S)
        compare("sum", got, plain, S)
        assert np.isfinite(got).all(), f"call {call}"


@pytest.mark.gpu
def test_noalloc_single_segment(gpu, oracle):
    R = DeviceRunner(load())
    r = W.rng(78)
    x = W.float64_normal(r, 123_457)
    one = np.array([len(x)], dtype=np.int32)
    got, _ = _noalloc(R, x, one)
    compare("sum", got, ops.scan_e(oracle, "add_sed", x, one), seg_abs_prefix(x, one))


@pytest.mark.gpu
def test_noalloc_timeout_is_reported(gpu, oracle):
    """With the wait limit forced to 1 the look-back waits give up at once:
    gcvl_sync must then report error 3, or, if no wait ran out, the result
    must be right.  Restoring the limit gives correct results again."""
    c = gpu.cvl
    old = c.gcvl_get_spin_limit()
    r = W.rng(79)
    n = 1 << 22
    x = W.float64_normal(r, n)
    one = np.array([n], dtype=np.int32)
    want = ops.scan_e(oracle, "add_sed", x, one)
    S = seg_abs_prefix(x, one)
    c.gcvl_sync()
    c.gcvl_clear_error()
    R = DeviceRunner(c, checked=False)
    sd, _, m = R.segd(one)
    xs = R.vec(x, "d")
    got = R.out(n, "d")
    assert c.gcvl_sync() == 0
    try:
        c.gcvl_set_spin_limit(1)
        assert c.gcvl_add_sed_noalloc(got.ptr, xs.ptr, sd.ptr, n, m) == 0
        code = c.gcvl_sync()
        assert code in (0, 3)
        if code == 3:
            assert "gcvl_add_sed_noalloc" in c.gcvl_error_string().decode()
        else:
            compare("sum", R.get(got, n), want, S)
    finally:
        c.gcvl_set_spin_limit(old)
        c.gcvl_clear_error()
    assert c.gcvl_sync() == 0  # the status word was cleared
    got, _ = _noalloc(DeviceRunner(c), x, one)
    compare("sum", got, want, S)


@pytest.mark.gpu
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


def test_noalloc_without_device_returns_error():
    """Where no GPU is visible the call cannot be issued: it must return a
    non-zero code and record why, not report success."""
    from conftest import _has_gpu
    if _has_gpu():
        pytest.skip("a GPU is visible")
    c = load()
    c.gcvl_clear_error()
    assert c.gcvl_add_sed_noalloc(None, None, None, 1024, 1) != 0
    assert c.gcvl_last_error() != 0 and c.gcvl_error_string()
    c.gcvl_clear_error()
