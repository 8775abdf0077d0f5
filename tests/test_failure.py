"""Failure detection without a GPU fault.  Every device wait in the library
is bounded: when it runs out the kernel records a status instead of hanging
and the host reads it as error 3 (timeout); the context stays usable.  Host
errors are recorded, never abort."""
import numpy as np
import pytest

from neslgpu_gb300 import ops, workloads as W


def test_host_error_is_recorded_not_fatal():
    from neslgpu_gb300.cvl import load
    c = load()
    c.gcvl_clear_error()
    assert c.alo_foz(-1) is None          # negative size (or no device): NULL, no abort
    assert c.gcvl_last_error() != 0
    assert c.gcvl_error_string()
    c.gcvl_clear_error()
    assert c.gcvl_last_error() == 0


@pytest.mark.gpu
def test_wait_that_nothing_releases_times_out(gpu):
    c = gpu.cvl
    c.gcvl_clear_error()
    assert c.gcvl_selftest_timeout(2000) == 3
    assert "bounded device wait" in c.gcvl_error_string().decode()
    c.gcvl_clear_error()
    # the context is still usable afterwards
    r = W.rng(3)
    x = W.int32_uniform(r, 10_000)
    lens = W.geometric_lengths(r, 10_000, 30)
    from oracle.oracle import HostRunner, load_oracle
    assert np.array_equal(ops.scan_e(gpu, "add_sez", x, lens),
                          ops.scan_e(HostRunner(load_oracle()), "add_sez", x, lens))


@pytest.mark.gpu
def test_injected_spin_limit_never_hangs(gpu):
    """With the wait limit forced to 1, look-back waits on tiles that have not
    published yet give up at once: the call finishes (correct or flagged),
    and after restoring the limit results are right again."""
    c = gpu.cvl
    old = c.gcvl_get_spin_limit()
    r = W.rng(4)
    n = 1 << 22
    x = W.float64_normal(r, n)
    one = np.array([n], dtype=np.int32)
    from cases import compare, seg_abs_prefix
    from oracle.oracle import HostRunner, load_oracle
    want = ops.scan_e(HostRunner(load_oracle()), "add_sed", x, one)
    S = seg_abs_prefix(x, one)
    try:
        c.gcvl_set_spin_limit(1)
        R = ops.DeviceRunner(c, checked=False)
        flagged = ops.scan_e(R, "add_sed", x, one)
        code = c.gcvl_sync()
        assert code in (0, 3)
        if code == 0:  # no wait ran out: the result must be right
            compare("sum", flagged, want, S)
        else:
            assert "bounded device wait" in c.gcvl_error_string().decode()
    finally:
        c.gcvl_set_spin_limit(old)
        c.gcvl_clear_error()
    compare("sum", ops.scan_e(gpu, "add_sed", x, one), want, S)
