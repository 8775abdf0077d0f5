"""Float64 parity at the benchmark's own configuration: add_sed and add_red
over 2^28 float64 N(0,1) values (generated on the device from the
benchmark's seed) with segment lengths round(LogNormal(5, 2)) clipped to
[1, 2^24], against the oracle (the CPU restatement of the serial CVL,
nesl/cvl/serial/vprims.c:62-109 and :155-201) on the same values.

Tolerance, per element: |gpu - serial| <= 1e-12 * max(|serial|, S), with S
the sum of |x| over the same prefix (scan) or segment (reduction): the
kernels reassociate float64 sums, and a bound relative to |serial| alone is
ill-conditioned for N(0,1) sums that cancel to about 0."""
import numpy as np
import pytest

from cases import sum_err_over_tol
from neslgpu_gb300 import workloads as W
from neslgpu_gb300.cvl import DeviceVector

pytestmark = pytest.mark.gpu

SEED = 0x5EED + 1  # the benchmark's seed for the values and the lengths


def test_add_sed_add_red_2e28_lognormal(gpu, oracle):
    c = gpu.cvl
    n = 1 << 28
    lens = W.lognormal_lengths(W.rng(SEED), n, 5.0, 2.0, 1 << 24)
    m = len(lens)
    assert int(lens.sum(dtype=np.int64)) == n and lens.min() >= 1 and lens.max() <= 1 << 24
    x = DeviceVector(c, n, "d")
    c.gcvl_fill_random(x.ptr, n, 1, SEED, 0.0, 0)
    sd, _, _ = gpu.segd(lens)
    ys = DeviceVector(c, n, "d")
    yr = DeviceVector(c, m, "d")
    scr = gpu.units(max(c.add_sed_scratch(n, m), c.add_red_scratch(n, m)))
    c.add_sed(ys.ptr, x.ptr, sd.ptr, n, m, scr.ptr)
    c.add_red(yr.ptr, x.ptr, sd.ptr, n, m, scr.ptr)
    gpu.done()
    xh = x.numpy(n)
    gs = ys.numpy(n)
    gr = yr.numpy(m)
    del x, ys, yr
    o = oracle.cvl
    ws = np.empty(n)
    wr = np.empty(m)
    o.add_sed(ws.ctypes.data, xh.ctypes.data, lens.ctypes.data, n, m, None)
    o.add_red(wr.ctypes.data, xh.ctypes.data, lens.ctypes.data, n, m, None)
    assert np.isfinite(gs).all() and np.isfinite(gr).all()
    e_scan = sum_err_over_tol(gs, ws, xh, lens, "scan")
    e_red = sum_err_over_tol(gr, wr, xh, lens, "reduce")
    assert e_scan <= 1.0, f"add_sed: max err/tol {e_scan:.3g}"
    assert e_red <= 1.0, f"add_red: max err/tol {e_red:.3g}"
