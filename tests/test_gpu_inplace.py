"""Scans in place: every scan declares that its output may be its input
(`*_inplace` returns 1, as in the serial CVL), which vinterp uses to reuse a
vector.  The ring scan reads each tile through TMA before it writes that
tile, so the result must equal the out-of-place call: bit for bit for
integer, min/max and xor scans; for float64 + within the sum tolerance,
since the decoupled look-back combines earlier tiles' aggregates in the
order their status words happen to be published (two runs may differ in
the last bits).  Checked on 16-byte aligned vectors (the ring) and 8 bytes
off (the generic kernel), past a thousand tiles, with the oracle on the
same inputs."""
import numpy as np
import pytest

from cases import compare, seg_abs_prefix
from neslgpu_gb300 import ops
from neslgpu_gb300 import workloads as W

pytestmark = pytest.mark.gpu

SCANS = [("add_sed", "d"), ("add_sez", "z"), ("max_sed", "d"), ("min_sez", "z"), ("xor_sez", "z")]


def _inplace_scan(R, name, x, lengths, unsegmented):
    k = ops._kind(name)
    n = len(x)
    a = R.vec(x, k)
    if unsegmented:
        scr = R.units(R.fn(name + "_scratch")(n))
        R.fn(name)(R.p(a), R.p(a), n, R.p(scr))
    else:
        sd, n, m = R.segd(lengths)
        scr = R.units(R.fn(name + "_scratch")(n, m))
        R.fn(name)(R.p(a), R.p(a), R.p(sd), n, m, R.p(scr))
    r = R.get(a, n)
    R.done()
    return r


@pytest.mark.parametrize("offset", [0, 1])
@pytest.mark.parametrize("n", [4097, (1 << 21) + 13])
def test_scans_in_place(gpu, oracle, n, offset):
    from neslgpu_gb300.cvl import load
    R = ops.DeviceRunner(load(), offset=offset)
    r = W.rng(70 + offset)
    lens = W.lognormal_lengths(r, n, 7.0, 2.0, n)
    xd = W.float64_normal(r, n)
    xz = W.int32_uniform(r, n)
    for name, t in SCANS:
        x = xd if t == "d" else xz
        for seg in (True, False):
            nm = name if seg else name.replace("_se", "_su")
            got = _inplace_scan(R, nm, x, lens, not seg)
            ref = ops.scan_e(R, nm, x, lens) if seg else ops.scan_u(R, nm, x)
            L = lens if seg else np.array([n], dtype=np.int32)
            want = ops.scan_e(oracle, nm, x, lens) if seg else ops.scan_u(oracle, nm, x)
            if nm.startswith("add_") and t == "d":
                S = seg_abs_prefix(x, L)
                compare("sum", got, ref, S)
                compare("sum", got, want, S)
            else:
                assert np.array_equal(np.asarray(got).view(np.uint8), np.asarray(ref).view(np.uint8)), nm
                compare("exact", got, want)
