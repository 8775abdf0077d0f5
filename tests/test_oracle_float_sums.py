"""The oracle against the reference's own serial CVL (built from its
sources into oracle/_ref) on the float64 sum inputs the GPU tests use:
magnitudes 2^-60..2^60 within segments, zeros, subnormals, values near
1e290, and infinities and NaNs -- so the GPU's special-value results are
checked against an oracle pinned on exactly those cases."""
import numpy as np
import pytest

import test_gpu_float_sums as F
from neslgpu_gb300 import ops
from neslgpu_gb300 import workloads as W

N = 100_003


@pytest.mark.parametrize("specials", [False, True])
@pytest.mark.parametrize("kind", ["geo", "tiny", "long"])
def test_oracle_matches_reference_on_float_sums(reference, oracle, kind, specials):
    r = W.rng(900 + 7 * specials + len(kind))
    x = F._values(r, N, specials)
    lens = F._lengths(r, N, kind)
    for name, fn, exclusive in (("add_sed", ops.scan_e, True), ("add_red", ops.reduce_e, False)):
        F._check(fn(oracle, name, x, lens), fn(reference, name, x, lens), F._seg_abs(x, lens, exclusive))
    one = np.array([N], dtype=np.int32)
    F._check(ops.scan_u(oracle, "add_sud", x), ops.scan_u(reference, "add_sud", x), F._seg_abs(x, one, True))
    F._check(ops.reduce_u(oracle, "add_rud", x), ops.reduce_u(reference, "add_rud", x), F._seg_abs(x, one, False))
