"""Known answers of the reference's NESL test suite
(nesl/neslsrc/test.nesl), restated at the CVL level, on the oracle (CPU)
and on the GPU library."""
import json
from pathlib import Path

import numpy as np
import pytest

from neslgpu_gb300 import ops

KA = json.loads((Path(__file__).parent / "golden" / "known_answers.json").read_text())


def run_case(R, c):
    f = c["call"]
    a = c["args"]
    if f == "scan_u":
        return ops.scan_u(R, c["fn"], np.array(a[0]))
    if f == "reduce_u":
        return np.asarray(ops.reduce_u(R, c["fn"], np.array(a[0])))
    if f == "reduce_e":
        return ops.reduce_e(R, c["fn"], np.array(a[0]), np.array(a[1]))
    if f == "scan_e":
        return ops.scan_e(R, c["fn"], np.array(a[0]), np.array(a[1]))
    if f == "smp_u":
        return ops.smp_u(R, c["fn"], np.array(a[0]), np.array(a[1]))
    if f == "dpe_u":
        return ops.dpe_u(R, c["fn"], np.array(a[0]), np.array(a[1]), np.array(a[2]))
    if f == "dfp_u":
        return ops.fpm_u(R, c["fn"], np.array(a[0]), np.array(a[1]), np.array(a[2]), len(a[3]), np.array(a[3]))
    if f == "bck_u":
        return ops.bck_u(R, c["fn"], np.array(a[0]), np.array(a[1]))
    if f == "pack_u":
        return ops.pack_u(R, c["fn"], np.array(a[0]), np.array(a[1]))
    if f == "rank_u":
        return ops.rank_u(R, c["fn"], np.array(a[0]))
    if f == "dis_e":
        return ops.dis_e(R, c["fn"], np.array(a[0]), np.array(a[1]))
    if f == "ew1":
        return ops.ew1(R, c["fn"], np.array(a[0]))
    raise ValueError(f)


def _check(R):
    for c in KA["cases"]:
        got = np.asarray(run_case(R, c))
        want = np.asarray(c["want"])
        if want.dtype.kind == "f" or c["fn"].endswith("d") and c["call"] not in ("rank_u",):
            ok = np.allclose(got, want, rtol=0, atol=0)
        else:
            ok = np.array_equal(got.astype(np.int64), want.astype(np.int64))
        assert ok, f"{c['what']} ({c['source']}): got {got.tolist()} want {want.tolist()}"


def test_known_answers_oracle(oracle):
    _check(oracle)


@pytest.mark.gpu
def test_known_answers_gpu(gpu):
    _check(gpu)
