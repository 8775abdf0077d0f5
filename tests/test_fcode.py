"""Fused super-ops (neslgpu_gb300/fcode.py): definitions in the fusion
compiler's notation parsed into expressions, generated as sm_103a CUDA and
compiled; on the GPU, each super-op against the chain of CVL elementwise
calls it replaces, and the fused quicksort program against the plain one."""
import glob
import os

import numpy as np
import pytest

from neslgpu_gb300 import fcode as F
from neslgpu_gb300 import vcode as V
from neslgpu_gb300 import vcode_programs as P

REF_CU = sorted(glob.glob("/root/reference/bench/NESL/*.cu"))


def test_parse_and_emit_qsort_defs():
    ops = F.parse_defs(P.QSORT_FUSED_DEFS)
    assert [o.number for o in ops] == [0, 1, 2, 3, 4, 5]
    assert [o.result for o in ops] == ["INT", "INT", "INT", "INT", "INT", "BOOL"]
    assert ops[4].params[-1] == (6, "INT")
    src = F.emit_cuda(ops)
    assert src.count("__global__") == 6 and "f_div_z::f(x0, (2))" in src


def test_rejects_what_cannot_be_fused():
    with pytest.raises(F.FcodeError):
        F.parse_defs("fused OP0#1 ($0 : INT, $1 : SEGDES) = (+_SCAN INT @ $0 $1)")
    with pytest.raises(F.FcodeError):
        F.parse_defs("fused OP0#1 ($0 : INT, $1 : SEGDES) = (DIST INT @ $0 $1)")


@pytest.mark.skipif(not REF_CU, reason="the reference tree is not present")
def test_reference_definitions_parse_and_compile(tmp_path):
    """Every super-op definition of the reference's fused benchmarks parses,
    and a library generated from a few of them compiles for sm_103a."""
    total = 0
    for f in REF_CU:
        txt = open(f).read()
        if "fused OP" in txt:
            total += len(F.parse_defs(txt))
    assert total > 500
    for name in ("qs.1000.cu", "black-scholes.10000000.cu"):
        path = os.path.join(os.path.dirname(REF_CU[0]), name)
        assert F.build_library(F.parse_defs(open(path).read()), tmp_path).exists()


@pytest.mark.gpu
def test_super_ops_match_their_chains(gpu):
    c = gpu.cvl
    lib = F.FusedLib(P.QSORT_FUSED_DEFS)
    r = np.random.default_rng(3)
    n = 100_003
    a = r.integers(-50, 50, size=n).astype(np.int32)
    b = r.integers(-50, 50, size=n).astype(np.int32)
    args7 = [r.integers(0, 2, size=n).astype(np.int32) for _ in range(2)] + \
        [r.integers(-10 ** 6, 10 ** 6, size=n).astype(np.int32) for _ in range(5)]
    it = V.Interpreter("FUNC MAIN RET", c, fused=lib)
    try:
        def run(k, host_args):
            vs = [it.from_host("I", x) for x in host_args]
            d = it.new(lib.result_kind(k), n)
            lib.fn[k](d.ptr, *[v.ptr for v in vs], n, None)
            out = it.to_host(d)
            for v in vs + [d]:
                it.drop(v)
            return out
        np.testing.assert_array_equal(run(1, [a, b]), (a < b).astype(np.int32))
        np.testing.assert_array_equal(run(2, [a, b]), (a == b).astype(np.int32))
        np.testing.assert_array_equal(run(3, [a, b]), (a > b).astype(np.int32))
        lt, eq, plt, peq0, dlt, pgt0, dlteq = args7
        want = np.where(lt != 0, plt, np.where(eq != 0, peq0 + dlt, pgt0 + dlteq)).astype(np.int32)
        np.testing.assert_array_equal(run(4, args7), want)
        # a segment-descriptor argument gives the length; the constant is distributed
        sdv = it.from_host("I", [n])
        sd = it.segdes_from_lengths(sdv)
        x = it.from_host("I", a)
        d = it.new("I", n)
        lib.fn[0](d.ptr, x.ptr, sd.ptr, n, None)
        np.testing.assert_array_equal(it.to_host(d), (np.trunc(a / 2)).astype(np.int32))
    finally:
        it.free_all()


@pytest.mark.gpu
@pytest.mark.parametrize("n", [0, 5, 100_003, (1 << 20) + 3])
def test_fused_quicksort_matches_plain(gpu, n):
    c = gpu.cvl
    text, defs = P.qsort_fcode_program()
    lib = F.FusedLib(defs)
    keys = np.random.default_rng(n).integers(-2 ** 31, 2 ** 31, size=n, dtype=np.int64).astype(np.int32)
    if n == 100_003:
        keys = keys % 7  # ties
    it = V.Interpreter(text, c, fused=lib)
    try:
        lv = it.from_host("I", [n])
        sd = it.segdes_from_lengths(lv)
        it.drop(lv)
        st = it.run("QSORT", [sd, it.from_host("I", keys)])
        np.testing.assert_array_equal(it.to_host(st[-1]), np.sort(keys))
    finally:
        it.free_all()
