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

from oracle.oracle import reference_root

_REF = reference_root()
REF_CU = sorted(glob.glob(str(_REF / "bench" / "NESL" / "*.cu"))) if _REF else []


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


# Float64 super-ops in the fusion compiler's notation, written for these
# tests: the Black-Scholes call price as a few fused steps (d1, d2, the
# normal CDF's polynomial approximation with its exp, the sign select, the
# discounted price), plus conversions and trigonometric/hyperbolic chains.
FLOAT_DEFS = """
fused OP0#1 ($0 : FLOAT, $1 : FLOAT, $2 : FLOAT, $3 : FLOAT, $4 : FLOAT, $5 : SEGDES) = (/ FLOAT @
  (+ FLOAT @ (LOG @ (/ FLOAT @ $0 $1))
    (* FLOAT @ (+ FLOAT @ $2 (* FLOAT @ (* FLOAT @ $3 $3) (DIST FLOAT @ (CONST FLOAT 0.5) $5))) $4))
  (* FLOAT @ $3 (SQRT @ $4)))
fused OP1#1 ($0 : FLOAT, $1 : FLOAT, $2 : FLOAT) = (- FLOAT @ $0 (* FLOAT @ $1 (SQRT @ $2)))
fused OP2#1 ($0 : FLOAT, $1 : SEGDES) = (/ FLOAT @ (DIST FLOAT @ (CONST FLOAT 1.0) $1)
  (+ FLOAT @ (DIST FLOAT @ (CONST FLOAT 1.0) $1) (* FLOAT @ (DIST FLOAT @ (CONST FLOAT 0.2316419) $1)
    (SELECT FLOAT @ (< FLOAT @ $0 (DIST FLOAT @ (CONST FLOAT 0.0) $1)) (- FLOAT @ (DIST FLOAT @ (CONST FLOAT 0.0) $1) $0) $0))))
fused OP3#1 ($0 : FLOAT, $1 : FLOAT, $2 : SEGDES) = (- FLOAT @ (DIST FLOAT @ (CONST FLOAT 1.0) $2)
  (* FLOAT @ (* FLOAT @ (DIST FLOAT @ (CONST FLOAT 0.3989422804014327) $2)
      (EXP @ (* FLOAT @ (DIST FLOAT @ (CONST FLOAT -0.5) $2) (* FLOAT @ $0 $0))))
    (* FLOAT @ $1 (+ FLOAT @ (DIST FLOAT @ (CONST FLOAT 0.31938153) $2) (* FLOAT @ $1
      (+ FLOAT @ (DIST FLOAT @ (CONST FLOAT -0.356563782) $2) (* FLOAT @ $1
        (+ FLOAT @ (DIST FLOAT @ (CONST FLOAT 1.781477937) $2) (* FLOAT @ $1
          (+ FLOAT @ (DIST FLOAT @ (CONST FLOAT -1.821255978) $2)
            (* FLOAT @ $1 (DIST FLOAT @ (CONST FLOAT 1.330274429) $2))))))))))))
fused OP4#1 ($0 : FLOAT, $1 : FLOAT, $2 : SEGDES) = (SELECT FLOAT @ (< FLOAT @ $0 (DIST FLOAT @ (CONST FLOAT 0.0) $2))
  (- FLOAT @ (DIST FLOAT @ (CONST FLOAT 1.0) $2) $1) $1)
fused OP5#1 ($0 : FLOAT, $1 : FLOAT, $2 : FLOAT, $3 : FLOAT, $4 : FLOAT, $5 : FLOAT, $6 : SEGDES) = (- FLOAT @
  (* FLOAT @ $0 $1) (* FLOAT @ (* FLOAT @ $2 (EXP @ (- FLOAT @ (DIST FLOAT @ (CONST FLOAT 0.0) $6) (* FLOAT @ $3 $4)))) $5))
fused OP6#1 ($0 : FLOAT, $1 : FLOAT) = (+ INT @ (+ INT @ (FLOOR @ $0) (CEIL @ $1))
  (+ INT @ (ROUND @ $0) (+ INT @ (TRUNC @ $1) (B_TO_I @ (< FLOAT @ $0 $1)))))
fused OP7#1 ($0 : FLOAT, $1 : FLOAT) = (+ FLOAT @ (SIN @ $0) (* FLOAT @ (COS @ $1) (ATAN @ (/ FLOAT @ $0 $1))))
fused OP8#1 ($0 : FLOAT, $1 : FLOAT) = (- FLOAT @ (TANH @ $0) (/ FLOAT @ (SINH @ $1) (COSH @ $0)))
fused OP9#1 ($0 : INT, $1 : FLOAT, $2 : SEGDES) = (* FLOAT @ (I_TO_F @ $0) (TAN @ (ASIN @ (/ FLOAT @ $1 (DIST FLOAT @ (CONST FLOAT 4.0) $2)))))
fused OP10#1 ($0 : FLOAT, $1 : FLOAT) = (OR BOOL @ (= FLOAT @ $0 $1) (NOT @ (I_TO_B @ (TRUNC @ (ACOS @ $1)))))
"""

_TRANSCENDENTAL = {"LOG", "SQRT", "EXP", "SIN", "COS", "TAN", "ASIN", "ACOS", "ATAN", "SINH", "COSH", "TANH"}


def _has_transcendental(node):
    return (node.kind == "op" and node.op in _TRANSCENDENTAL and node.op != "SQRT") or \
        any(_has_transcendental(a) for a in node.args)


def _chain(R, node, args, n):
    """Evaluate a super-op's expression as the chain of CVL calls it
    replaces (dis_vu*, *_wu*, sel_wu*) on runner R."""
    from neslgpu_gb300 import ops
    if node.kind == "arg":
        return args[node.index]
    if node.kind == "dist":
        c = node.args[0]
        sfx = F.SFX[c.typ]
        val = float(c.value) if c.typ == "FLOAT" else (1 if c.value in ("T", "1") else 0) if c.typ == "BOOL" \
            else int(c.value)
        return ops.dis_u(R, f"dis_vu{sfx}", val, n)
    if node.kind == "select":
        f, a, b = (_chain(R, x, args, n) for x in node.args)
        return ops.sel(R, f"sel_wu{F.SFX[node.optype]}", f, a, b)
    stem = F.OPS[node.op][0]
    name = f"{stem}_wu{F.SFX[node.optype]}"
    xs = [_chain(R, a, args, n) for a in node.args]
    return ops.ew1(R, name, xs[0]) if len(xs) == 1 else ops.ew2(R, name, xs[0], xs[1])


def test_float_defs_parse():
    ops = F.parse_defs(FLOAT_DEFS)
    assert [o.number for o in ops] == list(range(11))
    assert [o.result for o in ops] == ["FLOAT"] * 6 + ["INT", "FLOAT", "FLOAT", "FLOAT", "BOOL"]


@pytest.mark.gpu
@pytest.mark.parametrize("n", [1, 1000, 300_007])
def test_float_super_ops_match_chains_and_oracle(gpu, oracle, n):
    """Each float64 super-op against (a) the same chain of CVL calls on the
    GPU -- bit-identical, the kernels share the element functions -- and
    (b) that chain on the oracle (libm): bit-identical where the expression
    uses only + - * / sqrt, conversions, compares and selects, else within
    |a - b| <= 1e-11 * max(1, |b|) (CUDA's and libm's exp/log/sin/... each
    round differently in the last bit, and the chain carries that on)."""
    from neslgpu_gb300.ops import DeviceRunner
    lib = F.FusedLib(FLOAT_DEFS)
    r = np.random.default_rng(n)
    S = r.uniform(10.0, 200.0, n)
    K = r.uniform(10.0, 200.0, n)
    rate = r.uniform(0.0, 0.1, n)
    vol = r.uniform(0.05, 0.8, n)
    T = r.uniform(0.05, 5.0, n)
    d = r.normal(0.0, 2.0, n)
    w = r.uniform(0.0, 1.0, n)
    big = r.normal(0.0, 50.0, n)
    ii = r.integers(-1000, 1000, size=n).astype(np.int32)
    inputs = {0: [S, K, rate, vol, T, "sd"], 1: [d, vol, T], 2: [d, "sd"], 3: [d, w, "sd"], 4: [d, w, "sd"],
              5: [S, w, K, rate, T, w, "sd"], 6: [big, d], 7: [d, S], 8: [d / 4, d], 9: [ii, w, "sd"],
              10: [np.where(r.random(n) < 0.1, w, d), w]}
    it = V.Interpreter("FUNC MAIN RET", gpu.cvl, fused=lib)
    G = DeviceRunner(gpu.cvl)
    try:
        for o in lib.ops:
            host = inputs[o.number]
            assert len(host) == len(o.params), o.number
            vs = []
            for (j, t), x in zip(o.params, host):
                if t == "SEGDES":
                    lv = it.from_host("I", [n])
                    vs.append(it.segdes_from_lengths(lv))
                    it.drop(lv)
                else:
                    vs.append(it.from_host(F.KIND[t], x))
            dst = it.new(lib.result_kind(o.number), n)
            lib.fn[o.number](dst.ptr, *[v.ptr for v in vs], n, None)
            got = it.to_host(dst)
            for v in vs + [dst]:
                it.drop(v)
            args = {j: (None if t == "SEGDES" else np.asarray(x)) for (j, t), x in zip(o.params, host)}
            on_gpu = _chain(G, o.expr, args, n)
            on_cpu = _chain(oracle, o.expr, args, n)
            if got.dtype == np.float64:
                np.testing.assert_array_equal(got.view(np.int64), on_gpu.view(np.int64), err_msg=f"OP{o.number}")
            else:
                np.testing.assert_array_equal(got, on_gpu, err_msg=f"OP{o.number}")
            if _has_transcendental(o.expr):
                tol = 1e-11 * np.maximum(1.0, np.abs(on_cpu))
                bad = ~((np.abs(got - on_cpu) <= tol) | (got == on_cpu))
                assert not bad.any(), f"OP{o.number}: {got[bad][:4]} vs {on_cpu[bad][:4]}"
            elif got.dtype == np.float64:
                np.testing.assert_array_equal(got.view(np.int64), on_cpu.view(np.int64), err_msg=f"OP{o.number}")
            else:
                np.testing.assert_array_equal(got, on_cpu, err_msg=f"OP{o.number}")
    finally:
        it.free_all()
