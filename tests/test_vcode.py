"""The VCODE interpreter (neslgpu_gb300/vcode.py) and this repository's own
VCODE programs (quicksort, sparse matrix-vector product): on the oracle
here, on the GPU library under -m gpu.  Where the reference tree is
present, the interpreter also runs the NESL compiler's own quicksort VCODE
(bench/NESL/qs.1000000.vcode) on the oracle."""
import os

import numpy as np
import pytest

from neslgpu_gb300 import vcode as V
from neslgpu_gb300 import vcode_programs as P

from oracle.oracle import reference_root

_REF = reference_root()
REF_QS = str(_REF / "bench" / "NESL" / "qs.1000000.vcode") if _REF else ""


def _sort(cvl, keys, text=None, entry="QSORT"):
    it = V.Interpreter(text or P.qsort_program(), cvl)
    try:
        lv = it.from_host("I", [len(keys)])
        sd = it.segdes_from_lengths(lv)
        it.drop(lv)
        st = it.run(entry, [sd, it.from_host("I", keys)])
        assert len(st) == 2 and st[0].kind == "S" and st[1].kind == "I"
        return it.to_host(st[-1])
    finally:
        it.free_all()


def _spmv(cvl, lens, cols, vals, x):
    it = V.Interpreter(P.spmv_program(), cvl)
    try:
        lv = it.from_host("I", lens)
        rsd = it.segdes_from_lengths(lv)
        it.drop(lv)
        st = it.run("SPMV", [rsd, it.from_host("I", cols), it.from_host("F", vals), it.from_host("F", x)])
        assert len(st) == 1
        return it.to_host(st[0])
    finally:
        it.free_all()


def _keys(n, seed, ties=False):
    r = np.random.default_rng(seed)
    if ties:
        return r.integers(-3, 3, size=n).astype(np.int32)
    return r.integers(-2 ** 31, 2 ** 31, size=n, dtype=np.int64).astype(np.int32)


def _csr(rows, ncols, seed):
    r = np.random.default_rng(seed)
    lens = np.minimum(r.zipf(2.1, size=rows), 64).astype(np.int32)
    lens[r.random(rows) < 0.05] = 0  # some empty rows
    nnz = int(lens.sum())
    return lens, r.integers(0, ncols, size=nnz).astype(np.int32), r.normal(size=nnz), r.normal(size=ncols)


def _spmv_numpy(lens, cols, vals, x):
    starts = np.cumsum(lens) - lens
    return np.array([np.dot(vals[s:s + l], x[cols[s:s + l]]) for s, l in zip(starts, lens)])


def test_parse_control_flow():
    prog, funcs, main = V.parse("""
    { a comment } FUNC MAIN
    CONST BOOL T IF CONST INT 1 ELSE CONST INT 2 ENDIF
    CONST INT (1 2 3) RET
    FUNC OTHER I INT O INT RET""")
    assert main == "MAIN" and set(funcs) == {"MAIN", "OTHER"}
    ops = [i.op for i in prog]
    assert ops[:7] == ["CONST", "IF", "CONST", "ELSE", "CONST", "ENDIF", "CONSTV"]
    assert prog[1].b == 4 and prog[3].b == 5  # IF false -> else branch; ELSE -> ENDIF


@pytest.mark.parametrize("n,ties", [(0, False), (1, False), (2, False), (7, False), (5000, True), (40_000, False)])
def test_quicksort_on_oracle(oracle, n, ties):
    keys = _keys(n, n, ties)
    np.testing.assert_array_equal(_sort(oracle.cvl, keys), np.sort(keys))


def test_spmv_on_oracle(oracle):
    lens, cols, vals, x = _csr(300, 200, 3)
    np.testing.assert_allclose(_spmv(oracle.cvl, lens, cols, vals, x), _spmv_numpy(lens, cols, vals, x),
                               rtol=1e-12, atol=1e-12)


@pytest.mark.skipif(not os.path.exists(REF_QS), reason="the reference tree is not present")
def test_reference_quicksort_vcode_on_oracle(oracle):
    """The NESL compiler's own quicksort VCODE, QUICKSORT_3 called on our
    keys: the interpreter runs real compiler output."""
    text = open(REF_QS).read()
    keys = _keys(20_000, 9)
    np.testing.assert_array_equal(_sort(oracle.cvl, keys, text, "QUICKSORT_3"), np.sort(keys))


@pytest.mark.gpu
@pytest.mark.parametrize("n,ties", [(0, False), (3, False), (100_003, True), ((1 << 20) + 7, False)])
def test_quicksort_on_gpu(gpu, oracle, n, ties):
    keys = _keys(n, 100 + n, ties)
    got = _sort(gpu.cvl, keys)
    np.testing.assert_array_equal(got, np.sort(keys))
    if n <= 100_003:  # and the same program on the oracle gives the same vector
        np.testing.assert_array_equal(got, _sort(oracle.cvl, keys))


@pytest.mark.gpu
def test_spmv_on_gpu(gpu, oracle):
    lens, cols, vals, x = _csr(20_000, 5_000, 4)
    got = _spmv(gpu.cvl, lens, cols, vals, x)
    want = _spmv(oracle.cvl, lens, cols, vals, x)
    starts = np.cumsum(lens) - lens
    S = np.array([np.abs(vals[s:s + l] * x[cols[s:s + l]]).sum() for s, l in zip(starts, lens)])
    assert np.all(np.abs(got - want) <= 1e-12 * np.maximum(np.abs(want), S) + 1e-300)


def _long_rows_csr(rows, ncols, seed):
    """Rows of about 600 nonzeros: the unchained fold."""
    r = np.random.default_rng(seed)
    lens = r.integers(1, 1200, size=rows).astype(np.int32)
    lens[r.random(rows) < 0.05] = 0
    nnz = int(lens.sum())
    return lens, r.integers(0, ncols, size=nnz).astype(np.int32), r.normal(size=nnz), r.normal(size=ncols)


@pytest.mark.gpu
@pytest.mark.parametrize("case,offset", [("short", 0), ("short", 1), ("long", 0), ("many", 0)])
def test_fused_spmv_matches_vcode_program(gpu, oracle, case, offset):
    """gcvl_spmv_csr (gather, multiply and per-row sum in one pass) against
    the SPMV VCODE program on the oracle: power-law rows (the chained fold
    for short rows), rows of about 600 nonzeros, vectors off a 16-byte
    boundary (the form without TMA), and 2.8 million nonzeros (rows across
    about 1,400 tiles)."""
    from neslgpu_gb300.cvl import load
    from neslgpu_gb300.ops import DeviceRunner
    R = DeviceRunner(load(), offset=offset)
    c = R.cvl
    lens, cols, vals, x = {"short": lambda: _csr(30_000, 7_000, 5), "long": lambda: _long_rows_csr(3_000, 50_000, 6),
                           "many": lambda: _csr(1_000_003, 1 << 21, 7)}[case]()
    sd, nnz, rows = R.segd(lens)
    cv, vv, xv = R.vec(cols, "z"), R.vec(vals, "d"), R.vec(x, "d")
    y = R.out(rows, "d")
    scr = R.units(c.gcvl_spmv_csr_scratch(nnz, rows))
    c.gcvl_spmv_csr(y.ptr, vv.ptr, cv.ptr, xv.ptr, sd.ptr, nnz, rows, scr.ptr)
    got = R.get(y, rows)
    R.done()
    nz = lens > 0
    starts = (np.cumsum(lens, dtype=np.int64) - lens)[nz]
    prod = vals * x[cols]

    def row_sums(v):  # per row, empty rows 0
        out = np.zeros(rows)
        out[nz] = np.add.reduceat(v, starts)
        return out
    S = row_sums(np.abs(prod))
    # the oracle's VCODE run at 2.8 million nonzeros takes too long: numpy row sums there
    want = row_sums(prod) if case == "many" else _spmv(oracle.cvl, lens, cols, vals, x)
    assert np.all(np.abs(got - want) <= 1e-12 * np.maximum(np.abs(want), S) + 1e-300)
    assert np.all(got[lens == 0] == 0.0)
