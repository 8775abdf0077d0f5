"""The reference's own known-answer suite (nesl/neslsrc/test.nesl, compiled
to nesl/vcode/nesltest.vcode and run by `make test` in nesl/vcode).

* Where the reference tree is present, the suite runs on the oracle through
  this repository's VCODE interpreter.  Every check passes except two:
  - "checking the fail mechanism", which fails on purpose;
  - "rand (within range)", which expects rand(100) > 0.  The reference
    itself fails that check on Linux: its serial CVL draws from glibc's
    unseeded lrand48, whose first value is 0 (CVL_init's rnd_foz(0) is
    srandom(0) there, nesl/cvl/serial/facilt.c:292-319).
  The fresh run's report must also equal the one stored in the golden
  trace, so the trace belongs to this interpreter and oracle.
* tests/golden/nesltest_trace.npz (tests/golden/make_nesltest_trace.py)
  records every vector instruction of that run: primitive, type, the values
  it consumed and produced.  The trace is replayed instruction by
  instruction, with the recorded inputs, on the oracle (here) and on the
  GPU library (-m gpu).  Results must be bit-identical, except for float64
  results of sums, products and CUDA's transcendental functions, which are
  compared within the library's float64 tolerances.  RAND draws the same
  stream: replay starts from the unseeded state, and every SRAND and RAND
  of the suite is replayed in order.
"""
import sys
from pathlib import Path

import numpy as np
import pytest

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE / "golden"))
import make_nesltest_trace as T  # noqa: E402

from neslgpu_gb300 import vcode as V  # noqa: E402

from oracle.oracle import reference_root  # noqa: E402

_REF = reference_root()
REF_SUITE = _REF / "nesl" / "vcode" / "nesltest.vcode" if _REF else Path("/nonexistent")
EXPECTED_FAILED = ["checking the fail mechanism, failed message should appear", "rand (within range)"]
SUMS = {"+_SCAN", "*_SCAN", "+_REDUCE", "*_REDUCE"}
TRANSCENDENTAL = {"EXP", "LOG", "SIN", "COS", "TAN", "ASIN", "ACOS", "ATAN", "SINH", "COSH", "TANH"}


def _failed(report):
    return [ln[: -len("........failed")].strip() for ln in report.splitlines() if ln.endswith("........failed")]


@pytest.mark.skipif(not REF_SUITE.exists(), reason="the reference tree is not present")
def test_suite_on_oracle_passes_and_matches_trace():
    records, report = T.record(REF_SUITE.read_text(encoding="latin-1"))
    assert _failed(report) == EXPECTED_FAILED, _failed(report)
    assert "spawn" in report and "write-read string test" in report  # ran to the end
    stored_records, stored_report = T.load()
    assert report == stored_report
    assert [r[:2] for r in records] == [r[:2] for r in stored_records]


def _push(it, kind, seg_len, vals):
    if kind == "S":
        lv = it.from_host("I", vals)
        v = it.segdes_from_lengths(lv)
        it.drop(lv)
        assert v.seg_len == seg_len
        return v
    return it.from_host(kind, vals)


def _tolerance(op, want, consumed):
    """None: bit-identical; else the allowed |got - want| per element."""
    if want.dtype != np.float64:
        return None
    if op in SUMS:
        # a sum or product of any of the inputs: relative to the magnitudes
        mag = sum(float(np.abs(v).sum()) for k, _, v in consumed if k == "F")
        return 1e-12 * np.maximum(np.abs(want), mag) + 1e-300
    if op in TRANSCENDENTAL:
        return 1e-13 * np.abs(want) + 1e-300
    return None


def replay(cvl, records, set_unseeded):
    """Runs each recorded instruction with its recorded inputs on cvl;
    returns the number of instructions checked."""
    it = V.Interpreter("FUNC MAIN RET", cvl)
    set_unseeded()
    try:
        for i, (op, typ, consumed, produced) in enumerate(records):
            it.stack = [_push(it, *e) for e in consumed]
            it._vector_op(V.Ins(op, typ, line=i))
            got = [(v.kind, v.seg_len, it.to_host(v)) for v in it.stack]
            assert len(got) == len(produced), f"#{i} {op} {typ}: {len(got)} results"
            for (gk, gs, gv), (wk, ws, wv) in zip(got, produced):
                assert gk == wk and gs == ws and len(gv) == len(wv), f"#{i} {op} {typ}: result shape"
                tol = _tolerance(op, wv, consumed)
                if tol is None:
                    same = gv.view(np.int64) == wv.view(np.int64) if wv.dtype == np.float64 else gv == wv
                    assert np.all(same), f"#{i} {op} {typ}: {gv[~same][:4]} != {wv[~same][:4]}"
                else:
                    ok = (np.abs(gv - wv) <= tol) | (gv == wv) | (np.isnan(gv) & np.isnan(wv))
                    assert np.all(ok), f"#{i} {op} {typ}: {gv[~ok][:4]} vs {wv[~ok][:4]}"
            for v in it.stack:
                it.drop(v)
            it.stack = []
        return len(records)
    finally:
        it.free_all()


def test_trace_replays_on_oracle(oracle):
    records, _ = T.load()
    o = oracle.cvl
    zero = np.zeros(1, dtype=np.uint64)
    assert replay(o, records, lambda: o.lib.ocvl_rnd_state(None, zero.ctypes.data)) > 20000


@pytest.mark.gpu
def test_trace_replays_on_gpu(gpu):
    records, report = T.load()
    assert _failed(report) == EXPECTED_FAILED
    c = gpu.cvl
    n = replay(c, records, lambda: c.gcvl_set_rand_state(0))
    assert n == len(records)
    assert len({r[0] for r in records}) > 50  # the primitive families the suite exercises
