"""Golden vectors from the reference's known-answer suite.

nesl/vcode/nesltest.vcode is the NESL compiler's VCODE for the reference's
test suite (nesl/neslsrc/test.nesl, run by `make test` in nesl/vcode).  This
script runs it on the oracle (the CPU restatement of the serial CVL) with
this repository's VCODE interpreter, starting from glibc's unseeded lrand48
state (0), and records every vector instruction it executes -- primitive,
type, the stack entries it consumed and the ones it produced, as values --
together with the suite's printed report.  The GPU test replays each
instruction with the recorded inputs on the GPU library and compares the
results (tests/test_known_answer_suite.py).  I/O instructions are not
recorded.  The program text itself is not stored.

    python tests/golden/make_nesltest_trace.py [reference root]

writes tests/golden/nesltest_trace.npz.  The reference root defaults to
the one oracle.oracle.reference_root() finds ($GCVL_REFERENCE, else the tree
`make -C oracle ref` was built from).
"""
from __future__ import annotations

import contextlib
import io
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

KIND_CODE = {"I": 0, "B": 1, "F": 2, "S": 3}


def record(program_text: str):
    """(records, report): records is a list of (op, typ, consumed, produced)
    with (kind, seg_len, values) entries; report the suite's printed text."""
    from neslgpu_gb300 import vcode as V
    from oracle.oracle import load_oracle
    o = load_oracle()
    zero = np.zeros(1, dtype=np.uint64)
    o.lib.ocvl_rnd_state(None, zero.ctypes.data)
    it = V.Interpreter(program_text, o)
    records = []
    it.trace = lambda op, typ, a, b: records.append((op, typ, a, b))
    out = io.StringIO()
    it.files[1] = V._VStream(out)
    with contextlib.redirect_stdout(out):
        it.run(None, [])
    return records, out.getvalue()


def pack(records, report):
    """Flatten the records: every distinct vector is stored once (integer
    vectors as differences of consecutive values, which compress well), and
    each record refers to its vectors by number.

      names      "op typ" strings (JSON)
      rec        per record: name number, entries consumed, entries produced
      ent        per entry: kind (0 int, 1 bool, 2 float, 3 segdes), element
                 count of a segdes (else -1), vector number
      vec        per vector: 0 int32 / 1 float64, offset, length
      ideltas    int32 vectors, first value then successive differences
      floats     float64 vectors
    """
    names, rec, ent, vec = {}, [], [], []
    ideltas, floats = [], []
    seen = {}
    ni = nf = 0

    def vector_id(kind, vals):
        nonlocal ni, nf
        is_f = kind == "F"
        a = np.ascontiguousarray(vals, dtype=np.float64 if is_f else np.int32)
        key = (is_f, a.tobytes())
        if key not in seen:
            seen[key] = len(vec)
            if is_f:
                vec.append((1, nf, len(a)))
                floats.append(a)
                nf += len(a)
            else:
                vec.append((0, ni, len(a)))
                ideltas.append(np.diff(a.astype(np.int64), prepend=0).astype(np.int32))
                ni += len(a)
        return seen[key]

    for op, typ, a, b in records:
        nm = f"{op} {typ or ''}".strip()
        rec.append((names.setdefault(nm, len(names)), len(a), len(b)))
        for kind, seg_len, vals in list(a) + list(b):
            ent.append((KIND_CODE[kind], -1 if seg_len is None else int(seg_len), vector_id(kind, vals)))
    return {
        "names": np.frombuffer(json.dumps(sorted(names, key=names.get)).encode(), dtype=np.uint8),
        "rec": np.asarray(rec, dtype=np.int32).reshape(-1, 3),
        "ent": np.asarray(ent, dtype=np.int32).reshape(-1, 3),
        "vec": np.asarray(vec, dtype=np.int64).reshape(-1, 3),
        "ideltas": np.concatenate(ideltas) if ideltas else np.zeros(0, np.int32),
        "floats": np.concatenate(floats) if floats else np.zeros(0, np.float64),
        "report": np.frombuffer(report.encode("latin-1"), dtype=np.uint8),
    }


def load(path=HERE / "nesltest_trace.npz"):
    """The records back: (records, report) as record() returns them."""
    d = np.load(path)
    names = json.loads(bytes(d["names"]).decode())
    ints = d["ideltas"]
    vec = d["vec"]
    kinds = {v: k for k, v in KIND_CODE.items()}
    cache = {}

    def values(vid):
        if vid not in cache:
            is_f, off, n = (int(x) for x in vec[vid])
            if is_f:
                cache[vid] = d["floats"][off:off + n]
            else:
                cache[vid] = np.cumsum(ints[off:off + n], dtype=np.int64).astype(np.int64).astype(np.uint32).view(
                    np.int32) if n else np.zeros(0, np.int32)
        return cache[vid]

    ent = d["ent"]
    records, e = [], 0
    for name, na, nb in d["rec"]:
        op, _, typ = names[name].partition(" ")
        entries = [(kinds[int(k)], None if sl < 0 else int(sl), values(int(v))) for k, sl, v in ent[e:e + na + nb]]
        e += na + nb
        records.append((op, typ or None, entries[:na], entries[na:]))
    return records, bytes(d["report"]).decode("latin-1")


def main():
    from oracle.oracle import reference_root
    ref = Path(sys.argv[1]) if len(sys.argv) > 1 else reference_root()
    if ref is None:
        sys.exit("no reference tree: pass its root, or set GCVL_REFERENCE")
    text = (ref / "nesl" / "vcode" / "nesltest.vcode").read_text(encoding="latin-1")
    records, report = record(text)
    np.savez_compressed(HERE / "nesltest_trace.npz", **pack(records, report))
    print(f"{len(records)} instructions recorded; report of {report.count(chr(10))} lines")


if __name__ == "__main__":
    main()
