"""VCODE I/O in the interpreter (FOPEN / FREAD / FWRITE / FCLOSE / READ /
WRITE, with vinterp's text forms and stack effects: nesl/vcode/io.c) -- a
key file read by a VCODE program, as a quicksort at scale reads its keys
instead of drawing them with RAND.  Runs on the oracle."""
import numpy as np
import pytest

from neslgpu_gb300 import vcode as V
from neslgpu_gb300.vcode_asm import Func


def _codes(s):
    return [ord(ch) for ch in s]


def _io_program():
    f = Func("IOTEST", params=["fin", "fout"], results=["s", "okr", "okw", "oko"])
    f.const("INT 1", "rmode")
    f.op("FOPEN", ["fin", "rmode"], ["fd", "e1", "oko"])
    f.op("FREAD INT", ["fd"], ["v", "e2", "okr"])
    f.op("FCLOSE", ["fd"], ["e3", "okc"])
    f.op("LENGTH INT", ["v"], ["len"])
    f.op("MAKE_SEGDES", ["len"], ["sd"])
    f.op("+_REDUCE INT", ["v", "sd"], ["s"])
    f.const("INT 2", "wmode")
    f.op("FOPEN", ["fout", "wmode"], ["fdo", "e4", "oko2"])
    f.op("FWRITE INT", ["v", "fdo"], ["e5", "okw"])
    f.op("FCLOSE", ["fdo"], ["e6", "okc2"])
    return f.emit()


def test_fread_fwrite_program(oracle, tmp_path):
    keys = np.random.default_rng(4).integers(-2 ** 31, 2 ** 31, size=5000, dtype=np.int64).astype(np.int32)
    fin, fout = tmp_path / "keys.txt", tmp_path / "out.txt"
    fin.write_text("  (" + " ".join(map(str, keys.tolist())) + "\n)\n")
    it = V.Interpreter(_io_program(), oracle.cvl)
    try:
        st = it.run("IOTEST", [it.from_host("I", _codes(str(fin))), it.from_host("I", _codes(str(fout)))])
        s, okr, okw, oko = (it.to_host(v) for v in st)
    finally:
        it.free_all()
    assert okr[0] and okw[0] and oko[0]
    assert int(s[0]) == int(np.int32(np.sum(keys, dtype=np.int64) & 0xFFFFFFFF))  # int32 wrap-around
    assert fout.read_text() == "(" + "".join(f" {k}" for k in keys.tolist()) + " )\n"


def test_read_forms_and_errors(oracle, tmp_path):
    p = tmp_path / "v.txt"
    p.write_text("(1.5 -2e3 inf)\n(T F\tT)\n[3 0 2]\n(1 2 x)\n( )\n")
    # five reads from one descriptor (stack: fd below the values read so
    # far; POP k d drops k values at depth d, COPY k d copies them on top)
    text = """FUNC RD
CONST INT 1
FOPEN
POP 2 0
COPY 1 0
FREAD FLOAT
POP 2 0
COPY 1 1
FREAD BOOL
POP 2 0
COPY 1 2
FREAD SEGDES
POP 2 0
COPY 1 3
FREAD INT
COPY 1 6
FREAD INT
POP 2 0
COPY 1 7
FCLOSE
POP 2 0
POP 1 7
RET
"""
    it = V.Interpreter(text, oracle.cvl)
    try:
        st = it.run("RD", [it.from_host("I", _codes(str(p)))])
        fl, bl, sd, bad, err, flag, empty = st
        np.testing.assert_array_equal(it.to_host(fl), [1.5, -2000.0, np.inf])
        np.testing.assert_array_equal(it.to_host(bl), [1, 0, 1])
        assert sd.kind == "S"
        np.testing.assert_array_equal(it.to_host(sd), [3, 0, 2])
        assert bad.len == 0 and not it.to_host(flag)[0]
        assert "".join(map(chr, it.to_host(err).tolist())) == "input error: vector must end with )"
        assert empty.kind == "I" and empty.len == 0
    finally:
        it.free_all()


@pytest.mark.parametrize("kind,vals,text", [("I", [1, -2, 3], "( 1 -2 3 )\n"),
                                            ("F", [1.0], "( 1.00000000000000e+00 )\n"),
                                            ("B", [1, 0], "( T F )\n"), ("S", [2, 3], "[ 2 3 ]\n"),
                                            ("I", [], "( )\n")])
def test_write_forms(kind, vals, text):
    assert V.format_vector(kind, vals) == text


@pytest.mark.gpu
def test_fread_fwrite_program_on_gpu(gpu, oracle, tmp_path):
    keys = np.random.default_rng(5).integers(-2 ** 31, 2 ** 31, size=300_001, dtype=np.int64).astype(np.int32)
    fin = tmp_path / "keys.txt"
    fin.write_text("(" + " ".join(map(str, keys.tolist())) + ")")
    outs = {}
    for name, runner in (("gpu", gpu), ("oracle", oracle)):
        fout = tmp_path / f"out_{name}.txt"
        it = V.Interpreter(_io_program(), runner.cvl)
        try:
            st = it.run("IOTEST", [it.from_host("I", _codes(str(fin))), it.from_host("I", _codes(str(fout)))])
            outs[name] = [it.to_host(v).tolist() for v in st]
        finally:
            it.free_all()
        assert fout.read_text() == "(" + "".join(f" {k}" for k in keys.tolist()) + " )\n"
    assert outs["gpu"] == outs["oracle"]


_CHAR_RT = """FUNC RT
COPY 1 1
CONST INT 2
FOPEN
POP 2 0
COPY 1 0
CPOP 1 2
CPOP 1 1
FWRITE CHAR
POP 2 0
FCLOSE
POP 2 0
CONST INT 1
FOPEN
POP 2 0
CONST CHAR ""
CONST INT -1
COPY 1 2
FREAD_CHAR
POP 2 0
CPOP 1 2
CONST CHAR "x"
CONST INT 5
COPY 1 2
FREAD_CHAR
POP 2 0
CPOP 1 2
CONST CHAR "x"
CONST INT -1
COPY 1 2
FREAD_CHAR
POP 2 0
CPOP 1 2
FCLOSE
POP 2 0
RET
"""


def test_fread_char_round_trip(oracle, tmp_path):
    """FWRITE CHAR then FREAD_CHAR (io.c:1134-1300) give back every byte
    value, \\r and \\n included (files are byte streams, no newline
    translation); the stop status is -1 at the end of the file, -2 at the
    character limit, else the delimiter, which is consumed."""
    payload = list(range(1, 256)) + [13, 10, 13]
    p = tmp_path / "chars.txt"
    it = V.Interpreter(_CHAR_RT, oracle.cvl)
    try:
        st = it.run("RT", [it.from_host("I", _codes(str(p))), it.from_host("I", payload)])
        got = [it.to_host(v).tolist() for v in st]
    finally:
        it.free_all()
    assert p.read_bytes() == bytes(payload)
    whole, stop1, five, stop2, rest, stop3 = got
    assert whole == payload and stop1 == [-1]
    assert five == [] and stop2 == [-1]  # the file is at its end: nothing left
    assert rest == [] and stop3 == [-1]
    q = tmp_path / "abc.txt"
    q.write_bytes(b"abcdefxyz")
    text = """FUNC RD
CONST INT 1
FOPEN
POP 2 0
CONST CHAR "x"
CONST INT 4
COPY 1 2
FREAD_CHAR
POP 2 0
CPOP 1 2
CONST CHAR "x"
CONST INT -1
COPY 1 2
FREAD_CHAR
POP 2 0
CPOP 1 2
POP 1 0
RET
"""
    it = V.Interpreter(text, oracle.cvl)
    try:
        st = it.run("RD", [it.from_host("I", _codes(str(q)))])
        got = [it.to_host(v).tolist() for v in st]
    finally:
        it.free_all()
    assert got == [_codes("abcd"), [-2], _codes("ef"), [ord("x")]]


def test_spawn_cat_round_trip(oracle):
    """SPAWN (io.c do_spawn) of "cat -u" with pipes for its stdin and
    stdout and the interpreter's stderr: a vector written to the child
    comes back, as the reference suite's spawn test checks."""
    text = """FUNC SP
CONST CHAR "cat -u"
CONST INT -1
CONST INT -1
CONST INT 2
SPAWN
POP 2 0
CONST INT (23 -5 7)
COPY 1 1
FWRITE INT
POP 2 0
COPY 1 1
FREAD INT
POP 1 1
CPOP 1 3
FCLOSE
POP 2 0
CPOP 1 2
FCLOSE
POP 2 0
POP 1 2
RET
"""
    it = V.Interpreter(text, oracle.cvl)
    try:
        st = it.run("SP", [])
        got = [it.to_host(v).tolist() for v in st]
    finally:
        it.free_all()
    assert got == [[23, -5, 7], [1]]
