"""A VCODE interpreter over the CVL C ABI -- the role vinterp plays for the
reference (nesl/vcode/main.c, stack.c, vstack.c), written for this library.

VCODE is the stack-machine language the NESL compiler emits: every value on
the stack is a vector (a scalar is a vector of length 1) of INT, FLOAT or
BOOL elements, or a segment descriptor; every vector operation is one CVL
call.  The interpreter follows vinterp's conventions for the calls:

* elementwise ops call ``*_wu*`` with the length of their first argument;
* scans, reductions and ranks call the segmented form ``*_se*``/``*_re*``/
  ``rk*_le*`` with the segment descriptor on top of the stack (an
  unsegmented vector carries a one-segment descriptor);
* PACK is ``pk1_lev`` + ``add_ruz`` + ``mke_fov`` + ``pk2_le*``, and
  MAKE_SEGDES is ``add_ruz`` + ``mke_fov`` (main.c:510-641);
* argument i of an op is the i-th of the top arg_count stack entries, the
  deepest first (stack.c:361-376); results are pushed in order;
* COPY c s / POP c s / CPOP c s copy, drop or move the c entries that sit s
  below the top (stack.c:186-318);
* IF pops a BOOL scalar (stack.c:124-142); scalars that steer control flow
  are read back to the host, as in vinterp.

What differs from vinterp, by design: memory comes from a size-class cache
over ``alo_foz`` (one device allocation per size class and reuse, instead
of one heap with compaction); constants are uploaded once and then shared;
the same interpreter runs on any implementation of the ABI -- the GPU
library or, for the parity tests and the CPU baseline, the oracle.
"""
from __future__ import annotations

import bisect
import io
import re
import sys
import time
import warnings
from dataclasses import dataclass

import numpy as np

from .cvl import CVL, check, load

# ------------------------------------------------------------ op table ---
TYPE_SUFFIX = {"INT": "z", "FLOAT": "d", "BOOL": "b"}
KIND_OF = {"INT": "I", "FLOAT": "F", "BOOL": "B", "SEGDES": "S"}
SUFFIX_OF_KIND = {"I": "z", "F": "d", "B": "b"}

# elementwise: name -> (CVL stem, arity, result kind or None for "same as
# argument 1", or "A2" for "same as argument 2")
ELT = {
    "+": ("add", 2, None), "-": ("sub", 2, None), "*": ("mul", 2, None), "/": ("div", 2, None),
    "%": ("mod", 2, "I"), "<": ("les", 2, "B"), "<=": ("leq", 2, "B"), ">": ("grt", 2, "B"),
    ">=": ("geq", 2, "B"), "=": ("eql", 2, "B"), "!=": ("neq", 2, "B"), "LSHIFT": ("lsh", 2, "I"),
    "RSHIFT": ("rsh", 2, "I"), "NOT": ("not", 1, None), "AND": ("and", 2, None), "OR": ("ior", 2, None),
    "XOR": ("xor", 2, None), "SELECT": ("sel", 3, "A2"), "RAND": ("rnd", 1, "I"),
    "FLOOR": ("flr", 1, "I"), "CEIL": ("cei", 1, "I"), "TRUNC": ("trn", 1, "I"), "ROUND": ("rou", 1, "I"),
    "LOG": ("log", 1, "F"), "SQRT": ("sqt", 1, "F"), "EXP": ("exp", 1, "F"), "SIN": ("sin", 1, "F"),
    "COS": ("cos", 1, "F"), "TAN": ("tan", 1, "F"), "ASIN": ("asn", 1, "F"), "ACOS": ("acs", 1, "F"),
    "ATAN": ("atn", 1, "F"), "SINH": ("snh", 1, "F"), "COSH": ("csh", 1, "F"), "TANH": ("tnh", 1, "F"),
    "I_TO_F": ("dbl", 1, "F"), "I_TO_B": ("boo", 1, "B"), "B_TO_I": ("int", 1, "I"),
}
# the type an untyped elementwise op works on (grammar.yy:160-243)
ELT_DEFAULT_TYPE = {"%": "INT", "LSHIFT": "INT", "RSHIFT": "INT", "RAND": "INT", "I_TO_F": "INT",
                    "I_TO_B": "INT", "B_TO_I": "BOOL", "FLOOR": "FLOAT", "CEIL": "FLOAT", "TRUNC": "FLOAT",
                    "ROUND": "FLOAT", "LOG": "FLOAT", "SQRT": "FLOAT", "EXP": "FLOAT", "SIN": "FLOAT",
                    "COS": "FLOAT", "TAN": "FLOAT", "ASIN": "FLOAT", "ACOS": "FLOAT", "ATAN": "FLOAT",
                    "SINH": "FLOAT", "COSH": "FLOAT", "TANH": "FLOAT"}
SCAN = {"+_SCAN": "add", "*_SCAN": "mul", "MAX_SCAN": "max", "MIN_SCAN": "min", "AND_SCAN": "and",
        "OR_SCAN": "ior", "XOR_SCAN": "xor"}
REDUCE = {"+_REDUCE": "add", "*_REDUCE": "mul", "MAX_REDUCE": "max", "MIN_REDUCE": "min",
          "AND_REDUCE": "and", "OR_REDUCE": "ior", "XOR_REDUCE": "xor"}
VEC = {"PERMUTE", "DPERMUTE", "FPERMUTE", "BPERMUTE", "BFPERMUTE", "DFPERMUTE", "EXTRACT", "REPLACE",
       "DIST", "INDEX", "RANK_UP", "RANK_DOWN", "PACK"}
TYPES = {"INT", "FLOAT", "BOOL", "SEGDES", "CHAR"}
STACK_OPS = {"COPY", "POP", "CPOP"}


class VcodeError(RuntimeError):
    pass


# instructions a trace leaves out: host I/O and process control
_UNTRACED = {"READ", "WRITE", "FREAD", "FWRITE", "FOPEN", "FCLOSE", "FREAD_CHAR", "SPAWN"}

# Instructions that end a block captured as a CUDA graph: control flow, and
# instructions that read a value back to the host (MAKE_SEGDES and PACK need
# a length, IF a flag), write a host value into a new scalar (LENGTH), draw
# from host-side state (RAND, SRAND), do I/O or time.
_GRAPH_STOP = {"CALL", "RET", "IF", "ELSE", "ENDIF", "EXIT", "START_TIMER", "STOP_TIMER", "MAKE_SEGDES", "PACK",
               "LENGTH", "RAND", "SRAND"} | _UNTRACED
_HOST_ONLY = {"COPY", "POP", "CPOP", "CONST", "CONSTV"}


class _NeedsHost(Exception):
    """Raised inside a captured block when it would need the device
    allocator (a new heap block, a larger scratch vector)."""


# --------------------------------------------------------------- parse ---
@dataclass
class Ins:
    op: str
    typ: str | None = None
    a: object = None   # COPY/POP/CPOP count; CALL target name; CONST value
    b: object = None   # COPY/POP/CPOP depth; branch target
    line: int = 0


_TOKEN = re.compile(r"\{[^}]*\}|\(|\)|\"[^\"]*\"|[^\s(){}\"]+")


def parse(text: str) -> tuple[list[Ins], dict[str, int], str]:
    """VCODE text -> (instructions, function entry points, first function).
    Grammar after nesl/vcode/grammar.yy: FUNC name [I types O types]
    statements RET; comments in braces.  Comments and strings may run over
    several lines (nesl/vcode/tokens.ll:33-34)."""
    toks = []
    lineno, at = 1, 0
    for mt in _TOKEN.finditer(text):
        lineno += text.count("\n", at, mt.start())
        at = mt.start()
        t = mt.group(0)
        if not t.startswith("{"):
            toks.append((t, lineno))
    prog: list[Ins] = []
    funcs: dict[str, int] = {}
    first = None
    i = 0
    n = len(toks)
    ifs: list[int] = []

    def peek(k=0):
        return toks[i + k][0] if i + k < n else None

    while i < n:
        t, ln = toks[i]
        i += 1
        if t == "FUNC":
            name = toks[i][0]
            i += 1
            funcs[name] = len(prog)
            first = first or name
            if peek() == "I":  # input / output type declarations
                i += 1
                while peek() is not None and peek() != "O":
                    i += 1
                i += 1
                while peek() in TYPES:
                    i += 1
            continue
        if t in STACK_OPS:
            prog.append(Ins(t, None, int(toks[i][0]), int(toks[i + 1][0]), ln))
            i += 2
        elif t == "CALL":
            prog.append(Ins("CALL", None, toks[i][0], None, ln))
            i += 1
        elif t == "RET":
            prog.append(Ins("RET", line=ln))
        elif t == "IF":
            ifs.append(len(prog))
            prog.append(Ins("IF", line=ln))
        elif t == "ELSE":
            j = ifs.pop()
            ifs.append(len(prog))
            prog[j].b = len(prog) + 1  # IF false -> after ELSE
            prog.append(Ins("ELSE", line=ln))
        elif t == "ENDIF":
            j = ifs.pop()
            prog[j].b = len(prog)       # to here (IF false, or ELSE skipping the else-branch)
            prog.append(Ins("ENDIF", line=ln))
        elif t == "CONST":
            typ = toks[i][0]
            i += 1
            if typ == "CHAR" and peek() is not None and peek().startswith('"'):
                # a string: the codes of the characters between the quotes,
                # taken as they are (constant.c:124-155)
                prog.append(Ins("CONSTV", typ, [ord(ch) for ch in toks[i][0][1:-1]], None, ln))
                i += 1
            elif peek() == "(":
                i += 1
                vals = []
                while peek() != ")":
                    vals.append(toks[i][0])
                    i += 1
                i += 1
                prog.append(Ins("CONSTV", typ, vals, None, ln))
            else:
                prog.append(Ins("CONST", typ, toks[i][0], None, ln))
                i += 1
        elif t == "FUSED":
            prog.append(Ins("FUSED", None, int(toks[i][0]), None, ln))
            i += 1
        elif t in ("START_TIMER", "STOP_TIMER", "EXIT", "MAKE_SEGDES", "LENGTHS", "PAIR", "UNPAIR", "FOPEN",
                   "FCLOSE", "FREAD_CHAR", "SPAWN"):
            prog.append(Ins(t, line=ln))
        elif t in ("SRAND", "READ", "WRITE", "FREAD", "FWRITE", "LENGTH") or t in ELT or t in SCAN or \
                t in REDUCE or t in VEC:
            typ = None
            if peek() in TYPES:
                typ = toks[i][0]
                i += 1
            prog.append(Ins(t, typ, line=ln))
        else:
            raise VcodeError(f"line {ln}: unknown token {t!r}")
    # resolve calls
    for ins in prog:
        if ins.op == "CALL":
            if ins.a not in funcs:
                raise VcodeError(f"line {ins.line}: CALL of undefined {ins.a}")
            ins.b = funcs[ins.a]
    return prog, funcs, ("MAIN" if "MAIN" in funcs else first)


# ---------------------------------------------------------------- values ---
class Vec:
    __slots__ = ("kind", "len", "seg_len", "ptr", "cls", "ref", "const")

    def __init__(self, kind, length, seg_len, ptr, cls):
        self.kind, self.len, self.seg_len, self.ptr, self.cls = kind, length, seg_len, ptr, cls
        self.ref = 1
        self.const = False

    def __repr__(self):
        return f"Vec({self.kind}, len={self.len}, seg_len={self.seg_len})"


class Heap:
    """Size-class cache over alo_foz: freed blocks wait for the next request
    of their class instead of going back to the allocator."""

    def __init__(self, c: CVL):
        self.c = c
        self.free: dict[int, list[int]] = {}
        self.held = 0
        self.no_new = False
        self.on_trim = None  # called when blocks go back to the device
        self.log = None      # a list: every ("a"|"r", class, address) is appended

    @staticmethod
    def size_class(units: int) -> int:
        u = max(int(units), 4)
        return 1 << (u - 1).bit_length()

    def alloc(self, units: int) -> tuple[int, int]:
        cls = self.size_class(units)
        lst = self.free.get(cls)
        if lst:
            p = lst.pop()
            if self.log is not None:
                self.log.append(("a", cls, p))
            return p, cls
        if self.no_new:  # a captured or replayed block may not allocate
            raise _NeedsHost("heap")
        p = self.c.alo_foz(cls)
        if not p:
            self.trim()
            p = self.c.alo_foz(cls)
            if not p:
                raise MemoryError(f"alo_foz({cls}) failed")
        self.held += cls
        return p, cls

    def release(self, ptr: int, cls: int):
        # each class's free list is kept in descending address order and
        # allocation takes the lowest address: which addresses a sequence of
        # requests gets then depends only on which blocks are free, not on
        # the order they were freed in, so a block that runs again in the same
        # state gets the same vectors (graph replay relies on it)
        bisect.insort(self.free.setdefault(cls, []), ptr, key=lambda q: -q)
        if self.log is not None:
            self.log.append(("r", cls, ptr))

    def trim(self):
        if self.on_trim:
            self.on_trim()
        for cls, lst in self.free.items():
            for p in lst:
                self.c.fre_fov(p)
                self.held -= cls
        self.free.clear()


# ------------------------------------------------------------------ I/O ---
NULL_STREAM_FD = -1
MAX_FILES = 64
_OPEN_CLOSE = {"INT": "()", "FLOAT": "()", "BOOL": "()", "SEGDES": "[]", "CHAR": '""'}


def format_vector(kind: str, a) -> str:
    """A vector as vinterp writes it: "( 1 2 3 )", floats in %.14e, booleans
    as T/F, a segment descriptor as "[ lengths ]"; one line."""
    if kind == "F":
        body = "".join(f" {x:.14e}" for x in a)
    elif kind == "B":
        body = "".join(" T" if x else " F" for x in a)
    else:
        body = "".join(f" {int(x)}" for x in a)
    o, c = ("[", "]") if kind == "S" else ("(", ")")
    return f"{o}{body} {c}\n"


class _VStream:
    """A VCODE file: a text stream read vector by vector."""

    def __init__(self, f):
        self.f = f
        self.buf = ""

    def _fill(self) -> bool:
        # what is there now, up to 64 KB: a pipe or terminal must not wait
        # for a full block
        raw = getattr(self.f, "buffer", None)
        if raw is not None and hasattr(raw, "read1"):
            chunk = raw.read1(1 << 16).decode("latin-1")
        else:
            chunk = self.f.read(1 << 16)
        self.buf += chunk
        return bool(chunk)

    def write(self, text: str):
        self.f.write(text)
        self.f.flush()

    def read_chars(self, max_char: int, delims: set):
        """Characters up to a delimiter (consumed, not returned), the end of
        the file or max_char of them: (codes, stop) with stop -2 at
        max_char, -1 at the end, else the delimiter (io.c:1249-1290)."""
        out = []
        while len(out) < max_char:
            if not self.buf and not self._fill():
                return out, -1
            c = ord(self.buf[0])
            self.buf = self.buf[1:]
            if c in delims:
                return out, c
            out.append(c)
        return out, -2

    def read_vector(self, typ: str):
        """(values, None) or (None, error message)."""
        start, end = _OPEN_CLOSE.get(typ, "()")
        while True:
            self.buf = self.buf.lstrip()
            if self.buf or not self._fill():
                break
        if not self.buf or self.buf[0] != start:
            self.buf = self.buf[1:]
            return None, f"vinterp: input error: vector must start with {start}"
        self.buf = self.buf[1:]
        parts = []
        while True:
            j = self.buf.find(end)
            if j >= 0:
                parts.append(self.buf[:j])
                self.buf = self.buf[j + 1:]
                break
            parts.append(self.buf)
            self.buf = ""
            if not self._fill():
                return None, f"input error: vector must end with {end}"
        body = "".join(parts)
        if typ == "CHAR":
            return np.frombuffer(body.encode("latin-1"), dtype=np.uint8).astype(np.int32), None
        if typ == "BOOL":
            flags = body.replace(" ", "").replace("\t", "").replace("\n", "")
            if flags.strip("TF"):
                return None, f"input error: vector must end with {end}"
            return np.frombuffer(flags.encode(), dtype=np.uint8) == ord("T"), None
        if not body.strip():
            return np.empty(0, dtype=np.float64 if typ == "FLOAT" else np.int32), None
        with warnings.catch_warnings():
            warnings.simplefilter("error")
            try:
                if typ == "FLOAT":
                    return np.fromstring(body, dtype=np.float64, sep=" "), None
                v = np.fromstring(body, dtype=np.int64, sep=" ")
            except (ValueError, DeprecationWarning, RuntimeWarning):
                return None, f"input error: vector must end with {end}"
        # 32-bit wrap-around, as vinterp's own integer parser
        return (v & 0xFFFFFFFF).astype(np.uint32).view(np.int32), None


# ----------------------------------------------------------- interpreter ---
class Interpreter:
    """Runs a parsed VCODE program on one CVL implementation."""

    def __init__(self, text: str, cvl: CVL | None = None, sync=None, fused=None, graphs: bool = False,
                 graph_min_ops: int = 2):
        """fused: a FusedLib (neslgpu_gb300.fcode) for the program's FUSED ops.
        graphs: run each basic block of at least graph_min_ops device
        instructions as a CUDA graph, captured the first time the block runs
        in a given state and replayed whenever it runs in that state again
        (needs the library's gcvl_graph_* calls)."""
        self.fused = fused
        self.graphs = graphs
        self.graph_min_ops = graph_min_ops
        self.graph_cache_max = 1024
        self._block_ends: dict[int, int | None] = {}
        self._blocks: dict[int, dict] = {}  # pc -> {"recs": {depth: {signature: [record]}}, "warm": bool}
        self._n_graphs = 0
        self.graph_stats = {"captured": 0, "replayed": 0, "aborted": 0, "blocks_run": 0}
        self._capturing = False
        self.c = c = cvl or load()
        self.prog, self.funcs, self.main = parse(text)
        self.heap = Heap(c)
        self.heap.on_trim = self.drop_graphs
        self.stack: list[Vec] = []
        self.scratch_ptr, self.scratch_units = 0, 0
        self._consts: dict = {}
        self._scalar_cache: dict = {}
        self.sync = sync or (lambda: None)
        self.timer = 0.0
        self.ops_run = 0
        self._fn = {}
        # VCODE file descriptors: 0, 1, 2 are the standard streams
        self.files: dict[int, _VStream] = {0: _VStream(sys.stdin), 1: _VStream(sys.stdout), 2: _VStream(sys.stderr)}
        # trace(op, typ, consumed, produced): called after every vector
        # instruction other than I/O with (kind, segment count or None,
        # values) triples of the stack entries it took and left; None: off
        self.trace = None

    # -- memory
    def fn(self, name):
        f = self._fn.get(name)
        if f is None:
            f = self._fn[name] = getattr(self.c, name)
        return f

    def sfn(self, name):
        """The F_scratch function of name; an implementation that allocates
        its own temporaries (the oracle) has none, and needs no scratch."""
        f = self._fn.get(name)
        if f is None:
            f = getattr(self.c, name, None) or (lambda *a: 0)
            self._fn[name] = f
        return f

    def units(self, kind, length, seg_len=None):
        c = self.c
        if kind == "S":
            return c.siz_fos(seg_len, length)
        if kind == "F":
            return c.siz_fod(max(length, 1))
        return c.siz_foz(max(length, 1)) if kind == "I" else c.siz_fob(max(length, 1))

    def new(self, kind, length, seg_len=None) -> Vec:
        ptr, cls = self.heap.alloc(self.units(kind, length, seg_len))
        return Vec(kind, length, seg_len if kind == "S" else None, ptr, cls)

    def drop(self, v: Vec):
        v.ref -= 1
        if v.ref == 0 and not v.const:
            self.heap.release(v.ptr, v.cls)

    def scratch(self, units: int):
        if units > self.scratch_units:
            if self._capturing:
                raise _NeedsHost("scratch")
            self.drop_graphs()  # graphs hold the old scratch's address
            if self.scratch_ptr:
                self.c.fre_fov(self.scratch_ptr)
            self.scratch_units = max(int(units), 2 * self.scratch_units, 1024)
            self.scratch_ptr = self.c.alo_foz(self.scratch_units)
            if not self.scratch_ptr:
                raise MemoryError("scratch")
        return self.scratch_ptr

    def drop_graphs(self):
        """Forget the cached block graphs (the addresses they hold are about
        to change)."""
        for info in self._blocks.values():
            for by_sig in info["recs"].values():
                for recs in by_sig.values():
                    for r in recs:
                        self.c.gcvl_graph_destroy(r["graph"])
            info["recs"].clear()
        self._n_graphs = 0

    def free_all(self):
        self.drop_graphs()
        for v in self.stack:
            self.drop(v)
        self.stack.clear()
        for v in list(self._consts.values()) + list(self._scalar_cache.values()):
            v.const = False
            v.ref = 1
            self.drop(v)
        self._consts.clear()
        self._scalar_cache.clear()
        self.heap.trim()
        if self.scratch_ptr:
            self.c.fre_fov(self.scratch_ptr)
            self.scratch_ptr, self.scratch_units = 0, 0

    # -- host <-> vector
    def from_host(self, kind, arr) -> Vec:
        a = np.ascontiguousarray(arr, dtype=np.float64 if kind == "F" else np.int32)
        v = self.new(kind, len(a))
        if len(a):
            self.fn("c2v_fud" if kind == "F" else ("c2v_fuz" if kind == "I" else "c2v_fub"))(
                v.ptr, a.ctypes.data, len(a), None)
        return v

    def to_host(self, v: Vec) -> np.ndarray:
        if v.kind == "S":
            out = np.empty(v.len, dtype=np.int32)
            lv = self.new("I", v.len)
            if v.len:
                self.fn("len_fos")(lv.ptr, v.ptr, v.seg_len, v.len, self.scratch(self.sfn("len_fos_scratch")(
                    v.seg_len, v.len)))
                self.fn("v2c_fuz")(out.ctypes.data, lv.ptr, v.len, None)
            self.drop(lv)
            return out
        out = np.empty(v.len, dtype=np.float64 if v.kind == "F" else np.int32)
        if v.len:
            self.fn("v2c_fud" if v.kind == "F" else ("v2c_fuz" if v.kind == "I" else "v2c_fub"))(
                out.ctypes.data, v.ptr, v.len, None)
        return out

    def scalar_int(self, v: Vec) -> int:
        return int(self.fn("ext_vuz")(v.ptr, 0, 1, None))

    def scalar_bool(self, v: Vec) -> bool:
        return bool(self.fn("ext_vub")(v.ptr, 0, 1, None))

    def const_scalar(self, kind, value) -> Vec:
        key = (kind, value)
        v = self._scalar_cache.get(key)
        if v is None:
            v = self.new(kind, 1)
            if kind == "I":
                self.fn("rep_vuz")(v.ptr, 0, int(value), 1, None)
            elif kind == "F":
                self.fn("rep_vud")(v.ptr, 0, float(value), 1, None)
            else:
                self.fn("rep_vub")(v.ptr, 0, 1 if value else 0, 1, None)
            v.const = True
            self._scalar_cache[key] = v
        v.ref += 1
        return v

    def segdes_from_lengths(self, lens: Vec) -> Vec:
        c = self.c
        m = lens.len
        n = int(self.fn("add_ruz")(lens.ptr, m, self.scratch(self.sfn("add_ruz_scratch")(m)))) if m else 0
        sd = self.new("S", m, n)
        self.fn("mke_fov")(sd.ptr, lens.ptr, n, m, self.scratch(self.sfn("mke_fov_scratch")(n, m)))
        return sd

    # -- main loop
    def run(self, entry: str | None = None, args: list[Vec] | None = None) -> list[Vec]:
        """Runs from `entry` (default: MAIN or the first function) with
        `args` pushed; returns the final stack (the caller owns it)."""
        prog = self.prog
        self.stack = list(args or [])
        st = self.stack
        pc = self.funcs[entry or self.main]
        rstack = [-1]
        t_start = None
        while pc >= 0:
            if self.graphs:
                end = self._block_end(pc)
                if end is not None:
                    self._run_block(pc, end)
                    pc = end
                    continue
            ins = prog[pc]
            op = ins.op
            pc += 1
            self.ops_run += 1
            if op == "COPY":
                k, d = ins.a, ins.b
                seg = st[len(st) - d - k: len(st) - d]
                for v in seg:
                    v.ref += 1
                st.extend(seg)
            elif op == "CPOP":
                k, d = ins.a, ins.b
                lo, hi = len(st) - d - k, len(st) - d
                seg = st[lo:hi]
                del st[lo:hi]
                st.extend(seg)
            elif op == "POP":
                k, d = ins.a, ins.b
                lo, hi = len(st) - d - k, len(st) - d
                for v in st[lo:hi]:
                    self.drop(v)
                del st[lo:hi]
            elif op == "CALL":
                rstack.append(pc)
                pc = ins.b
            elif op == "RET":
                pc = rstack.pop()
            elif op == "IF":
                f = st.pop()
                taken = self.scalar_bool(f)
                self.drop(f)
                if not taken:
                    pc = ins.b
            elif op == "ELSE":  # end of the then-branch: skip the else-branch
                pc = ins.b
            elif op == "ENDIF":
                pass
            elif op == "CONST":
                st.append(self._const(ins))
            elif op == "CONSTV":
                st.append(self._const_vec(ins))
            elif op == "START_TIMER":
                self.sync()
                t_start = time.perf_counter()
            elif op == "STOP_TIMER":
                self.sync()
                self.timer = time.perf_counter() - (t_start or time.perf_counter())
                v = self.new("F", 1)
                self.fn("rep_vud")(v.ptr, 0, self.timer, 1, None)
                st.append(v)
            elif op == "EXIT":
                break
            elif self.trace is not None and op not in _UNTRACED:
                self._traced_op(ins)
            else:
                self._vector_op(ins)
        return self.stack

    # -- basic blocks as CUDA graphs
    def _block_end(self, pc: int):
        """End (exclusive) of the block of graph-capturable instructions that
        starts at pc, or None when it holds too few device instructions."""
        if pc in self._block_ends:
            return self._block_ends[pc]
        prog = self.prog
        j, dev = pc, 0
        while j < len(prog) and prog[j].op not in _GRAPH_STOP:
            if prog[j].op not in _HOST_ONLY:
                dev += 1
            j += 1
        end = j if dev >= self.graph_min_ops else None
        self._block_ends[pc] = end
        return end

    def _exec_range(self, pc: int, end: int):
        """Runs the straight-line instructions [pc, end) (no control flow)."""
        st = self.stack
        for ins in self.prog[pc:end]:
            op = ins.op
            self.ops_run += 1
            if op == "COPY":
                k, d = ins.a, ins.b
                seg = st[len(st) - d - k: len(st) - d]
                for v in seg:
                    v.ref += 1
                st.extend(seg)
            elif op == "CPOP":
                k, d = ins.a, ins.b
                lo, hi = len(st) - d - k, len(st) - d
                seg = st[lo:hi]
                del st[lo:hi]
                st.extend(seg)
            elif op == "POP":
                k, d = ins.a, ins.b
                lo, hi = len(st) - d - k, len(st) - d
                for v in st[lo:hi]:
                    self.drop(v)
                del st[lo:hi]
            elif op == "CONST":
                st.append(self._const(ins))
            elif op == "CONSTV":
                st.append(self._const_vec(ins))
            else:
                self._vector_op(ins)

    @staticmethod
    def _stack_sig(top, refs=None) -> tuple:
        """Shapes, addresses, reference counts (refs: id -> count, else the
        current ones) and aliasing of stack entries.  A cached constant's
        count is left out: it is never freed, so the count changes nothing."""
        first: dict[int, int] = {}
        return tuple((v.kind, v.len, v.seg_len, v.ptr, -1 if v.const else (v.ref if refs is None else refs[id(v)]),
                      v.const, first.setdefault(id(v), i)) for i, v in enumerate(top))

    def _snapshot(self):
        vecs = list(self.stack) + list(self._consts.values()) + list(self._scalar_cache.values())
        return (list(self.stack), [(v, v.ref) for v in vecs], {c: list(lst) for c, lst in self.heap.free.items()},
                self.heap.held)

    def _restore(self, snap):
        stack, refs, free, held = snap
        self.stack[:] = stack
        for v, r in refs:
            v.ref = r
        self.heap.free = free
        self.heap.held = held

    def _replay(self, info, pc: int, end: int) -> bool:
        """Runs the block from its graph if one was captured in the state the
        block now reads: the top `depth` stack entries, the lowest free
        addresses of each size class it allocates from (allocation takes the
        lowest) and the scratch vector.  The host side is the recorded
        effect: stack rewrite, reference counts, heap operations."""
        st = self.stack
        free = self.heap.free
        rec = None
        for D, by_sig in info["recs"].items():  # the depths the block reached in the states it was captured in
            if len(st) < D:
                continue
            base = len(st) - D
            top = st[base:]
            for r in by_sig.get(self._stack_sig(top), ()):
                if r["scratch"] != (self.scratch_ptr, self.scratch_units):
                    continue
                if all(len(free.get(c, ())) >= len(req) and tuple(free[c][len(free[c]) - len(req):]) == req
                       for c, req in r["req"].items()):
                    rec = r
                    break
            if rec is not None:
                break
        if rec is None:
            return False
        news = []
        for kind, ln, sl, ptr, cls, ref in rec["new"]:
            v = Vec(kind, ln, sl, ptr, cls)
            v.ref = ref
            news.append(v)
        for i, delta in rec["refs"]:
            top[i].ref += delta
        for op, c, ptr in rec["log"]:
            if op == "a":
                free[c].pop()
            else:
                bisect.insort(free.setdefault(c, []), ptr, key=lambda q: -q)
        st[base:] = [top[j] if w == "o" else (news[j] if w == "n" else j) for w, j in rec["out"]]
        self.ops_run += end - pc
        if self.c.gcvl_graph_launch(rec["graph"]) != 0:
            raise VcodeError(f"graph launch: {self.c.gcvl_error_string().decode()}")
        self.graph_stats["replayed"] += 1
        return True

    def _capture(self, info, pc: int, end: int):
        """Runs the block while capturing its calls into a graph, then
        launches the graph and records the block's host effect for replay.
        Abandoned (state restored, block run plainly) when the block would
        need the device allocator."""
        c, st = self.c, self.stack
        snap = self._snapshot()
        if c.gcvl_graph_begin() != 0:
            c.gcvl_clear_error()
            self._exec_range(pc, end)
            return
        start = list(st)
        L0 = len(start)
        start_ref = {id(v): v.ref for v in start}
        lowest = L0
        self._capturing, self.heap.no_new, self.heap.log = True, True, []
        try:
            for q in range(pc, end):  # _exec_range, noting the lowest stack entry each instruction reaches
                ins = self.prog[q]
                if ins.op in ("COPY", "POP", "CPOP"):
                    lowest = min(lowest, len(st) - ins.b - ins.a)
                    self._exec_range(q, q + 1)
                elif ins.op in ("CONST", "CONSTV"):
                    self._exec_range(q, q + 1)
                else:
                    before = list(st)
                    self._exec_range(q, q + 1)
                    p = 0
                    while p < len(before) and p < len(st) and st[p] is before[p]:
                        p += 1
                    lowest = min(lowest, p)
        except _NeedsHost:
            self._capturing, self.heap.no_new, self.heap.log = False, False, None
            gx = c.gcvl_graph_end()
            if gx:
                c.gcvl_graph_destroy(gx)
            c.gcvl_clear_error()
            self._restore(snap)
            self._exec_range(pc, end)
            self.graph_stats["aborted"] += 1
            return
        finally:
            log = self.heap.log
            self._capturing, self.heap.no_new, self.heap.log = False, False, None
        g = c.gcvl_graph_end()
        if not g:
            raise VcodeError(f"graph capture: {c.gcvl_error_string().decode()}")
        if c.gcvl_graph_launch(g) != 0:
            raise VcodeError(f"graph launch: {c.gcvl_error_string().decode()}")
        self.graph_stats["captured"] += 1
        if self._n_graphs >= self.graph_cache_max:
            c.gcvl_graph_destroy(g)
            return
        D = L0 - lowest
        top = start[lowest:]
        pos = {}
        for i, v in enumerate(top):
            pos.setdefault(id(v), i)
        new_ix: dict[int, int] = {}
        new_spec, out = [], []
        for v in st[lowest:]:
            if id(v) in pos:
                out.append(("o", pos[id(v)]))
            elif v.const:
                out.append(("c", v))  # a cached constant: the same vector
            else:
                if id(v) not in new_ix:
                    new_ix[id(v)] = len(new_spec)
                    new_spec.append((v.kind, v.len, v.seg_len, v.ptr, v.cls, v.ref))
                out.append(("n", new_ix[id(v)]))
        refs = [(i, top[i].ref - start_ref[id(top[i])]) for i in sorted(set(pos.values()))
                if top[i].ref != start_ref[id(top[i])]]
        initial_free = snap[2]
        allocs: dict[int, int] = {}
        for op, cls, _ in log:
            if op == "a":
                allocs[cls] = allocs.get(cls, 0) + 1
        req = {cls: tuple(initial_free[cls][len(initial_free[cls]) - k:]) for cls, k in allocs.items()}
        rec = {"graph": g, "req": req, "scratch": (self.scratch_ptr, self.scratch_units), "new": new_spec,
               "refs": refs, "log": log, "out": out}
        info["recs"].setdefault(D, {}).setdefault(self._stack_sig(top, start_ref), []).append(rec)
        self._n_graphs += 1

    def _run_block(self, pc: int, end: int):
        """Runs the block [pc, end) through a CUDA graph: replayed when it ran
        before in the state it reads now, else captured while it runs."""
        self.graph_stats["blocks_run"] += 1
        info = self._blocks.get(pc)
        if info is None:
            info = self._blocks[pc] = {"recs": {}, "warm": False}
        if not info["warm"]:
            # constants first: their first use copies from the host
            for ins in self.prog[pc:end]:
                if ins.op == "CONST":
                    self.drop(self._const(ins))
                elif ins.op == "CONSTV":
                    self.drop(self._const_vec(ins))
            info["warm"] = True
        if not self._replay(info, pc, end):
            self._capture(info, pc, end)

    def _traced_op(self, ins, depth: int = 8):
        """_vector_op, reporting the values it consumed and produced to
        self.trace (an instruction takes and leaves entries at the top of
        the stack only, so the first position whose entry changed splits
        the two).  The top entries are held by one more reference during
        the instruction, so none is updated in place and returned as its
        own result."""
        st = self.stack
        old = list(st)
        top = old[max(0, len(old) - depth):]
        snap = [(v.kind, v.seg_len, self.to_host(v)) for v in top]
        for v in top:
            v.ref += 1
        self._vector_op(ins)
        for v in top:
            self.drop(v)
        p = 0
        while p < len(old) and p < len(st) and st[p] is old[p]:
            p += 1
        taken = len(old) - p
        if taken > len(top):
            raise VcodeError(f"line {ins.line}: {ins.op} took more than {depth} stack entries")
        consumed = snap[len(snap) - taken:] if taken else []
        produced = [(v.kind, v.seg_len, self.to_host(v)) for v in st[p:]]
        self.trace(ins.op, ins.typ, consumed, produced)

    def _const(self, ins):
        t = ins.typ
        if t == "INT":
            return self.const_scalar("I", int(ins.a))
        if t == "FLOAT":
            return self.const_scalar("F", float(ins.a))
        if t == "BOOL":
            return self.const_scalar("B", ins.a in ("T", "1"))
        if t == "SEGDES":  # one segment of the given length
            key = ("S", int(ins.a))
            v = self._consts.get(key)
            if v is None:
                lens = self.from_host("I", [int(ins.a)])
                v = self.segdes_from_lengths(lens)
                self.drop(lens)
                v.const = True
                self._consts[key] = v
            v.ref += 1
            return v
        raise VcodeError(f"line {ins.line}: CONST of type {t}")

    def _const_vec(self, ins):
        key = id(ins)
        v = self._consts.get(key)
        if v is None:
            t = ins.typ
            if t == "FLOAT":
                v = self.from_host("F", [float(x) for x in ins.a])
            elif t == "BOOL":
                v = self.from_host("B", [1 if x == "T" else 0 for x in ins.a])
            elif t == "SEGDES":
                lens = self.from_host("I", [int(x) for x in ins.a])
                v = self.segdes_from_lengths(lens)
                self.drop(lens)
            else:
                v = self.from_host("I", [int(x) for x in ins.a])
            v.const = True
            self._consts[key] = v
        v.ref += 1
        return v

    # -- vector operations
    def _vector_op(self, ins):
        op, st = ins.op, self.stack
        if op in ELT:
            stem, ar, res = ELT[op]
            t = ins.typ or ELT_DEFAULT_TYPE.get(op) or "INT"
            args = st[-ar:]
            a0 = args[0]
            kind = a0.kind if res is None else (args[1].kind if res == "A2" else res)
            L = a0.seg_len if a0.kind == "S" else a0.len
            d = self.new(kind, L)
            name = f"{stem}_wu{TYPE_SUFFIX[t]}"
            scr = self.scratch(self.sfn(name + "_scratch")(L))
            self.fn(name)(d.ptr, *[a.ptr for a in args], L, scr)
            self._finish(ar, [d])
        elif op in SCAN or op in REDUCE or op in ("RANK_UP", "RANK_DOWN"):
            t = TYPE_SUFFIX[ins.typ or "INT"]
            x, sd = st[-2], st[-1]
            if op in SCAN:
                name, kind, L = f"{SCAN[op]}_se{t}", x.kind, x.len
            elif op in REDUCE:
                name, kind, L = f"{REDUCE[op]}_re{t}", x.kind, sd.len
            else:
                name, kind, L = ("rku_le" if op == "RANK_UP" else "rkd_le") + t, "I", x.len
            d = self.new(kind, L)
            scr = self.scratch(self.sfn(name + "_scratch")(sd.seg_len, sd.len))
            self.fn(name)(d.ptr, x.ptr, sd.ptr, sd.seg_len, sd.len, scr)
            self._finish(2, [d])
        elif op == "MAKE_SEGDES":
            lens = st[-1]
            sd = self.segdes_from_lengths(lens)
            self._finish(1, [sd])
        elif op == "LENGTHS":
            sd = st[-1]
            d = self.new("I", sd.len)
            self.fn("len_fos")(d.ptr, sd.ptr, sd.seg_len, sd.len,
                               self.scratch(self.sfn("len_fos_scratch")(sd.seg_len, sd.len)))
            self._finish(1, [d])
        elif op == "LENGTH":
            v = st[-1]
            self._finish(1, [self.const_scalar("I", v.seg_len if v.kind == "S" else v.len)])
        elif op == "PACK":
            self._pack(ins)
        elif op == "DIST":
            t = TYPE_SUFFIX[ins.typ or "INT"]
            v, sd = st[-2], st[-1]
            d = self.new(v.kind, sd.seg_len)
            name = f"dis_ve{t}"
            self.fn(name)(d.ptr, v.ptr, sd.ptr, sd.seg_len, sd.len,
                          self.scratch(self.sfn(name + "_scratch")(sd.seg_len, sd.len)))
            self._finish(2, [d])
        elif op == "INDEX":
            init, stride, sd = st[-3], st[-2], st[-1]
            d = self.new("I", sd.seg_len)
            self.fn("ind_lez")(d.ptr, init.ptr, stride.ptr, sd.ptr, sd.seg_len, sd.len,
                               self.scratch(self.sfn("ind_lez_scratch")(sd.seg_len, sd.len)))
            self._finish(3, [d])
        elif op == "EXTRACT":
            t = TYPE_SUFFIX[ins.typ or "INT"]
            x, idx, sd = st[-3], st[-2], st[-1]
            d = self.new(x.kind, idx.len)
            name = f"ext_ve{t}"
            self.fn(name)(d.ptr, x.ptr, idx.ptr, sd.ptr, sd.seg_len, sd.len,
                          self.scratch(self.sfn(name + "_scratch")(sd.seg_len, sd.len)))
            self._finish(3, [d])
        elif op == "REPLACE":
            t = TYPE_SUFFIX[ins.typ or "INT"]
            x, idx, val, sd = st[-4], st[-3], st[-2], st[-1]
            if x.ref == 1 and not x.const:  # the only reference: replace in place
                x.ref += 1
                d = x
            else:
                d = self.new(x.kind, x.len)
                cp = f"cpy_wu{t}"
                self.fn(cp)(d.ptr, x.ptr, x.len, self.scratch(self.sfn(cp + "_scratch")(x.len)))
            name = f"rep_ve{t}"
            self.fn(name)(d.ptr, idx.ptr, val.ptr, sd.ptr, sd.seg_len, sd.len,
                          self.scratch(self.sfn(name + "_scratch")(sd.seg_len, sd.len)))
            self._finish(4, [d])
        elif op == "PERMUTE":
            t = TYPE_SUFFIX[ins.typ or "INT"]
            x, idx, sd = st[-3], st[-2], st[-1]
            d = self.new(x.kind, x.len)
            name = f"smp_pe{t}"
            self.fn(name)(d.ptr, x.ptr, idx.ptr, sd.ptr, sd.seg_len, sd.len,
                          self.scratch(self.sfn(name + "_scratch")(sd.seg_len, sd.len)))
            self._finish(3, [d])
        elif op == "BPERMUTE":
            t = TYPE_SUFFIX[ins.typ or "INT"]
            x, idx, sds, sdd = st[-4], st[-3], st[-2], st[-1]
            d = self.new(x.kind, idx.len)
            name = f"bck_pe{t}"
            self.fn(name)(d.ptr, x.ptr, idx.ptr, sds.ptr, sds.seg_len, sds.len, sdd.ptr, sdd.seg_len, sdd.len,
                          self.scratch(self.sfn(name + "_scratch")(sds.seg_len, sds.len, sdd.seg_len, sdd.len)))
            self._finish(4, [d])
        elif op == "DPERMUTE":
            t = TYPE_SUFFIX[ins.typ or "INT"]
            x, idx, dflt, sds, sdd = st[-5], st[-4], st[-3], st[-2], st[-1]
            if dflt.ref == 1 and not dflt.const:  # the default dies here: permute into it
                dflt.ref += 1
                d = dflt
            else:
                d = self.new(x.kind, dflt.len)
            name = f"dpe_pe{t}"
            self.fn(name)(d.ptr, x.ptr, idx.ptr, dflt.ptr, sds.ptr, sds.seg_len, sds.len, sdd.ptr, sdd.seg_len,
                          sdd.len,
                          self.scratch(self.sfn(name + "_scratch")(sds.seg_len, sds.len, sdd.seg_len, sdd.len)))
            self._finish(5, [d])
        elif op in ("FPERMUTE", "BFPERMUTE"):
            t = TYPE_SUFFIX[ins.typ or "INT"]
            x, idx, flg, sds, sdd = st[-5], st[-4], st[-3], st[-2], st[-1]
            d = self.new(x.kind, sdd.seg_len)
            name = ("fpm_pe" if op == "FPERMUTE" else "bfp_pe") + t
            self.fn(name)(d.ptr, x.ptr, idx.ptr, flg.ptr, sds.ptr, sds.seg_len, sds.len, sdd.ptr, sdd.seg_len,
                          sdd.len,
                          self.scratch(self.sfn(name + "_scratch")(sds.seg_len, sds.len, sdd.seg_len, sdd.len)))
            self._finish(5, [d])
        elif op == "DFPERMUTE":
            t = TYPE_SUFFIX[ins.typ or "INT"]
            x, idx, flg, dflt, sds, sdd = st[-6:]
            d = self.new(x.kind, dflt.len)
            name = f"dfp_pe{t}"
            self.fn(name)(d.ptr, x.ptr, idx.ptr, flg.ptr, dflt.ptr, sds.ptr, sds.seg_len, sds.len, sdd.ptr,
                          sdd.seg_len, sdd.len,
                          self.scratch(self.sfn(name + "_scratch")(sds.seg_len, sds.len, sdd.seg_len, sdd.len)))
            self._finish(6, [d])
        elif op == "FUSED":
            fz = self.fused
            if fz is None:
                raise VcodeError(f"line {ins.line}: FUSED {ins.a} without a fused library")
            k = ins.a
            ar = fz.arity(k)
            args = st[-ar:]
            a0 = args[0]
            L = a0.seg_len if a0.kind == "S" else a0.len
            d = self.new(fz.result_kind(k), L)
            fz.fn[k](d.ptr, *[a.ptr for a in args], L, None)
            self._finish(ar, [d])
        elif op == "SRAND":
            s = st[-1]
            self.fn("rnd_foz")(self.scalar_int(s))
            self._finish(1, [self.const_scalar("B", True)])
        elif op in ("READ", "WRITE", "FREAD", "FWRITE", "FOPEN", "FCLOSE", "FREAD_CHAR", "SPAWN"):
            self._io(ins)
        else:
            raise VcodeError(f"line {ins.line}: {op} is not supported")

    # -- I/O (vinterp's nesl/vcode/io.c: text forms "(1 2 3)" INT, "(1.0 2.0)"
    # FLOAT, "(T F)" BOOL, "[1 2 3]" SEGDES by its lengths, "\"text\"" CHAR as
    # character codes; every operation leaves an error string -- empty on
    # success -- and a success flag on top of the stack)
    def _push_io_status(self, err: str | None):
        codes = np.frombuffer(err.encode("latin-1"), dtype=np.uint8).astype(np.int32) if err else []
        self.stack.append(self.from_host("I", codes))
        self.stack.append(self.const_scalar("B", not err))

    def _fd_from_stack(self, ins):
        v = self.stack.pop()
        fd = self.scalar_int(v)
        self.drop(v)
        if fd == NULL_STREAM_FD:
            return fd, None  # as vinterp: no message, and no stream
        if fd not in self.files:
            return None, f"vinterp: line {ins.line}: illegal VCODE file descriptor for {ins.op}: {fd}"
        return fd, None

    def _read(self, ins, stream):
        kind = KIND_OF.get(ins.typ, "I")
        empty_kind = "I" if kind == "S" or ins.typ == "CHAR" else kind
        value, err = stream.read_vector(ins.typ) if stream is not None else (None, None)
        if value is None:
            self.stack.append(self.new(empty_kind, 0))
        elif ins.typ == "SEGDES":
            lens = self.from_host("I", value)
            self.stack.append(self.segdes_from_lengths(lens))
            self.drop(lens)
        else:
            self.stack.append(self.from_host("I" if ins.typ == "CHAR" else kind, value))
        self._push_io_status(err)

    def _write(self, ins, stream):
        v = self.stack.pop()
        err = None
        try:
            if ins.typ == "CHAR":
                stream.write("".join(map(chr, self.to_host(v).tolist())))
            else:
                stream.write(format_vector(v.kind, self.to_host(v)))
        except (OSError, ValueError) as e:
            err = str(e)
        self.drop(v)
        self._push_io_status(err)

    def _io(self, ins):
        st = self.stack
        op = ins.op
        if op == "READ":
            self._read(ins, self.files[0])
        elif op == "WRITE":
            self._write(ins, self.files[1])
        elif op == "FREAD":
            fd, err = self._fd_from_stack(ins)
            if fd is None or fd < 0:
                st.append(self.new("I" if ins.typ in ("SEGDES", "CHAR") else KIND_OF.get(ins.typ, "I"), 0))
                self._push_io_status(err)
            else:
                self._read(ins, self.files[fd])
        elif op == "FWRITE":
            fd, err = self._fd_from_stack(ins)
            if fd is None or fd < 0:
                self.drop(st.pop())
                self._push_io_status(err or f"illegal VCODE file descriptor in FWRITE")
            else:
                self._write(ins, self.files[fd])
        elif op == "FOPEN":
            mv = st.pop()
            mode = self.scalar_int(mv)
            self.drop(mv)
            if mode not in (1, 2, 3):
                raise VcodeError(f"line {ins.line}: FOPEN: top of stack ({mode}) not legal mode.")
            nv = st.pop()
            name = "".join(map(chr, self.to_host(nv).tolist()))
            self.drop(nv)
            fd, err = -1, None
            try:
                # bytes in and out as they are (vinterp's stdio streams): no
                # newline translation, one character per byte
                f = open(name, {1: "r", 2: "w", 3: "a"}[mode], encoding="latin-1", newline="")
                free = [k for k in range(3, MAX_FILES) if k not in self.files]
                if free:
                    fd = free[0]
                    self.files[fd] = _VStream(f)
                else:
                    f.close()
                    err = "no room in internal file table"
            except OSError as e:
                err = e.strerror or str(e)
            st.append(self.from_host("I", [fd]))
            self._push_io_status(err)
        elif op == "FREAD_CHAR":
            # fd, the most characters to read (negative: no limit) and a
            # string of delimiters -> the characters, the stop status, the
            # error string and the success flag (io.c:1134-1300)
            fd, err = self._fd_from_stack(ins)
            mv, dv = st.pop(), st.pop()
            if fd is None or fd < 0:
                self.drop(mv)
                self.drop(dv)
                st.append(self.new("I", 0))
                st.append(self.new("I", 0))
                self._push_io_status(err or "illegal VCODE file descriptor in FREAD")
            else:
                max_char = self.scalar_int(mv)
                delims = set(self.to_host(dv).tolist())
                self.drop(mv)
                self.drop(dv)
                codes, stop = self.files[fd].read_chars(max_char if max_char >= 0 else 1 << 30, delims)
                st.append(self.from_host("I", codes))
                st.append(self.from_host("I", [stop]))
                self._push_io_status(None)
        elif op == "SPAWN":
            self._spawn(ins)
        elif op == "FCLOSE":
            fd, err = self._fd_from_stack(ins)
            if fd is not None and fd >= 0:
                stream = self.files.pop(fd)
                if fd > 2:
                    stream.f.close()
                else:
                    stream.f.flush()
            self._push_io_status(err)

    def _spawn(self, ins):
        """SPAWN (io.c do_spawn): a command string and the child's stdin,
        stdout and stderr descriptors (top of stack last); a null stream
        (-1) gets a pipe whose other end becomes a new descriptor here.
        The command is split at white space and run from PATH.  Leaves the
        child's stderr, stdout and stdin descriptors, then the error string
        and the success flag."""
        import subprocess
        st = self.stack
        fds, err = [], None
        for _ in range(3):  # err, out, in
            fd, e = self._fd_from_stack(ins)
            fds.append(fd)
            err = err or e
        err_fd, out_fd, in_fd = fds
        cv = st.pop()
        argv = "".join(map(chr, self.to_host(cv).tolist())).split()
        self.drop(cv)
        if err is None:
            def target(fd, pipe):
                return subprocess.PIPE if fd == NULL_STREAM_FD else self.files[fd].f.fileno()
            free = [k for k in range(3, MAX_FILES) if k not in self.files]
            if len(free) < [in_fd, out_fd, err_fd].count(NULL_STREAM_FD):
                err = "no room in internal file table"
            else:
                for f in (self.files.get(k) for k in (in_fd, out_fd, err_fd)):
                    if f is not None:
                        f.f.flush()
                try:
                    proc = subprocess.Popen(argv, stdin=target(in_fd, 0), stdout=target(out_fd, 1),
                                            stderr=target(err_fd, 2))
                    new = []
                    for fd, pipe in ((in_fd, proc.stdin), (out_fd, proc.stdout), (err_fd, proc.stderr)):
                        if fd == NULL_STREAM_FD:
                            k = free.pop(0)
                            self.files[k] = _VStream(io.TextIOWrapper(pipe, encoding="latin-1", newline="",
                                                                      write_through=True))
                            new.append(k)
                        else:
                            new.append(fd)
                    in_fd, out_fd, err_fd = new
                except OSError as e:
                    err = "SPAWN: error performing fork:" + (e.strerror or str(e))
        if err is not None:
            in_fd = out_fd = err_fd = NULL_STREAM_FD
        for fd in (err_fd, out_fd, in_fd):
            st.append(self.from_host("I", [fd]))
        self._push_io_status(err)

    def _finish(self, nargs, results):
        st = self.stack
        for v in st[len(st) - nargs:]:
            self.drop(v)
        del st[len(st) - nargs:]
        st.extend(results)

    def _pack(self, ins):
        st = self.stack
        t = TYPE_SUFFIX[ins.typ or "INT"]
        x, flg, sd = st[-3], st[-2], st[-1]
        n, m = sd.seg_len, sd.len
        lens = self.new("I", m)
        self.fn("pk1_lev")(lens.ptr, flg.ptr, sd.ptr, n, m, self.scratch(self.sfn("pk1_lev_scratch")(n, m)))
        dsd = self.segdes_from_lengths(lens)
        self.drop(lens)
        d = self.new(x.kind, dsd.seg_len)
        name = f"pk2_le{t}"
        self.fn(name)(d.ptr, x.ptr, flg.ptr, sd.ptr, n, m, dsd.ptr, dsd.seg_len, m,
                      self.scratch(self.sfn(name + "_scratch")(n, m, dsd.seg_len, m)))
        self._finish(3, [d, dsd])


def run_program(text: str, cvl: CVL | None = None, entry: str | None = None, args=None, sync=None):
    """Parses and runs; returns (interpreter, final stack)."""
    it = Interpreter(text, cvl, sync=sync)
    out = it.run(entry, args)
    return it, out
