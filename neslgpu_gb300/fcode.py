"""Fused super-ops for .fcode programs, generated as sm_103a CUDA kernels.

The NESL fusion compiler turns chains of elementwise VCODE operations into
super-ops (``FUSED k`` in an .fcode program) and records each one's
definition as a small expression, e.g.

    fused OP3#2 ($0 : INT, $1 : SEGDES) = (/ INT @ $0 (DIST INT @ (CONST INT 2) $1))

(the format of the trailing comments of the reference's bench/NESL/*.cu;
semantics after nesl/fusion/super-op-gen.sml).  This module parses such
definitions and generates one CUDA kernel per super-op that evaluates the
whole expression per element with the library's own element functions
(``csrc/elt_ops.cuh``), so a fused op computes exactly what the chain of
``*_wu*`` calls it replaces computes.  The kernels read every input once
and write the result once (four elements in flight per thread), take
``vec_p`` device pointers and run on the library stream.

``FusedLib(defs)`` compiles the definitions with nvcc (cached by content)
and exposes them to the VCODE interpreter (``vcode.Interpreter(...,
fused=lib)``), which runs ``FUSED k`` like vinterp runs a fused library's
op k: arguments from the stack, result length that of the first argument
(the element count of a segment descriptor argument).

The generated library is also a fused library for the reference's own
interpreter: vinterp ``dlopen``s the library named by its ``-l`` flag and
takes the operation table ``vops[]`` and the function table ``cvl_funs[]``
from it (nesl/vcode/fusion.c:18-42); the reference's CUDA CVL also calls the
library's ``init`` with its heap base (nesl/cvl/cuda/facilities.c:206-221).
All three are exported, with the layouts of ``vopdes_t`` and
``cvl_triple_t`` (nesl/vcode/vcode.h:73-100) and entries made by the fusion
compiler's rules (nesl/fusion/super-op-gen.sml:346-440).  The entries carry
vinterp's token numbers: pass its ``y.tab.h`` as ``build_library(...,
ytab=path)``; without one, the numbers bison -y gives the grammar
(nesl/vcode/grammar.yy:43-96, 258 + declaration index) are used.
"""
from __future__ import annotations

import ctypes as C
import hashlib
import os
import re
import subprocess
from dataclasses import dataclass
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
INCLUDE = PKG.parent / "include"
CACHE = PKG / "_fused"

CTYPE = {"INT": "int", "BOOL": "int", "FLOAT": "double"}
KIND = {"INT": "I", "BOOL": "B", "FLOAT": "F", "SEGDES": "S"}
SFX = {"INT": "z", "BOOL": "b", "FLOAT": "d"}

# op -> (element-function stem, arity, result type rule)
#   rule: a type name, "T" (the op's own type), or "B" (BOOL)
OPS = {
    "+": ("add", 2, "T"), "-": ("sub", 2, "T"), "*": ("mul", 2, "T"), "/": ("div", 2, "T"),
    "%": ("mod", 2, "INT"), "<": ("les", 2, "BOOL"), "<=": ("leq", 2, "BOOL"), ">": ("grt", 2, "BOOL"),
    ">=": ("geq", 2, "BOOL"), "=": ("eql", 2, "BOOL"), "!=": ("neq", 2, "BOOL"), "LSHIFT": ("lsh", 2, "INT"),
    "RSHIFT": ("rsh", 2, "INT"), "AND": ("and", 2, "T"), "OR": ("ior", 2, "T"), "XOR": ("xor", 2, "T"),
    "NOT": ("not", 1, "T"), "I_TO_F": ("dbl", 1, "FLOAT"), "I_TO_B": ("boo", 1, "BOOL"),
    "B_TO_I": ("int", 1, "INT"), "FLOOR": ("flr", 1, "INT"), "CEIL": ("cei", 1, "INT"),
    "TRUNC": ("trn", 1, "INT"), "ROUND": ("rou", 1, "INT"), "LOG": ("log", 1, "FLOAT"),
    "SQRT": ("sqt", 1, "FLOAT"), "EXP": ("exp", 1, "FLOAT"), "SIN": ("sin", 1, "FLOAT"),
    "COS": ("cos", 1, "FLOAT"), "TAN": ("tan", 1, "FLOAT"), "ASIN": ("asn", 1, "FLOAT"),
    "ACOS": ("acs", 1, "FLOAT"), "ATAN": ("atn", 1, "FLOAT"), "SINH": ("snh", 1, "FLOAT"),
    "COSH": ("csh", 1, "FLOAT"), "TANH": ("tnh", 1, "FLOAT"),
}
# the operand type of ops written without one (grammar.yy:160-243)
UNTYPED = {"%": "INT", "LSHIFT": "INT", "RSHIFT": "INT", "I_TO_F": "INT", "I_TO_B": "INT", "B_TO_I": "BOOL",
           "FLOOR": "FLOAT", "CEIL": "FLOAT", "TRUNC": "FLOAT", "ROUND": "FLOAT", "LOG": "FLOAT",
           "SQRT": "FLOAT", "EXP": "FLOAT", "SIN": "FLOAT", "COS": "FLOAT", "TAN": "FLOAT", "ASIN": "FLOAT",
           "ACOS": "FLOAT", "ATAN": "FLOAT", "SINH": "FLOAT", "COSH": "FLOAT", "TANH": "FLOAT"}


class FcodeError(ValueError):
    pass


@dataclass
class Node:
    kind: str          # "arg", "const", "op", "select", "dist"
    typ: str           # result type: INT, BOOL, FLOAT
    op: str = ""
    optype: str = ""   # the op's operand type
    args: tuple = ()
    index: int = -1    # arg number
    value: str = ""    # const literal


@dataclass
class FusedOp:
    number: int
    params: list       # [(index, type)]
    expr: Node

    @property
    def result(self) -> str:
        return self.expr.typ


_DEF = re.compile(r"fused\s+OP(\d+)#\d+\s*\(([^)]*)\)\s*=\s*", re.S)
_TOK = re.compile(r"\(|\)|@|\$\d+|[^\s()@]+")


def parse_defs(text: str) -> list[FusedOp]:
    """All `fused OPk#c (...) = EXPR` definitions in text (expressions may
    run over several lines)."""
    out = []
    for mt in _DEF.finditer(text):
        number = int(mt.group(1))
        params = []
        for p in mt.group(2).split(","):
            p = p.strip()
            if not p:
                continue
            name, typ = (x.strip() for x in p.split(":"))
            params.append((int(name[1:]), typ))
        # the expression: balanced parentheses from here
        i, depth, start = mt.end(), 0, mt.end()
        while i < len(text):
            ch = text[i]
            if ch == "(":
                depth += 1
            elif ch == ")":
                depth -= 1
                if depth == 0:
                    i += 1
                    break
            elif ch == "$" and depth == 0:  # a bare argument
                m2 = re.match(r"\$\d+", text[i:])
                i += m2.end()
                break
            i += 1
        toks = _TOK.findall(text[start:i])
        ptype = dict(params)
        node, k = _parse_expr(toks, 0, ptype)
        if k != len(toks):
            raise FcodeError(f"OP{number}: trailing tokens")
        out.append(FusedOp(number, params, node))
    out.sort(key=lambda o: o.number)
    return out


def _parse_expr(toks, k, ptype):
    t = toks[k]
    if t.startswith("$"):
        j = int(t[1:])
        typ = ptype[j]
        return Node("arg", typ, index=j), k + 1
    if t != "(":
        raise FcodeError(f"unexpected {t!r}")
    op = toks[k + 1]
    if op == "CONST":
        typ, val = toks[k + 2], toks[k + 3]
        if toks[k + 4] != ")":
            raise FcodeError("CONST takes one value")
        return Node("const", typ, value=val), k + 5
    k += 2
    optype = None
    if toks[k] != "@":
        optype = toks[k]
        k += 1
    if toks[k] != "@":
        raise FcodeError(f"{op}: expected @")
    k += 1
    args = []
    while toks[k] != ")":
        a, k = _parse_expr(toks, k, ptype)
        args.append(a)
    k += 1
    if op == "DIST":
        if len(args) != 2 or args[0].kind != "const":
            raise FcodeError("DIST of a constant only")
        return Node("dist", args[0].typ, args=tuple(args)), k
    if op == "SELECT":
        if len(args) != 3:
            raise FcodeError("SELECT takes three operands")
        return Node("select", optype or args[1].typ, optype=optype or args[1].typ, args=tuple(args)), k
    if op not in OPS:
        raise FcodeError(f"operation {op} cannot be fused")
    stem, ar, rule = OPS[op]
    if len(args) != ar:
        raise FcodeError(f"{op} takes {ar} operands")
    optype = optype or UNTYPED.get(op) or args[0].typ
    typ = optype if rule == "T" else rule
    return Node("op", typ, op=op, optype=optype, args=tuple(args)), k


# ------------------------------------------------------------- emission ---
def _literal(typ, value):
    if typ == "FLOAT":
        return repr(float(value))
    if typ == "BOOL":
        return "1" if value in ("T", "1") else "0"
    return f"({int(value)})"


def _expr(n: Node) -> str:
    if n.kind == "arg":
        return f"x{n.index}"
    if n.kind == "const":
        return _literal(n.typ, n.value)
    if n.kind == "dist":
        return _literal(n.args[0].typ, n.args[0].value)
    if n.kind == "select":
        c, a, b = (_expr(x) for x in n.args)
        return f"(({c}) ? ({a}) : ({b}))"
    stem = OPS[n.op][0]
    sfx = SFX[n.optype]
    if n.optype == "BOOL" and stem in ("eql", "neq"):
        sfx = "z"  # booleans compare as ints (eql_wub)
    return f"gcvl::f_{stem}_{sfx}::f({', '.join(_expr(a) for a in n.args)})"


# vinterp's enumerations (nesl/vcode/vcode.h:12-13, 38-48, 58-70) and the
# bison -y token numbers of the two opcodes a fused table names
# (nesl/vcode/grammar.yy: MAKE_SEGDES is token 66 and FUSED token 112 in
# declaration order, numbered from 258)
VTYPE = {"BOOL": 3, "INT": 4, "FLOAT": 5, "SEGDES": 6}
AGREE1, COMPAT1 = 0x1, 0x20
CVL_DESC_SEGOP, CVL_DESC_NOT_SUPPORTED = 44, 56
BISON_FUSED, BISON_MAKE_SEGDES = 258 + 112, 258 + 66
MAX_ARGS = 40


def _vinterp_tables(ops: list[FusedOp]) -> list[str]:
    """vops[], cvl_funs[] and init() for vinterp's fused-library loader,
    indexed by super-op number (numbers missing from the definitions get a
    NotSupported entry)."""
    lines = [
        "// ---- the fused-library interface of vinterp (fusion.c:18-42) ----",
        "#ifdef GCVL_VINTERP_YTAB",
        "#include GCVL_VINTERP_YTAB",
        "#endif",
        "#ifndef FUSED",
        f"#define FUSED {BISON_FUSED}",
        "#endif",
        "#ifndef MAKE_SEGDES",
        f"#define MAKE_SEGDES {BISON_MAKE_SEGDES}",
        "#endif",
        "struct gcvl_vopdes {  // vopdes_t",
        "  int vop; const char *vopname; int arg_num; int result_num;",
        f"  int arg_type[{MAX_ARGS}]; unsigned arg_len[{MAX_ARGS}]; int result_type[3]; unsigned result_len[3];",
        f"  int arg_for_scratch[{MAX_ARGS}]; int cvl_desc;",
        "};",
        "struct gcvl_funct { void (*function)(); int (*scratch_function)(); unsigned (*inplace_function)(); };",
        "struct gcvl_triple { gcvl_funct cvl_int, cvl_float, cvl_boolean; };  // cvl_triple_t",
        "// vec_p is a device pointer in this library: the heap base is not needed",
        "static void *g_heap_base = 0;",
        'extern "C" __attribute__((visibility("default"))) void init(void *mem) { g_heap_base = mem; }',
        'extern "C" __attribute__((visibility("default"))) void fused_unsupported(void) {}',
        'extern "C" __attribute__((visibility("default"))) int fused_unsupported_scratch(void) { return 0; }',
        'extern "C" __attribute__((visibility("default"))) unsigned fused_unsupported_inplace(void) { return 0; }',
    ]
    by = {o.number: o for o in ops}
    top = max(by) + 1 if by else 0
    vops, funs = [], []
    for k in range(top):
        o = by.get(k)
        if o is None:
            vops.append(f'  {{FUSED + {k}, "unsupported", 0, 0, {{0}}, {{0}}, {{0}}, {{0}}, {{0}}, '
                        f'{CVL_DESC_NOT_SUPPORTED}}},')
            f = ("fused_unsupported",) * 3
        else:
            arity = len(o.params)
            if arity > MAX_ARGS:
                raise FcodeError(f"OP{k}: {arity} arguments, vinterp takes at most {MAX_ARGS}")
            types = ", ".join(str(VTYPE[t]) for _, t in o.params) or "0"
            seg_result = o.result == "SEGDES"
            vop = "MAKE_SEGDES" if seg_result else f"FUSED + {k}"
            rlen = COMPAT1 if o.params and o.params[0][1] == "SEGDES" else AGREE1
            desc = CVL_DESC_SEGOP if seg_result else arity
            vops.append(f'  {{{vop}, "fused{k}", {arity}, 1, {{{types}}}, {{0}}, {{{VTYPE[o.result]}}}, '
                        f'{{{rlen}}}, {{1}}, {desc}}},')
            f = (f"fused{k}", f"fused{k}_scratch", f"fused{k}_inplace")
        slot = f"{{(void (*)()){f[0]}, (int (*)()){f[1]}, (unsigned (*)()){f[2]}}}"
        funs.append(f"  {{{slot}, {slot}, {slot}}},")
    lines.append(f'extern "C" __attribute__((visibility("default"))) gcvl_vopdes vops[{max(top, 1)}] = {{')
    lines += vops or ['  {0, "none", 0, 0, {0}, {0}, {0}, {0}, {0}, ' + f"{CVL_DESC_NOT_SUPPORTED}}},"]
    lines.append("};")
    lines.append(f'extern "C" __attribute__((visibility("default"))) gcvl_triple cvl_funs[{max(top, 1)}] = {{')
    unsup = "{(void (*)())fused_unsupported, (int (*)())fused_unsupported_scratch, " \
            "(unsigned (*)())fused_unsupported_inplace}"
    lines += funs or [f"  {{{unsup}, {unsup}, {unsup}}},"]
    lines.append("};")
    return lines


def _inplace_flag(o: FusedOp) -> int:
    """INPLACE_i for the first argument i (from 1) that is not a segment
    descriptor, none for a descriptor result (super-op-gen.sml:355-366).
    Every generated kernel reads all of an element's inputs before writing
    it, so any such argument may share the result's memory."""
    if o.result == "SEGDES":
        return 0
    for i, (_, t) in enumerate(o.params, start=1):
        if t != "SEGDES":
            return 1 << (i - 1)
    return 0


def emit_cuda(ops: list[FusedOp]) -> str:
    lines = [
        "// generated by neslgpu_gb300/fcode.py from fused super-op definitions",
        "#include <cuda_runtime.h>",
        "#include <math.h>",
        '#include "elt_ops.cuh"',
        'extern "C" void *gcvl_get_stream(void);',
        "static int fused_grid(long n) { long g = (n + 1023) / 1024; return (int)(g < 1 ? 1 : (g > 4864 ? 4864 : g)); }",
    ]
    for o in ops:
        k = o.number
        ins = [(j, t) for j, t in o.params]
        rt = CTYPE[o.result]
        kparams = [f"{rt} *__restrict__ d"] + [
            f"const {CTYPE[t]} *__restrict__ s{j}" for j, t in ins if t != "SEGDES"] + ["long n"]
        lines.append(f"__global__ void __launch_bounds__(256) k_fused{k}({', '.join(kparams)}) {{")
        lines.append("  const long stride = (long)gridDim.x * 256 * 4;")
        lines.append("  for (long b = (long)blockIdx.x * 256 * 4 + threadIdx.x; b < n; b += stride) {")
        used = sorted({j for j, t in ins if t != "SEGDES"})
        for j in used:
            t = dict(ins)[j]
            lines.append(f"    {CTYPE[t]} v{j}[4];")
        lines.append("#pragma unroll")
        lines.append("    for (int u = 0; u < 4; u++) { const long i = b + (long)u * 256; if (i < n) {")
        for j in used:
            lines.append(f"      v{j}[u] = __ldcs(s{j} + i);")
        lines.append("    } }")
        lines.append("#pragma unroll")
        lines.append("    for (int u = 0; u < 4; u++) { const long i = b + (long)u * 256; if (i < n) {")
        for j in used:
            lines.append(f"      const {CTYPE[dict(ins)[j]]} x{j} = v{j}[u];")
        lines.append(f"      d[i] = ({rt})({_expr(o.expr)});")
        lines.append("    } }")
        lines.append("  }")
        lines.append("}")
        cparams = ["void *d"] + [f"void *s{j}" for j, _ in ins] + ["int len", "void *scratch"]
        kargs = [f"({rt} *)d"] + [f"(const {CTYPE[t]} *)s{j}" for j, t in ins if t != "SEGDES"] + ["len"]
        lines.append(f'extern "C" __attribute__((visibility("default"))) void fused{k}({", ".join(cparams)}) {{')
        lines.append("  (void)scratch;")
        for j, t in ins:
            if t == "SEGDES":
                lines.append(f"  (void)s{j};")
        lines.append("  if (len <= 0) return;")
        lines.append(f"  k_fused{k}<<<fused_grid(len), 256, 0, (cudaStream_t)gcvl_get_stream()>>>({', '.join(kargs)});")
        lines.append("}")
        lines.append(f'extern "C" __attribute__((visibility("default"))) int fused{k}_scratch(int len) '
                     "{ (void)len; return 0; }")
        lines.append(f'extern "C" __attribute__((visibility("default"))) unsigned fused{k}_inplace(void) '
                     f"{{ return {_inplace_flag(o)}u; }}")
    lines += _vinterp_tables(ops)
    return "\n".join(lines) + "\n"


def build_library(ops: list[FusedOp], out_dir: Path | None = None, ytab: Path | None = None) -> Path:
    """nvcc the generated source for sm_103a into a shared library (cached
    by the source's hash); returns its path.  ytab: the y.tab.h of the
    vinterp build that will load the library (its token numbers go into
    vops[])."""
    src = emit_cuda(ops)
    key = src + (Path(ytab).read_text() if ytab else "")
    h = hashlib.sha256(key.encode()).hexdigest()[:16]
    d = Path(out_dir or CACHE)
    d.mkdir(parents=True, exist_ok=True)
    so = d / f"fused_{h}.so"
    if so.exists():
        return so
    cu = d / f"fused_{h}.cu"
    cu.write_text(src)
    tmp = d / f"fused_{h}.{os.getpid()}.so"
    # linked against the library for its stream (gcvl_get_stream)
    cmd = ["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-shared",
           "-Xcompiler", "-fPIC", f"-I{CSRC}", f"-I{INCLUDE}", "-o", str(tmp), str(cu),
           *([f'-DGCVL_VINTERP_YTAB="{Path(ytab).resolve()}"'] if ytab else []),
           f"-L{PKG}", "-lcvl_gb300", "-Xlinker", "-rpath", "-Xlinker", str(PKG)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise FcodeError(f"nvcc failed:\n{r.stderr[-3000:]}")
    tmp.replace(so)
    return so


class FusedLib:
    """A compiled set of super-ops, callable as fused k by the interpreter."""

    def __init__(self, defs: str | list[FusedOp], out_dir: Path | None = None):
        self.ops = parse_defs(defs) if isinstance(defs, str) else list(defs)
        self.by_number = {o.number: o for o in self.ops}
        self.path = build_library(self.ops, out_dir)
        self.lib = C.CDLL(str(self.path), mode=C.RTLD_GLOBAL)
        self.fn = {}
        for o in self.ops:
            f = getattr(self.lib, f"fused{o.number}")
            f.restype = None
            f.argtypes = [C.c_void_p] * (1 + len(o.params)) + [C.c_int, C.c_void_p]
            self.fn[o.number] = f

    def arity(self, k: int) -> int:
        return len(self.by_number[k].params)

    def result_kind(self, k: int) -> str:
        return KIND[self.by_number[k].result]
