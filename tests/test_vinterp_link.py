"""vinterp, the reference's VCODE interpreter, compiles unchanged against
include/cvl_gb300.h (installed as cvl.h) and links against
libcvl_gb300.so: every CVL function it calls resolves in this library.

The interpreter's sources are compiled where they lie in the reference tree
(the test is skipped where that tree is not mounted).  Its yacc grammar
cannot be generated here (no yacc/lex), so the token header is derived from
the grammar's %token declarations in declaration order from 257, as yacc
numbers them, and tests/vinterp/parser_stub.c stands in for the parser."""
import os
import re
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
REF = Path(os.environ.get("GCVL_REFERENCE", "/root/reference")) / "nesl" / "vcode"
SOURCES = ["actions", "link_list", "main", "symbol_table", "program", "vcode_table", "rtstack", "stack",
           "vstack", "check_args", "cvl_table", "constant", "io", "vcode_hash", "fusion", "vcode-profile"]


def _ytab(grammar: str) -> str:
    toks = []
    for line in grammar.splitlines():
        m = re.match(r"%token\s*(<\w+>)?\s*(.*)", line)
        if m:
            toks += m.group(2).split()
    union = re.search(r"%union\s*\{(.*?)\}", grammar, re.S).group(1)
    lines = ["#ifndef Y_TAB_H", "#define Y_TAB_H"]
    lines += [f"#define {t} {257 + i}" for i, t in enumerate(toks)]
    lines += ["typedef union {" + union + "} YYSTYPE;", "extern YYSTYPE yylval;", "#endif"]
    return "\n".join(lines) + "\n"


@pytest.mark.skipif(not (REF / "main.c").exists(), reason="reference tree not mounted")
def test_vinterp_links_against_library(tmp_path):
    lib = ROOT / "neslgpu_gb300" / "libcvl_gb300.so"
    assert lib.exists(), "build the library first"
    (tmp_path / "y.tab.h").write_text(_ytab((REF / "grammar.yy").read_text()))
    shutil.copy(ROOT / "include" / "cvl_gb300.h", tmp_path / "cvl.h")
    objs = []
    for name in SOURCES:
        obj = tmp_path / f"{name}.o"
        r = subprocess.run(["gcc", "-std=gnu89", "-w", "-O1", f"-I{tmp_path}", f"-I{REF}", "-c",
                            str(REF / f"{name}.c"), "-o", str(obj)], capture_output=True, text=True)
        assert r.returncode == 0, f"{name}.c: {r.stderr[-1500:]}"
        objs.append(str(obj))
    stub = tmp_path / "parser_stub.o"
    r = subprocess.run(["gcc", "-w", f"-I{tmp_path}", f"-I{REF}", "-c",
                        str(ROOT / "tests" / "vinterp" / "parser_stub.c"), "-o", str(stub)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    exe = tmp_path / "vinterp"
    r = subprocess.run(["gcc", "-o", str(exe), *objs, str(stub), f"-L{lib.parent}", "-lcvl_gb300",
                        "-lm", "-ldl"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    # every CVL symbol vinterp references is defined by the library
    undef = subprocess.run(["nm", "-u", str(exe)], capture_output=True, text=True).stdout.split()
    from neslgpu_gb300 import abi
    cvl_refs = [s for s in undef if s in abi.CVL]
    exported = subprocess.run(["nm", "-D", "--defined-only", str(lib)], capture_output=True, text=True).stdout
    missing = [s for s in cvl_refs if f" T {s}\n" not in exported]
    assert cvl_refs and not missing, missing
