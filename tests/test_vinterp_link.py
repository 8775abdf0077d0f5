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
from oracle.oracle import reference_root

_REF = reference_root()
REF = _REF / "nesl" / "vcode" if _REF else Path("/nonexistent")
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


# Reads a generated fused library the way vinterp's loader does
# (nesl/vcode/fusion.c:18-42): dlopen, then vops and cvl_funs through the
# reference's own vopdes_t / cvl_triple_t (nesl/vcode/vcode.h:73-100), and
# init as the reference's CUDA CVL calls it.  Prints one line per entry.
_LOADER = r"""
#include <dlfcn.h>
#include <stdio.h>
#include <stdlib.h>
#include "config.h"
#include "vcode.h"
#include "y.tab.h"
int main(int argc, char **argv) {
  int n = atoi(argv[2]), k, i;
  void *h = dlopen(argv[1], RTLD_NOW);
  if (!h) { printf("dlopen: %s\n", dlerror()); return 1; }
  vopdes_t *v = (vopdes_t *)dlsym(h, "vops");
  cvl_triple_t *f = (cvl_triple_t *)dlsym(h, "cvl_funs");
  void (*init)(void *) = (void (*)(void *))dlsym(h, "init");
  if (!v || !f || !init) { printf("missing symbol\n"); return 1; }
  init((void *)0);
  for (k = 0; k < n; k++) {
    char name[32];
    sprintf(name, "fused%d", k);
    printf("%d %s %d %d %d", v[k].vop - FUSED, v[k].vopname, v[k].arg_num, v[k].result_num, (int)v[k].cvl_desc);
    for (i = 0; i < v[k].arg_num; i++) printf(" t%d l%u", (int)v[k].arg_type[i], v[k].arg_len[i]);
    printf(" r%d rl%u s%d", (int)v[k].result_type[0], v[k].result_len[0], v[k].arg_for_scratch[0]);
    printf(" fn%d sc%d ip%u\n", (void *)f[k].cvl_int.function == dlsym(h, name),
           f[k].cvl_int.scratch_function(1000), f[k].cvl_int.inplace_function());
  }
  return 0;
}
"""


@pytest.mark.skipif(not (REF / "vcode.h").exists(), reason="reference tree not mounted")
def test_generated_fused_library_loads_like_vinterp(tmp_path):
    """A library generated from the reference's muladd super-op definitions
    (bench/NESL/muladd.cu's trailing comment) holds the tables vinterp reads,
    laid out as its vcode.h declares them, with the fusion compiler's entries
    (nesl/fusion/super-op-gen.sml:346-440): argument types, AGREE1 or COMPAT1
    result length, ElwiseK, INPLACE of the first non-descriptor argument."""
    from neslgpu_gb300 import fcode as F
    muladd = REF.parent.parent / "bench" / "NESL" / "muladd.cu"
    ops = F.parse_defs(muladd.read_text())
    assert [o.number for o in ops] == [0, 1]
    ytab = tmp_path / "y.tab.h"
    ytab.write_text(_ytab((REF / "grammar.yy").read_text()))
    so = F.build_library(ops, tmp_path, ytab=ytab)
    src = tmp_path / "loader.c"
    src.write_text(_LOADER)
    exe = tmp_path / "loader"
    r = subprocess.run(["gcc", "-w", "-std=gnu99", f"-I{tmp_path}", f"-I{REF}", str(src), "-o", str(exe), "-ldl"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe), str(so), "2"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = r.stdout.splitlines()
    # vcode.h: Int = 4, Segdes = 6; NONE = 0, AGREE1 = 1, COMPAT1 = 0x20; ElwiseK = K
    assert lines[0] == "0 fused0 1 1 1 t6 l0 r4 rl32 s1 fn1 sc0 ip0"
    assert lines[1] == "1 fused1 3 1 3 t4 l0 t4 l0 t4 l0 r4 rl1 s1 fn1 sc0 ip1"
