"""This repository's VCODE programs, written with ``vcode_asm``.

* ``QSORT`` -- quicksort of an int sequence, flattened the way the NESL
  compiler flattens ``quicksort`` (the algorithm of the reference's
  bench/NESL/qs.nesl: the pivot of each segment is its element #a/2;
  lesser, equal and greater elements are split per segment, and the
  recursion works on every segment at once).  One level per call of
  QS_LOOP: per-segment min and max decide whether anything is left to do;
  otherwise three-way split flags, their per-segment exclusive scans and
  counts give every element its place inside its segment (PERMUTE), and
  the counts, interleaved, become the next level's segment lengths (empty
  segments packed away).  A sequence is a (segment descriptor, data) pair
  with the data on top, as NESL represents it.
* ``SPMV`` -- y = A x for A stored as a nested sequence of (column, value)
  rows (CSR): BPERMUTE gathers x by column, elementwise product, segmented
  +_REDUCE per row.
* ``qsort_fcode_program`` -- QSORT with its elementwise chains replaced by
  ``FUSED k`` super-ops, in the form the NESL fusion compiler produces (an
  .fcode program plus the super-op definitions), for ``neslgpu_gb300.fcode``.
"""
from __future__ import annotations

from .vcode_asm import Block, Func


def _qs_loop(fused: bool = False) -> str:
    f = Func("QS_LOOP", params=["keys", "sd"], results=["out"])
    f.op("LENGTHS", ["sd"], ["lens"])
    f.op("MIN_REDUCE INT", ["keys", "sd"], ["mn"])
    f.op("MAX_REDUCE INT", ["keys", "sd"], ["mx"])
    f.op("< INT", ["mn", "mx"], ["ne"])  # unsettled: min < max (never true of an empty segment)
    f.op("B_TO_I", ["ne"], ["nei"])
    f.op("LENGTH INT", ["nei"], ["m"])
    f.op("MAKE_SEGDES", ["m"], ["one_m"])
    f.op("+_REDUCE INT", ["nei", "one_m"], ["open"])
    f.const("INT 0", "zero")
    f.op("> INT", ["open", "zero"], ["more"])

    t = Block()
    # pivot: element #a/2 of each segment
    if fused:
        t.op("FUSED 0", ["lens", "one_m"], ["mid"])          # lens / 2
    else:
        t.const("INT 2", "two")
        t.op("DIST INT", ["two", "one_m"], ["twos"])
        t.op("/ INT", ["lens", "twos"], ["mid"])
    t.op("EXTRACT INT", ["keys", "mid", "sd"], ["piv"])
    t.op("DIST INT", ["piv", "sd"], ["pv"])
    if fused:
        t.op("FUSED 1", ["keys", "pv"], ["lti"])             # B_TO_I (keys < pv)
        t.op("FUSED 2", ["keys", "pv"], ["eqi"])             # B_TO_I (keys = pv)
        t.op("FUSED 3", ["keys", "pv"], ["gti"])             # B_TO_I (keys > pv)
    else:
        t.op("< INT", ["keys", "pv"], ["lt"])
        t.op("= INT", ["keys", "pv"], ["eq"])
        t.op("> INT", ["keys", "pv"], ["gt"])
        t.op("B_TO_I", ["lt"], ["lti"])
        t.op("B_TO_I", ["eq"], ["eqi"])
        t.op("B_TO_I", ["gt"], ["gti"])
    t.op("+_REDUCE INT", ["lti", "sd"], ["clt"])
    t.op("+_REDUCE INT", ["eqi", "sd"], ["ceq"])
    t.op("+_REDUCE INT", ["gti", "sd"], ["cgt"])
    t.op("+_SCAN INT", ["lti", "sd"], ["plt"])
    t.op("+_SCAN INT", ["eqi", "sd"], ["peq0"])
    t.op("+_SCAN INT", ["gti", "sd"], ["pgt0"])
    t.op("DIST INT", ["clt", "sd"], ["dlt"])
    t.op("+ INT", ["clt", "ceq"], ["clteq"])
    t.op("DIST INT", ["clteq", "sd"], ["dlteq"])
    if fused:  # the whole position computation in one pass
        t.op("FUSED 4", ["lti", "eqi", "plt", "peq0", "dlt", "pgt0", "dlteq"], ["pos"])
    else:
        t.op("+ INT", ["peq0", "dlt"], ["peq"])
        t.op("+ INT", ["pgt0", "dlteq"], ["pgt"])
        t.op("SELECT INT", ["eq", "peq", "pgt"], ["pos1"])
        t.op("SELECT INT", ["lt", "plt", "pos1"], ["pos"])
    t.op("PERMUTE INT", ["keys", "pos", "sd"], ["keys2"])
    # next lengths: (lesser, equal, greater) of every segment, interleaved
    t.const("INT 3", "three")
    t.const("INT 1", "one")
    t.op("* INT", ["m", "three"], ["m3"])
    t.op("MAKE_SEGDES", ["m3"], ["one_3m"])
    t.op("INDEX", ["zero", "three", "one_m"], ["i0"])
    t.op("DIST INT", ["one", "one_m"], ["ones"])
    t.op("+ INT", ["i0", "ones"], ["i1"])
    t.op("+ INT", ["i1", "ones"], ["i2"])
    t.op("DIST INT", ["zero", "one_3m"], ["z3"])
    t.op("DPERMUTE INT", ["clt", "i0", "z3", "one_m", "one_3m"], ["l1"])
    t.op("DPERMUTE INT", ["ceq", "i1", "l1", "one_m", "one_3m"], ["l2"])
    t.op("DPERMUTE INT", ["cgt", "i2", "l2", "one_m", "one_3m"], ["l3"])
    if fused:
        t.op("FUSED 5", ["l3", "one_3m"], ["nonempty"])    # l3 > 0
    else:
        t.op("DIST INT", ["zero", "one_3m"], ["zz"])
        t.op("> INT", ["l3", "zz"], ["nonempty"])
    t.op("PACK INT", ["l3", "nonempty", "one_3m"], ["l4", "l4sd"])
    t.op("MAKE_SEGDES", ["l4"], ["sd2"])
    t.call("QS_LOOP", ["keys2", "sd2"], ["out"])

    e = Block()
    e.alias("keys", "out")  # every segment is settled: the keys as they are
    f.if_return("more", t, e)
    return f.emit()


def qsort_program(fused: bool = False) -> str:
    """FUNC QSORT: (sd, keys) -> (sd, sorted keys), sd one segment."""
    main = Func("QSORT", params=["sd", "keys"], results=["sd", "out"])
    main.call("QS_LOOP", ["keys", "sd"], ["out"])
    return "{ quicksort of an int sequence; generated by neslgpu_gb300/vcode_programs.py }\n" + \
        main.emit() + "\n" + _qs_loop(fused)


# the super-ops of qsort_fcode_program, in the fusion compiler's notation
QSORT_FUSED_DEFS = """
fused OP0#1 ($0 : INT, $1 : SEGDES) = (/ INT @ $0 (DIST INT @ (CONST INT 2) $1))
fused OP1#1 ($0 : INT, $1 : INT) = (B_TO_I @ (< INT @ $0 $1))
fused OP2#1 ($0 : INT, $1 : INT) = (B_TO_I @ (= INT @ $0 $1))
fused OP3#1 ($0 : INT, $1 : INT) = (B_TO_I @ (> INT @ $0 $1))
fused OP4#1 ($0 : INT, $1 : INT, $2 : INT, $3 : INT, $4 : INT, $5 : INT, $6 : INT) =
  (SELECT INT @ (I_TO_B @ $0) $2 (SELECT INT @ (I_TO_B @ $1) (+ INT @ $3 $4) (+ INT @ $5 $6)))
fused OP5#1 ($0 : INT, $1 : SEGDES) = (> INT @ $0 (DIST INT @ (CONST INT 0) $1))
"""


def qsort_fcode_program() -> tuple[str, str]:
    """(the .fcode program, its super-op definitions)."""
    return qsort_program(fused=True), QSORT_FUSED_DEFS


def spmv_program() -> str:
    """FUNC SPMV: (rows sd, cols, vals, x) -> y, rows sd segmenting cols/vals."""
    f = Func("SPMV", params=["rsd", "cols", "vals", "x"], results=["y"])
    f.op("LENGTH INT", ["cols"], ["nnz"])
    f.op("MAKE_SEGDES", ["nnz"], ["one_nnz"])
    f.op("LENGTH FLOAT", ["x"], ["nx"])
    f.op("MAKE_SEGDES", ["nx"], ["one_x"])
    f.op("BPERMUTE FLOAT", ["x", "cols", "one_x", "one_nnz"], ["xg"])
    f.op("* FLOAT", ["xg", "vals"], ["prod"])
    f.op("+_REDUCE FLOAT", ["prod", "rsd"], ["y"])
    return "{ sparse matrix-vector product, CSR rows as a nested sequence; generated by " \
           "neslgpu_gb300/vcode_programs.py }\n" + f.emit()
