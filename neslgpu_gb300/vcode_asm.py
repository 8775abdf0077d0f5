"""A small assembler for VCODE: write a function as named, single-assignment
vector operations; get the stack program (COPY / CPOP / POP to bring each
argument to the top and drop values after their last use).

Used to write this repository's own VCODE programs (quicksort and sparse
matrix-vector product, ``vcode_programs.py``) in the shape the NESL compiler
gives its output: sequences as (segment descriptor, data) pairs, nested
parallelism flattened into segmented operations, loops as recursion.

    f = Func("SUM", params=["v", "sd"], results=["s"])
    f.op("+_REDUCE INT", ["v", "sd"], ["s"])
    text = f.emit()
"""
from __future__ import annotations


class Func:
    def __init__(self, name: str, params: list[str], results: list[str]):
        self.name = name
        self.params = list(params)
        self.results = list(results)
        self.body: list[tuple] = []  # ("op", text, args, outs) | ("if", cond, then, else) | ("call", ...)

    # -- building
    def op(self, text: str, args: list[str], outs: list[str]):
        """A VCODE statement consuming `args` (deepest first) and pushing
        `outs` (in order)."""
        self.body.append(("op", text, list(args), list(outs)))
        return self

    def const(self, text: str, out: str):
        """CONST <text> -> out (e.g. "INT 3", "BOOL T")."""
        self.body.append(("op", "CONST " + text, [], [out]))
        return self

    def call(self, fname: str, args: list[str], outs: list[str]):
        self.body.append(("op", "CALL " + fname, list(args), list(outs)))
        return self

    def if_return(self, cond: str, then_block: "Block", else_block: "Block"):
        """The function's last statement: IF cond, each branch computing the
        function's results from the values live here."""
        self.body.append(("if", cond, then_block, else_block))
        return self

    # -- emission
    def emit(self) -> str:
        lines = [f"FUNC {self.name}"]
        stack = list(self.params)
        _emit_block(self.body, stack, self.results, lines)
        lines.append("RET")
        return "\n".join(lines) + "\n"


class Block:
    """A branch of if_return: statements, then the function's results."""

    def __init__(self):
        self.body: list[tuple] = []

    def op(self, text, args, outs):
        self.body.append(("op", text, list(args), list(outs)))
        return self

    def const(self, text, out):
        self.body.append(("op", "CONST " + text, [], [out]))
        return self

    def call(self, fname, args, outs):
        self.body.append(("op", "CALL " + fname, list(args), list(outs)))
        return self

    def alias(self, src, dst):
        """dst names the value of src (no VCODE is emitted when src dies here)."""
        self.body.append(("op", None, [src], [dst]))
        return self


def _uses_after(body, k, results):
    """Names read by statements after index k, plus the results."""
    used = set(results)
    for st in body[k + 1:]:
        if st[0] == "op":
            used.update(st[2])
        else:
            used.add(st[1])
            for blk in (st[2], st[3]):
                used.update(_reads(blk.body))
    return used


def _reads(body):
    r = set()
    for st in body:
        if st[0] == "op":
            r.update(st[2])
    return r


def _depth(stack, name):
    return len(stack) - 1 - max(i for i, v in enumerate(stack) if v == name)


def _emit_block(body, stack, results, lines, extra_live=frozenset()):
    for k, st in enumerate(body):
        if st[0] == "op":
            _, text, args, outs = st
            later = _uses_after(body, k, results) | extra_live
            if text is None:  # alias: rename, or copy when the source lives on
                a, o = args[0], outs[0]
                d = _depth(stack, a)
                if a in later:
                    lines.append(f"COPY 1 {d}")
                    stack.append(o)
                else:
                    stack[len(stack) - 1 - d] = o
                continue
            # bring the arguments to the top, in order; move a value whose
            # last use this is (and which is not needed again by this op)
            for j, a in enumerate(args):
                if a not in stack:
                    raise ValueError(f"{text}: {a} is not defined")
                d = _depth(stack, a)
                moving = a not in later and a not in args[j + 1:]
                if moving:
                    lines.append(f"CPOP 1 {d}")
                    stack.append(stack.pop(len(stack) - 1 - d))
                else:
                    lines.append(f"COPY 1 {d}")
                    stack.append(a)
            lines.append(text)
            del stack[len(stack) - len(args):]
            stack.extend(outs)
            # drop what nobody reads any more
            later = _uses_after(body, k, results) | extra_live
            _drop_dead(stack, later, lines)
        else:
            _, cond, then_blk, else_blk = st
            if cond not in stack:
                raise ValueError(f"IF: {cond} is not defined")
            d = _depth(stack, cond)
            live_after = _reads(then_blk.body) | _reads(else_blk.body) | set(results)
            if cond in live_after:
                lines.append(f"COPY 1 {d}")
                stack.append(cond)
            else:
                lines.append(f"CPOP 1 {d}")
                stack.append(stack.pop(len(stack) - 1 - d))
            lines.append("IF")
            stack.pop()
            _drop_dead(stack, live_after, lines)
            s1 = list(stack)
            _emit_block(then_blk.body, s1, results, lines)
            lines.append("ELSE")
            s2 = list(stack)
            _emit_block(else_blk.body, s2, results, lines)
            lines.append("ENDIF")
            stack[:] = list(results)
            return
    # arrange the results: move them to the top in order, then drop the rest
    for r in results:
        d = _depth(stack, r)
        lines.append(f"CPOP 1 {d}")
        stack.append(stack.pop(len(stack) - 1 - d))
    rest = len(stack) - len(results)
    if rest:
        lines.append(f"POP {rest} {len(results)}")
        del stack[:rest]


def _drop_dead(stack, live, lines):
    i = len(stack) - 1
    while i >= 0:
        v = stack[i]
        if v not in live:
            d = len(stack) - 1 - i
            lines.append(f"POP 1 {d}")
            del stack[i]
        i -= 1
