"""numpy-level calls of CVL primitives, written once over a *runner*.

A runner owns the memory the C functions see: ``DeviceRunner`` (this
module) places vectors on the GPU heap of libcvl_gb300.so; the oracle
package supplies a host runner with the same interface for the CPU
restatement.  Each helper follows the calling convention vinterp uses for
the primitive (nesl/vcode/main.c:510-668, 1732-1884): allocate the result,
ask ``F_scratch`` for scratch, call ``F``, read the result back.

Type letters: ``z`` int32, ``b`` cvl_bool (int32 0/1), ``d`` float64.
"""
from __future__ import annotations

import numpy as np

from .cvl import CVL, DeviceVector, check, load


def np_dtype(kind: str):
    return np.float64 if kind == "d" else np.int32


class DeviceRunner:
    """Vectors live on the GPU heap; every call goes through the C ABI."""

    def __init__(self, cvl: CVL | None = None, checked: bool = True, offset: int = 0):
        """offset: allocate every vector that many 8-byte units into its
        allocation (exercises the kernels' unaligned paths)."""
        self.cvl = cvl or load()
        self.checked = checked
        self.offset = offset

    def fn(self, name):
        return getattr(self.cvl, name)

    def vec(self, arr, kind):
        arr = np.ascontiguousarray(arr, dtype=np_dtype(kind))
        if arr.size == 0:
            return DeviceVector(self.cvl, 1, kind, offset=self.offset)
        return DeviceVector.from_numpy(self.cvl, arr, kind, offset=self.offset)

    def out(self, n, kind):
        return DeviceVector(self.cvl, max(int(n), 1), kind, offset=self.offset)

    def units(self, u):
        return DeviceVector(self.cvl, 0, "u", units=max(int(u), 1), offset=self.offset)

    def p(self, h):
        return None if h is None else h.ptr

    def get(self, h, n):
        if n == 0:
            return np.empty(0, dtype=np.float64 if h.kind == "d" else np.int32)
        return h.numpy(n)

    def segd(self, lengths):
        lengths = np.ascontiguousarray(lengths, dtype=np.int32)
        m = int(lengths.size)
        n = int(lengths.sum(dtype=np.int64))
        lv = self.vec(lengths, "z")
        sd = self.units(self.cvl.siz_fos(n, m))
        scr = self.units(self.cvl.mke_fov_scratch(n, m))
        self.cvl.mke_fov(sd.ptr, lv.ptr, n, m, scr.ptr)
        return sd, n, m

    def done(self):
        if self.checked:
            check(self.cvl)


def _kind(name: str) -> str:
    return name[-1] if name[-1] in "zbd" else "z"


# --------------------------------------------------------- elementwise ---
_BOOL_OUT = {"grt", "les", "geq", "leq", "eql", "neq"}
_INT_OUT_FROM_D = {"int", "flr", "cei", "trn", "rou"}


def out_kind(name: str) -> str:
    op, k = name[:3], _kind(name)
    if op in _BOOL_OUT:
        return "b"
    if op in _INT_OUT_FROM_D or (op == "int" and k == "b"):
        return "z"
    if op == "dbl":
        return "d"
    if op == "boo":
        return "b"
    return k


def ew2(R, name, x, y):
    k = _kind(name)
    n = len(x)
    a, b = R.vec(x, k), R.vec(y, k)
    d = R.out(n, out_kind(name))
    R.fn(name)(R.p(d), R.p(a), R.p(b), n, None)
    r = R.get(d, n)
    R.done()
    return r


def ew1(R, name, x):
    k = _kind(name)
    if name[:3] == "dbl":
        k = "z"
    n = len(x)
    a = R.vec(x, k)
    d = R.out(n, out_kind(name))
    R.fn(name)(R.p(d), R.p(a), n, None)
    r = R.get(d, n)
    R.done()
    return r


def sel(R, name, f, x, y):
    k = _kind(name)
    n = len(x)
    c, a, b = R.vec(f, "b"), R.vec(x, k), R.vec(y, k)
    d = R.out(n, k)
    R.fn(name)(R.p(d), R.p(c), R.p(a), R.p(b), n, None)
    r = R.get(d, n)
    R.done()
    return r


# --------------------------------------------------- scans / reductions ---
def scan_u(R, name, x):
    k = _kind(name)
    n = len(x)
    a = R.vec(x, k)
    d = R.out(n, k)
    scr = R.units(R.fn(name + "_scratch")(n))
    R.fn(name)(R.p(d), R.p(a), n, R.p(scr))
    r = R.get(d, n)
    R.done()
    return r


def scan_e(R, name, x, lengths):
    k = _kind(name)
    sd, n, m = R.segd(lengths)
    a = R.vec(x, k)
    d = R.out(n, k)
    scr = R.units(R.fn(name + "_scratch")(n, m))
    R.fn(name)(R.p(d), R.p(a), R.p(sd), n, m, R.p(scr))
    r = R.get(d, n)
    R.done()
    return r


def reduce_u(R, name, x):
    k = _kind(name)
    n = len(x)
    a = R.vec(x, k)
    scr = R.units(R.fn(name + "_scratch")(n))
    r = R.fn(name)(R.p(a), n, R.p(scr))
    R.done()
    return r


def reduce_e(R, name, x, lengths):
    k = _kind(name)
    sd, n, m = R.segd(lengths)
    a = R.vec(x, k)
    d = R.out(m, k)
    scr = R.units(R.fn(name + "_scratch")(n, m))
    R.fn(name)(R.p(d), R.p(a), R.p(sd), n, m, R.p(scr))
    r = R.get(d, m)
    R.done()
    return r


# ------------------------------------------------------------- vprims ---
def ext_u(R, name, x, i):
    k = _kind(name)
    a = R.vec(x, k)
    r = R.fn(name)(R.p(a), int(i), len(x), None)
    R.done()
    return r


def ext_e(R, name, x, idx, lengths):
    k = _kind(name)
    sd, n, m = R.segd(lengths)
    a, ix = R.vec(x, k), R.vec(idx, "z")
    d = R.out(m, k)
    R.fn(name)(R.p(d), R.p(a), R.p(ix), R.p(sd), n, m, None)
    r = R.get(d, m)
    R.done()
    return r


def rep_u(R, name, x, i, val):
    k = _kind(name)
    a = R.vec(x, k)
    R.fn(name)(R.p(a), int(i), val, len(x), None)
    r = R.get(a, len(x))
    R.done()
    return r


def rep_e(R, name, x, idx, vals, lengths):
    k = _kind(name)
    sd, n, m = R.segd(lengths)
    a, ix, v = R.vec(x, k), R.vec(idx, "z"), R.vec(vals, k)
    R.fn(name)(R.p(a), R.p(ix), R.p(v), R.p(sd), n, m, None)
    r = R.get(a, n)
    R.done()
    return r


def dis_u(R, name, val, n):
    k = _kind(name)
    d = R.out(n, k)
    R.fn(name)(R.p(d), val, int(n), None)
    r = R.get(d, n)
    R.done()
    return r


def dis_e(R, name, vals, lengths):
    k = _kind(name)
    sd, n, m = R.segd(lengths)
    v = R.vec(vals, k)
    d = R.out(n, k)
    R.fn(name)(R.p(d), R.p(v), R.p(sd), n, m, None)
    r = R.get(d, n)
    R.done()
    return r


def ind_u(R, init, stride, n):
    d = R.out(n, "z")
    R.fn("ind_luz")(R.p(d), int(init), int(stride), int(n), None)
    r = R.get(d, n)
    R.done()
    return r


def ind_e(R, init, stride, lengths):
    sd, n, m = R.segd(lengths)
    a, b = R.vec(init, "z"), R.vec(stride, "z")
    d = R.out(n, "z")
    R.fn("ind_lez")(R.p(d), R.p(a), R.p(b), R.p(sd), n, m, None)
    r = R.get(d, n)
    R.done()
    return r


# ------------------------------------------------------------ permutes ---
def smp_u(R, name, x, idx):
    k = _kind(name)
    n = len(x)
    a, ix = R.vec(x, k), R.vec(idx, "z")
    d = R.out(n, k)
    scr = R.units(R.fn(name + "_scratch")(n))
    R.fn(name)(R.p(d), R.p(a), R.p(ix), n, R.p(scr))
    r = R.get(d, n)
    R.done()
    return r


def smp_e(R, name, x, idx, lengths):
    k = _kind(name)
    sd, n, m = R.segd(lengths)
    a, ix = R.vec(x, k), R.vec(idx, "z")
    d = R.out(n, k)
    scr = R.units(R.fn(name + "_scratch")(n, m))
    R.fn(name)(R.p(d), R.p(a), R.p(ix), R.p(sd), n, m, R.p(scr))
    r = R.get(d, n)
    R.done()
    return r


def bck_u(R, name, x, idx):
    k = _kind(name)
    a, ix = R.vec(x, k), R.vec(idx, "z")
    nd = len(idx)
    d = R.out(nd, k)
    R.fn(name)(R.p(d), R.p(a), R.p(ix), len(x), nd, None)
    r = R.get(d, nd)
    R.done()
    return r


def bck_e(R, name, x, idx, len_s, len_d):
    k = _kind(name)
    sds, ns, ms = R.segd(len_s)
    sdd, nd, md = R.segd(len_d)
    a, ix = R.vec(x, k), R.vec(idx, "z")
    d = R.out(nd, k)
    R.fn(name)(R.p(d), R.p(a), R.p(ix), R.p(sds), ns, ms, R.p(sdd), nd, md, None)
    r = R.get(d, nd)
    R.done()
    return r


def fpm_u(R, name, x, idx, flags, nd, init=None):
    """fpm_pu*/bfp_pu* (init=None) or dfp_pu* (init = default vector)."""
    k = _kind(name)
    a, ix, f = R.vec(x, k), R.vec(idx, "z"), R.vec(flags, "b")
    op = name[:3]
    if op == "bfp":
        d = R.out(len(idx), k)
        R.fn(name)(R.p(d), R.p(a), R.p(ix), R.p(f), len(x), len(idx), None)
        r = R.get(d, len(idx))
    elif op == "dfp":
        d = R.vec(init, k)
        v = R.vec(init, k)
        R.fn(name)(R.p(d), R.p(a), R.p(ix), R.p(f), R.p(v), len(x), nd, None)
        r = R.get(d, nd)
    else:
        d = R.vec(init if init is not None else np.zeros(nd), k)
        R.fn(name)(R.p(d), R.p(a), R.p(ix), R.p(f), len(x), nd, None)
        r = R.get(d, nd)
    R.done()
    return r


def fpm_e(R, name, x, idx, flags, len_s, len_d, init=None):
    k = _kind(name)
    sds, ns, ms = R.segd(len_s)
    sdd, nd, md = R.segd(len_d)
    op = name[:3]
    a, ix, f = R.vec(x, k), R.vec(idx, "z"), R.vec(flags, "b")
    if op == "bfp":
        d = R.out(nd, k)
        R.fn(name)(R.p(d), R.p(a), R.p(ix), R.p(f), R.p(sds), ns, ms, R.p(sdd), nd, md, None)
    elif op == "dfp":
        d = R.vec(init, k)
        v = R.vec(init, k)
        R.fn(name)(R.p(d), R.p(a), R.p(ix), R.p(f), R.p(v), R.p(sds), ns, ms, R.p(sdd), nd, md, None)
    else:
        d = R.vec(init if init is not None else np.zeros(nd), k)
        R.fn(name)(R.p(d), R.p(a), R.p(ix), R.p(f), R.p(sds), ns, ms, R.p(sdd), nd, md, None)
    r = R.get(d, nd)
    R.done()
    return r


def dpe_u(R, name, x, idx, default):
    k = _kind(name)
    a, ix = R.vec(x, k), R.vec(idx, "z")
    d, v = R.vec(default, k), R.vec(default, k)
    scr = R.units(R.fn(name + "_scratch")(len(x), len(default)))
    R.fn(name)(R.p(d), R.p(a), R.p(ix), R.p(v), len(x), len(default), R.p(scr))
    r = R.get(d, len(default))
    R.done()
    return r


def dpe_e(R, name, x, idx, default, len_s, len_d):
    k = _kind(name)
    sds, ns, ms = R.segd(len_s)
    sdd, nd, md = R.segd(len_d)
    a, ix = R.vec(x, k), R.vec(idx, "z")
    d, v = R.vec(default, k), R.vec(default, k)
    scr = R.units(R.fn(name + "_scratch")(ns, ms, nd, md))
    R.fn(name)(R.p(d), R.p(a), R.p(ix), R.p(v), R.p(sds), ns, ms, R.p(sdd), nd, md, R.p(scr))
    r = R.get(d, nd)
    R.done()
    return r


# ---------------------------------------------------------------- pack ---
def pk1_u(R, flags):
    f = R.vec(flags, "b")
    scr = R.units(R.fn("pk1_luv_scratch")(len(flags)))
    r = R.fn("pk1_luv")(R.p(f), len(flags), R.p(scr))
    R.done()
    return r


def pack_u(R, name, x, flags):
    k = _kind(name)
    n = len(x)
    cnt = int(np.count_nonzero(flags))
    a, f = R.vec(x, k), R.vec(flags, "b")
    d = R.out(cnt, k)
    scr = R.units(R.fn(name + "_scratch")(n))
    R.fn(name)(R.p(d), R.p(a), R.p(f), n, cnt, R.p(scr))
    r = R.get(d, cnt)
    R.done()
    return r


def pack_e(R, name, x, flags, lengths):
    """The PACK vop sequence: pk1_lev, add_ruz, mke_fov, pk2_le*
    (nesl/vcode/main.c:577-641).  Returns (values, new lengths)."""
    k = _kind(name)
    sd, n, m = R.segd(lengths)
    a, f = R.vec(x, k), R.vec(flags, "b")
    lens = R.out(m, "z")
    scr = R.units(R.fn("pk1_lev_scratch")(n, m))
    R.fn("pk1_lev")(R.p(lens), R.p(f), R.p(sd), n, m, R.p(scr))
    new_len = R.get(lens, m)
    cnt = int(new_len.sum(dtype=np.int64))
    sd2, n2, m2 = R.segd(new_len)
    d = R.out(cnt, k)
    scr2 = R.units(R.fn(name + "_scratch")(n, m, n2, m2))
    R.fn(name)(R.p(d), R.p(a), R.p(f), R.p(sd), n, m, R.p(sd2), n2, m2, R.p(scr2))
    r = R.get(d, cnt)
    R.done()
    return r, new_len


def pk1_e(R, flags, lengths):
    sd, n, m = R.segd(lengths)
    f = R.vec(flags, "b")
    d = R.out(m, "z")
    scr = R.units(R.fn("pk1_lev_scratch")(n, m))
    R.fn("pk1_lev")(R.p(d), R.p(f), R.p(sd), n, m, R.p(scr))
    r = R.get(d, m)
    R.done()
    return r


# ---------------------------------------------------------------- rank ---
def rank_u(R, name, x):
    k = _kind(name)
    n = len(x)
    a = R.vec(x, k)
    d = R.out(n, "z")
    scr = R.units(R.fn(name + "_scratch")(n))
    R.fn(name)(R.p(d), R.p(a), n, R.p(scr))
    r = R.get(d, n)
    R.done()
    return r


def rank_e(R, name, x, lengths):
    k = _kind(name)
    sd, n, m = R.segd(lengths)
    a = R.vec(x, k)
    d = R.out(n, "z")
    scr = R.units(R.fn(name + "_scratch")(n, m))
    R.fn(name)(R.p(d), R.p(a), R.p(sd), n, m, R.p(scr))
    r = R.get(d, n)
    R.done()
    return r


def rand_u(R, bounds, seed=None):
    if seed is not None:
        R.fn("rnd_foz")(int(seed))
    n = len(bounds)
    a = R.vec(bounds, "z")
    d = R.out(n, "z")
    R.fn("rnd_wuz")(R.p(d), R.p(a), n, None)
    r = R.get(d, n)
    R.done()
    return r
