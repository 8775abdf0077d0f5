"""CPU oracle loader -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU
baseline leg import this module; the product library never does.

* ``load_oracle()``: the C restatement of the serial CVL
  (``oracle/cvl_oracle.c``, symbols ``ocvl_<name>``), built into
  ``oracle/_build/libcvl_oracle.so``.
* ``load_reference()``: the reference's own serial CVL compiled from its
  sources (``make -C oracle ref``) into ``oracle/_ref/libcvl_serial.so``,
  or None where it was not built (it cannot be: the reference tree is not
  mounted there).

``HostRunner`` lets the numpy-level helpers of ``neslgpu_gb300.ops`` drive
either library with host arrays, so a parity test runs the same helper on
the GPU library and on the oracle.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
ORACLE_SO = ROOT / "_build" / "libcvl_oracle.so"
REF_SO = ROOT / "_ref" / "libcvl_serial.so"

_cache: dict = {}


def _cvl_class():
    from neslgpu_gb300.cvl import CVL  # ABI table only; no product code runs
    return CVL


def build() -> Path:
    if not ORACLE_SO.exists() or ORACLE_SO.stat().st_mtime < (ROOT / "cvl_oracle.c").stat().st_mtime:
        subprocess.run(["make", "-s", "-C", str(ROOT)], check=True)
    return ORACLE_SO


def load_oracle():
    if "oracle" not in _cache:
        build()
        _cache["oracle"] = _cvl_class()(C.CDLL(str(ORACLE_SO), mode=C.RTLD_LOCAL), prefix="ocvl_",
                                        extensions=False)
        lib = _cache["oracle"].lib
        for nm, rt, at in (("ocvl_now", C.c_double, []),
                           ("ocvl_rnd_state", None, [C.c_void_p, C.c_void_p])):
            f = getattr(lib, nm)
            f.restype, f.argtypes = rt, at
    return _cache["oracle"]


def load_reference():
    if "ref" not in _cache:
        _cache["ref"] = (_cvl_class()(C.CDLL(str(REF_SO), mode=C.RTLD_LOCAL), prefix="",
                                      extensions=False) if REF_SO.exists() else None)
    return _cache["ref"]


def reference_root():
    """The reference tree's root for tests that read its files: the
    GCVL_REFERENCE environment variable, else the tree `make ref` built
    oracle/_ref from; None where neither exists."""
    import os
    env = os.environ.get("GCVL_REFERENCE")
    if env:
        return Path(env) if Path(env).is_dir() else None
    rec = ROOT / "_ref" / "REFERENCE"
    if rec.exists():
        p = Path(rec.read_text().strip())
        return p if p.is_dir() else None
    return None


def now() -> float:
    return load_oracle().lib.ocvl_now()


def _dt(kind):
    return np.float64 if kind == "d" else np.int32


class HostRunner:
    """Runner over host memory for a CPU implementation of the CVL ABI
    (serial segment descriptor: the m lengths)."""

    def __init__(self, cvl):
        self.cvl = cvl

    def fn(self, name):
        f = getattr(self.cvl, name, None)
        if f is None and name.endswith("_scratch"):
            return lambda *a: 0  # the restatement allocates its own temporaries
        if f is None:
            raise AttributeError(name)
        return f

    def vec(self, arr, kind):
        a = np.array(arr, dtype=_dt(kind), copy=True).ravel()
        return a if a.size else np.zeros(1, dtype=_dt(kind))

    def out(self, n, kind):
        return np.zeros(max(int(n), 1), dtype=_dt(kind))

    def units(self, u):
        return np.zeros(max(int(u), 1), dtype=np.float64)

    def p(self, h):
        return None if h is None else h.ctypes.data

    def get(self, h, n):
        return np.array(h[:n], copy=True)

    def segd(self, lengths):
        lengths = np.ascontiguousarray(lengths, dtype=np.int32)
        m = int(lengths.size)
        n = int(lengths.sum(dtype=np.int64))
        lv = self.vec(lengths, "z")
        sd = np.zeros(max(self.cvl.siz_fos(n, m), 1) * 2, dtype=np.int32)
        self.cvl.mke_fov(sd.ctypes.data, lv.ctypes.data, n, m, None)
        return sd, n, m

    def done(self):
        pass
