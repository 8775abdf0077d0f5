"""ctypes binding of libcvl_gb300.so, the GB300 CVL library.

``load()`` returns a :class:`CVL` whose attributes are the library's C
functions with the argument meaning of the reference's ``cvl.h`` (same
names, same order, vec_p = device pointer as an int).  ``DeviceVector``
wraps a heap allocation made with ``alo_foz`` and moves numpy data in and
out with ``c2v_fu*`` / ``v2c_fu*``.

The binding never falls back to anything: if the shared library is missing
or fails to load, ``load()`` raises.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

from . import abi

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libcvl_gb300.so"


class Timespec(C.Structure):
    _fields_ = [("tv_sec", C.c_long), ("tv_nsec", C.c_long)]


_CT = {
    "v": None, "i": C.c_int, "u": C.c_uint, "d": C.c_double, "b": C.c_int,
    "p": C.c_void_p, "I": C.c_void_p, "B": C.c_void_p, "D": C.c_void_p,
    "T": C.POINTER(Timespec), "c": C.c_char_p, "z": C.c_size_t, "P": C.c_void_p,
    "f": C.c_float, "q": C.c_ulonglong, "l": C.c_long,
}


def bind(lib: C.CDLL, name: str, sig: str, symbol: str | None = None):
    ret, args = sig.split(":")
    fn = getattr(lib, symbol or name)
    fn.restype = _CT[ret]
    fn.argtypes = [_CT[a] for a in args]
    return fn


class CVL:
    """The C functions of one CVL implementation, bound by name."""

    def __init__(self, lib: C.CDLL, prefix: str = "", extensions: bool = True, names=None):
        self.lib = lib
        self.prefix = prefix
        table = {k: v[0] for k, v in abi.CVL.items()}
        if extensions:
            table.update(abi.EXTENSIONS)
        for name, sig in table.items():
            if names is not None and name not in names:
                continue
            try:
                setattr(self, name, bind(lib, name, sig, prefix + name))
            except AttributeError:
                pass

    def has(self, name: str) -> bool:
        return hasattr(self, name)


_LOADED: CVL | None = None


def load(path: str | os.PathLike | None = None) -> CVL:
    """Load the CUDA library (once per process)."""
    global _LOADED
    if _LOADED is not None and path is None:
        return _LOADED
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(
            f"{p} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(str(p), mode=C.RTLD_LOCAL)
    cvl = CVL(lib)
    if path is None:
        _LOADED = cvl
    return cvl


class CVLError(RuntimeError):
    pass


def check(cvl: CVL, sync: bool = True) -> None:
    """Raise CVLError if the library recorded an error (optionally after
    synchronising the library stream)."""
    code = cvl.gcvl_sync() if sync else cvl.gcvl_last_error()
    if code:
        msg = cvl.gcvl_error_string().decode(errors="replace")
        cvl.gcvl_clear_error()
        raise CVLError(f"gcvl error {code}: {msg}")


_KIND = {np.dtype(np.int32): "z", np.dtype(np.float64): "d"}


class DeviceVector:
    """A vector on the device heap (alo_foz) with numpy transfer helpers.

    kind: 'z' int, 'b' cvl_bool, 'd' double, 'u' raw 8-byte units."""

    def __init__(self, cvl: CVL, length: int, kind: str = "z", units: int | None = None,
                 offset: int = 0):
        """offset: place the vector that many 8-byte units into its
        allocation (vinterp sub-allocates its heap in 8-byte units, so a
        vec_p need not be 16-byte aligned)."""
        self.cvl = cvl
        self.len = int(length)
        self.kind = kind
        if units is None:
            units = {"z": cvl.siz_foz, "b": cvl.siz_fob, "d": cvl.siz_fod}[kind](self.len) if kind != "u" else self.len
        self.units = max(int(units), 1)
        base = cvl.alo_foz(self.units + offset)
        if not base:
            raise CVLError(f"alo_foz({self.units}) failed: {cvl.gcvl_error_string().decode()}")
        self.base = base
        self.ptr = cvl.add_fov(base, offset) if offset else base

    @classmethod
    def from_numpy(cls, cvl: CVL, arr, kind: str | None = None, offset: int = 0) -> "DeviceVector":
        arr = np.ascontiguousarray(arr)
        if kind is None:
            kind = _KIND.get(arr.dtype)
            if kind is None:
                raise TypeError(f"no CVL type for {arr.dtype}")
        dt = np.float64 if kind == "d" else np.int32
        arr = np.ascontiguousarray(arr, dtype=dt)
        v = cls(cvl, arr.size, kind, offset=offset)
        v.upload(arr)
        return v

    def upload(self, arr) -> None:
        dt = np.float64 if self.kind == "d" else np.int32
        arr = np.ascontiguousarray(arr, dtype=dt)
        assert arr.size <= self.len
        fn = {"z": self.cvl.c2v_fuz, "b": self.cvl.c2v_fub, "d": self.cvl.c2v_fud}[self.kind]
        fn(self.ptr, arr.ctypes.data, arr.size, None)

    def numpy(self, length: int | None = None):
        n = self.len if length is None else int(length)
        dt = np.float64 if self.kind == "d" else np.int32
        out = np.empty(n, dtype=dt)
        fn = {"z": self.cvl.v2c_fuz, "b": self.cvl.v2c_fub, "d": self.cvl.v2c_fud}[self.kind]
        fn(out.ctypes.data, self.ptr, n, None)
        return out

    def free(self) -> None:
        if self.ptr:
            self.cvl.fre_fov(self.base)
            self.ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def segdes(cvl: CVL, lengths) -> tuple[DeviceVector, int, int]:
    """Build a device segment descriptor from host lengths: returns
    (descriptor, n, m) as vinterp's MAKE_SEGDES does (add_ruz + mke_fov)."""
    lengths = np.ascontiguousarray(lengths, dtype=np.int32)
    m = int(lengths.size)
    n = int(lengths.sum(dtype=np.int64))
    lv = DeviceVector.from_numpy(cvl, lengths, "z") if m else DeviceVector(cvl, 1, "z")
    sd = DeviceVector(cvl, 0, "u", units=cvl.siz_fos(n, m))
    scr = DeviceVector(cvl, 0, "u", units=max(cvl.mke_fov_scratch(n, m), 1))
    cvl.mke_fov(sd.ptr, lv.ptr, n, m, scr.ptr)
    lv.free()
    scr.free()
    return sd, n, m
