"""RAND: rnd_wuz draws (int)lrand48() % s[i] for i = 0, 1, ... in order
(nesl/cvl/serial/elwise.c:211-236), one draw per element, from the POSIX
48-bit generator X' = (0x5DEECE66D X + 0xB) mod 2^48 whose output is the
top 31 bits.  Unseeded, glibc's generator (the C library the serial CVL
calls on Linux) starts from state 0, and so do this library and the oracle.

Seeding differs between the serial CVL's build branches: on Linux its
rnd_foz calls srandom(seed) (nesl/cvl/serial/facilt.c:292-311), which does
not touch the lrand48 stream, so a seeded serial run keeps drawing the
unseeded stream; on HP-UX and SVR4 it calls srand48(seed).  This library
and the oracle follow the srand48 branch (rnd_foz reseeds the stream the
draws come from).  The CPU tests pin the oracle against the compiled serial
CVL on both: the unseeded stream, its continuation after the serial
rnd_foz, and the stream after libc's own srand48.  The GPU tests compare
the library's parallel jump-ahead stream with the oracle, seeded and
unseeded, over calls that continue one another."""
import json
import subprocess
import sys

import numpy as np
import pytest

from neslgpu_gb300 import ops, workloads as W

UNSEEDED = 0  # glibc's lrand48 state before any seeding


def _bounds(r, n):
    b = r.integers(1, 2 ** 31, size=n, dtype=np.int64)
    small = r.random(n) < 0.2
    b[small] = r.integers(1, 11, size=int(small.sum()))
    neg = r.random(n) < 0.1
    b[neg] = -r.integers(1, 2 ** 31, size=int(neg.sum()), dtype=np.int64)
    return b.astype(np.int32)


_SERIAL_SCRIPT = r"""
import ctypes as C, json, sys
import numpy as np
ref = C.CDLL(sys.argv[1])
libc = C.CDLL(None)
b = np.array(json.loads(sys.argv[2]), dtype=np.int32)
out = []
def draw():
    d = np.zeros(len(b), dtype=np.int32)
    ref.rnd_wuz(C.c_void_p(d.ctypes.data), C.c_void_p(b.ctypes.data), C.c_int(len(b)), None)
    out.append(d.tolist())
draw()                      # unseeded
ref.rnd_foz(C.c_int(1234))  # Linux branch: srandom, the lrand48 stream goes on
draw()
libc.srand48(C.c_long(1234))
draw()                      # what the srand48 branch of rnd_foz gives
print(json.dumps(out))
"""


def test_oracle_rand_matches_compiled_serial_cvl(reference, oracle):
    from oracle.oracle import REF_SO
    b = _bounds(W.rng(11), 4099)
    # a fresh process: the serial CVL draws from libc's process-wide state
    r = subprocess.run([sys.executable, "-c", _SERIAL_SCRIPT, str(REF_SO), json.dumps(b.tolist())],
                       capture_output=True, text=True, check=True)
    unseeded, continued, srand48_seeded = (np.array(v, dtype=np.int32) for v in json.loads(r.stdout))
    o = oracle.cvl
    st = np.array([UNSEEDED], dtype=np.uint64)
    o.lib.ocvl_rnd_state(None, st.ctypes.data)
    assert np.array_equal(ops.rand_u(oracle, b), unseeded)
    assert np.array_equal(ops.rand_u(oracle, b), continued)
    assert np.array_equal(ops.rand_u(oracle, b, seed=1234), srand48_seeded)
    # the Linux serial rnd_foz leaves the stream alone, the srand48 branch does not
    assert not np.array_equal(continued, srand48_seeded)


def _oracle_state(o):
    v = np.zeros(1, dtype=np.uint64)
    o.lib.ocvl_rnd_state(v.ctypes.data, None)
    return int(v[0])


@pytest.mark.gpu
@pytest.mark.parametrize("seed", [None, 0, 987654321, -5])
def test_gpu_rand_matches_oracle(gpu, oracle, seed):
    c, o = gpu.cvl, oracle.cvl
    if seed is None:
        c.gcvl_set_rand_state(UNSEEDED)
        st = np.array([UNSEEDED], dtype=np.uint64)
        o.lib.ocvl_rnd_state(None, st.ctypes.data)
    else:
        c.rnd_foz(seed)
        o.rnd_foz(seed)
    r = W.rng(12 if seed is None else abs(seed) % 1000 + 13)
    # consecutive calls continue one stream: sizes cross the grid-stride
    # boundary of the kernel and leave the state at odd positions
    for n in [1, 2, 7, 4097, 300_001, (1 << 22) + 3]:
        b = _bounds(r, n)
        got = ops.rand_u(gpu, b)
        want = ops.rand_u(oracle, b)
        if not np.array_equal(got, want):
            i = int(np.flatnonzero(got != want)[0])
            raise AssertionError(f"n={n}: first mismatch at {i}: {got[i]} != {want[i]}")
        assert c.gcvl_rand_state() == _oracle_state(o), f"state after n={n}"
