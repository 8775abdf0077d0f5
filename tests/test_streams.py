"""Library streams and overlapped transfers: a segmented float64 vector cut
at segment starts into pieces, each piece uploaded, scanned and reduced,
and downloaded on its own stage's stream (gcvl_stream_create,
gcvl_set_stream, gcvl_event_record, gcvl_stream_wait_event,
gcvl_h2d_async, gcvl_d2h_async into pinned host memory), two rounds back
to back.  The pieces' results must agree with the whole vector's and with
the oracle within the float64 sum tolerance (the tiles' boundaries move
with the cuts, so the fixed-point folds may round differently)."""
import ctypes as C

import numpy as np
import pytest

from cases import compare, seg_abs_prefix, seg_abs_total
from neslgpu_gb300 import ops
from neslgpu_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def test_pipelined_pieces_match_whole_vector(gpu, oracle):
    c = gpu.cvl
    r = W.rng(808)
    n = (1 << 21) + 333
    lens = W.lognormal_lengths(r, n, 5.0, 2.0, 1 << 18)
    x = W.float64_normal(r, n)
    m = len(lens)
    ends = np.cumsum(lens, dtype=np.int64)
    starts = ends - lens
    # four pieces, cut at segment starts
    cuts = sorted({0, *[int(np.searchsorted(starts, n * k // 4)) for k in (1, 2, 3)], m})
    hx = c.gcvl_host_alloc(8 * n)
    hs = c.gcvl_host_alloc(8 * n)
    hr = c.gcvl_host_alloc(8 * m)
    assert hx and hs and hr
    streams = [c.gcvl_stream_create() for _ in range(3)]
    assert all(streams)
    pieces = []
    try:
        C.memmove(hx, x.ctypes.data, 8 * n)
        for s0, s1 in zip(cuts[:-1], cuts[1:]):
            pl = np.ascontiguousarray(lens[s0:s1], dtype=np.int32)
            pn, pm, e0 = int(pl.sum()), s1 - s0, int(starts[s0])
            p = {"e0": e0, "s0": s0, "n": pn, "m": pm,
                 "x": gpu.out(pn, "d"), "y": gpu.out(pn, "d"), "r": gpu.out(pm, "d")}
            sd, _, _ = gpu.segd(pl)
            p["sd"] = sd
            p["scr"] = gpu.units(max(c.add_sed_scratch(pn, pm), c.add_red_scratch(pn, pm)))
            p["ev"] = [c.gcvl_event_create() for _ in range(3)]
            pieces.append(p)
        c.gcvl_sync()
        up, ker, down = streams
        c.gcvl_set_stream(ker)
        for p in pieces:
            for e in p["ev"]:
                c.gcvl_event_record(e)
        for _ in range(2):  # two rounds: buffers reused under the events' ordering
            for p in pieces:
                eu, ek, ed = p["ev"]
                c.gcvl_set_stream(up)
                c.gcvl_stream_wait_event(ek)
                c.gcvl_h2d_async(p["x"].ptr, hx + 8 * p["e0"], 8 * p["n"])
                c.gcvl_event_record(eu)
                c.gcvl_set_stream(ker)
                c.gcvl_stream_wait_event(eu)
                c.gcvl_stream_wait_event(ed)
                c.add_sed(p["y"].ptr, p["x"].ptr, p["sd"].ptr, p["n"], p["m"], p["scr"].ptr)
                c.add_red(p["r"].ptr, p["x"].ptr, p["sd"].ptr, p["n"], p["m"], p["scr"].ptr)
                c.gcvl_event_record(ek)
                c.gcvl_set_stream(down)
                c.gcvl_stream_wait_event(ek)
                c.gcvl_d2h_async(hs + 8 * p["e0"], p["y"].ptr, 8 * p["n"])
                c.gcvl_d2h_async(hr + 8 * p["s0"], p["r"].ptr, 8 * p["m"])
                c.gcvl_event_record(ed)
        for q in streams:
            c.gcvl_set_stream(q)
            assert c.gcvl_sync() == 0
        c.gcvl_set_stream(None)
        got_scan = np.ctypeslib.as_array(C.cast(hs, C.POINTER(C.c_double)), shape=(n,)).copy()
        got_red = np.ctypeslib.as_array(C.cast(hr, C.POINTER(C.c_double)), shape=(m,)).copy()
    finally:
        c.gcvl_set_stream(None)
        for p in pieces:
            for e in p["ev"]:
                c.gcvl_event_destroy(e)
        for q in streams:
            c.gcvl_stream_destroy(q)
        c.gcvl_host_free(hx)
        c.gcvl_host_free(hs)
        c.gcvl_host_free(hr)
    whole_scan = ops.scan_e(gpu, "add_sed", x, lens)
    whole_red = ops.reduce_e(gpu, "add_red", x, lens)
    compare("sum", got_scan, whole_scan, seg_abs_prefix(x, lens))
    compare("sum", got_red, whole_red, seg_abs_total(x, lens))
    compare("sum", got_scan, ops.scan_e(oracle, "add_sed", x, lens), seg_abs_prefix(x, lens))
    compare("sum", got_red, ops.reduce_e(oracle, "add_red", x, lens), seg_abs_total(x, lens))
