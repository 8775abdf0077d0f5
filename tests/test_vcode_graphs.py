"""Basic blocks of a VCODE program run as CUDA graphs (vcode.Interpreter
with graphs=True): a block of device instructions between host reads is
captured the first time it runs in a given interpreter state and replayed
(host bookkeeping redone without calls, then the graph launched) whenever it
runs in that state again.

On CPU the oracle stands in for the library behind a fake of the graph
calls with stream-capture semantics: calls made between gcvl_graph_begin and
gcvl_graph_end are recorded, not run; gcvl_graph_launch runs the recorded
calls.  A host read or a device allocation during a capture makes the fake
fail.  Results must equal the plain run's bit for bit.  On the GPU the same
programs run on the library with real graphs."""
import numpy as np
import pytest

from neslgpu_gb300 import vcode as V
from neslgpu_gb300 import vcode_programs as P

HOST_CALLS = {"alo_foz", "fre_fov", "add_ruz", "ext_vuz", "ext_vub", "ext_vud", "v2c_fuz", "v2c_fub", "v2c_fud",
              "c2v_fuz", "c2v_fub", "c2v_fud", "rep_vuz", "rep_vub", "rep_vud", "pk1_luv", "rnd_foz", "rnd_wuz"}


class FakeGraphs:
    """The oracle's CVL with gcvl_graph_* that defer calls, as capture does."""

    def __init__(self, cvl):
        self._c = cvl
        self._rec = None
        self.launched = 0

    def __getattr__(self, name):
        f = getattr(self._c, name)
        if name.endswith("_scratch") or name.startswith("siz_") or name in ("add_fov", "sub_fov", "cmp_fov"):
            return f

        def call(*a):
            if self._rec is not None:
                if name in HOST_CALLS:
                    raise AssertionError(f"{name} during a capture")
                self._rec.append((f, a))
                return None
            return f(*a)
        return call

    def gcvl_graph_begin(self):
        assert self._rec is None
        self._rec = []
        return 0

    def gcvl_graph_end(self):
        g, self._rec = self._rec, None
        return g

    def gcvl_graph_launch(self, g):
        self.launched += 1
        for f, a in g:
            f(*a)
        return 0

    def gcvl_graph_destroy(self, g):
        pass

    def gcvl_clear_error(self):
        pass

    def gcvl_error_string(self):
        return b""


def _sort(cvl, keys, graphs, it=None):
    it = it or V.Interpreter(P.qsort_program(), cvl, graphs=graphs)
    lv = it.from_host("I", [len(keys)])
    sd = it.segdes_from_lengths(lv)
    it.drop(lv)
    st = it.run("QSORT", [sd, it.from_host("I", keys)])
    out = it.to_host(st[-1])
    for v in st:
        it.drop(v)
    return out, it


def _spmv(it, lens, cols, vals, x):
    lv = it.from_host("I", lens)
    rsd = it.segdes_from_lengths(lv)
    it.drop(lv)
    st = it.run("SPMV", [rsd, it.from_host("I", cols), it.from_host("F", vals), it.from_host("F", x)])
    out = it.to_host(st[0])
    for v in st:
        it.drop(v)
    return out


def _csr(rows, ncols, seed):
    r = np.random.default_rng(seed)
    lens = np.minimum(r.zipf(2.1, size=rows), 64).astype(np.int32)
    nnz = int(lens.sum())
    return lens, r.integers(0, ncols, size=nnz).astype(np.int32), r.normal(size=nnz), r.normal(size=ncols)


def test_spmv_blocks_replay_on_oracle(oracle):
    fake = FakeGraphs(oracle.cvl)
    plain = V.Interpreter(P.spmv_program(), oracle.cvl)
    it = V.Interpreter(P.spmv_program(), fake, graphs=True)
    lens, cols, vals, x = _csr(500, 300, 1)
    want = _spmv(plain, lens, cols, vals, x)
    outs = [_spmv(it, lens, cols, vals, x) for _ in range(4)]
    for got in outs:
        assert np.array_equal(got.view(np.int64), want.view(np.int64))
    assert it.graph_stats["captured"] >= 1 and it.graph_stats["replayed"] >= 2, it.graph_stats
    assert fake.launched == it.graph_stats["captured"] + it.graph_stats["replayed"]
    # other sizes: new blocks are captured, the results still right
    lens2, cols2, vals2, x2 = _csr(300, 200, 2)
    got = _spmv(it, lens2, cols2, vals2, x2)
    assert np.array_equal(got.view(np.int64), _spmv(plain, lens2, cols2, vals2, x2).view(np.int64))
    it.free_all()
    plain.free_all()


@pytest.mark.parametrize("n", [0, 1, 7, 3000])
def test_quicksort_blocks_on_oracle(oracle, n):
    fake = FakeGraphs(oracle.cvl)
    keys = np.random.default_rng(n).integers(-1000, 1000, size=n).astype(np.int32)
    it = None
    for _ in range(4):  # the same sort again: once the heap has settled, its blocks replay
        got, it = _sort(fake, keys, True, it)
        assert np.array_equal(got, np.sort(keys))
    if n >= 3000:
        assert it.graph_stats["replayed"] > 0, it.graph_stats
        # settled: a further run replays every block and captures none
        before = dict(it.graph_stats)
        got, it = _sort(fake, keys, True, it)
        assert np.array_equal(got, np.sort(keys))
        assert it.graph_stats["captured"] == before["captured"], (before, it.graph_stats)
        assert it.graph_stats["replayed"] - before["replayed"] == it.graph_stats["blocks_run"] - before["blocks_run"]
    it.free_all()


@pytest.mark.gpu
def test_graph_blocks_on_gpu(gpu):
    c = gpu.cvl
    lens, cols, vals, x = _csr(20_000, 5_000, 4)
    plain = V.Interpreter(P.spmv_program(), c)
    want = _spmv(plain, lens, cols, vals, x)
    it = V.Interpreter(P.spmv_program(), c, graphs=True)
    for _ in range(4):
        got = _spmv(it, lens, cols, vals, x)
        assert np.array_equal(got.view(np.int64), want.view(np.int64))
    assert it.graph_stats["captured"] >= 1 and it.graph_stats["replayed"] >= 2, it.graph_stats
    it.free_all()
    plain.free_all()
    keys = np.random.default_rng(9).integers(-2 ** 31, 2 ** 31, size=100_003, dtype=np.int64).astype(np.int32)
    it = None
    for _ in range(4):
        got, it = _sort(c, keys, True, it)
        assert np.array_equal(got, np.sort(keys))
    assert it.graph_stats["replayed"] > 0, it.graph_stats
    it.free_all()
