"""Host-side logic that needs no GPU: the batched workloads' generators and
the build's tuning defines."""
import numpy as np

from neslgpu_gb300 import batch as B
from neslgpu_gb300 import build


def _consistent(b):
    assert b.nvec == len(b.vec_len) == len(b.nseg)
    assert int(b.nseg.sum()) == b.m == len(b.seg_lens)
    assert int(b.vec_len.sum()) == b.n == int(b.seg_lens.sum(dtype=np.int64))
    # each vector's inner segments sum to its length (segments never cross vectors)
    ends = np.cumsum(b.nseg)
    per_vec = np.add.reduceat(b.seg_lens.astype(np.int64), np.concatenate([[0], ends[:-1]]))
    np.testing.assert_array_equal(per_vec, b.vec_len)
    assert (b.seg_lens >= 1).all()


def test_skewed_batch_shape():
    b = B.make_skewed_batch(huge=3, huge_len=1 << 12, tiny=500, tiny_hi=100, seed=9)
    _consistent(b)
    assert b.nvec == 503
    assert int((b.vec_len == 1 << 12).sum()) == 3
    small = b.vec_len[b.vec_len != 1 << 12]
    assert small.min() >= 1 and small.max() <= 100
    # the huge vectors are spread among the tiny ones, not all at the front
    assert np.flatnonzero(b.vec_len == 1 << 12).max() > 3


def test_single_vector_batch_matches_total():
    b = B.single_vector_batch(12_345, seed=2)
    _consistent(b)
    assert b.nvec == 1 and b.n == 12_345


def test_make_batch_unchanged_by_refactor():
    b = B.make_batch(64, 1 << 16, seed=3)
    _consistent(b)
    assert b.nvec == 64 and abs(b.n - (1 << 16)) < (1 << 16) // 4


def test_tuning_defines_from_environment(monkeypatch):
    monkeypatch.setenv("GCVL_TUNE", "GCVL_RK_ITEMS=16  OTHER=1 GCVL_WR_NB=3")
    assert build.tuning_defines() == ["-DGCVL_RK_ITEMS=16", "-DGCVL_WR_NB=3"]
    monkeypatch.delenv("GCVL_TUNE")
    assert build.tuning_defines() == []
