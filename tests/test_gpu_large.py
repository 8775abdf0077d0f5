"""Sizes past the point where rank and permute switch from a direct random
scatter to the partitioned one (index/value pairs grouped into 256 windows
of the output, then scattered window by window): results must stay
bit-identical to the oracle there too.  Also the destination-longer-than-
source case of the default permute, whose windows follow the destination."""
import numpy as np
import pytest

from cases import compare
from neslgpu_gb300 import ops
from neslgpu_gb300 import workloads as W

pytestmark = pytest.mark.gpu

N = (1 << 23) + 4099  # just past the switch for 4-byte values


@pytest.fixture(scope="module")
def data():
    r = W.rng(4242)
    xi = r.integers(-(2 ** 31), 2 ** 31, size=N, dtype=np.int64).astype(np.int32)
    ties = r.integers(-50, 50, size=N).astype(np.int32)
    xd = W.float64_normal(r, N)
    lens = W.geometric_lengths(r, N, 64.0)
    perm = W.permutation(r, N)
    return dict(xi=xi, ties=ties, xd=xd, lens=lens, perm=perm, r=r)


@pytest.mark.parametrize("name,key", [("rku_luz", "xi"), ("rkd_luz", "ties"), ("rku_lud", "xd"),
                                      ("rkd_lud", "xd")])
def test_rank_unsegmented(gpu, oracle, data, name, key):
    compare("exact", ops.rank_u(gpu, name, data[key]), ops.rank_u(oracle, name, data[key]))


@pytest.mark.parametrize("name,key", [("rku_lez", "ties"), ("rkd_led", "xd")])
def test_rank_segmented(gpu, oracle, data, name, key):
    got = ops.rank_e(gpu, name, data[key], data["lens"])
    compare("exact", got, ops.rank_e(oracle, name, data[key], data["lens"]))


@pytest.mark.parametrize("t", ["z", "d", "b"])
def test_permute(gpu, oracle, data, t):
    x = {"z": data["xi"], "d": data["xd"], "b": (data["ties"] > 0).astype(np.int32)}[t]
    compare("exact", ops.smp_u(gpu, f"smp_pu{t}", x, data["perm"]),
            ops.smp_u(oracle, f"smp_pu{t}", x, data["perm"]))
    one = np.array([N], dtype=np.int32)
    compare("exact", ops.smp_e(gpu, f"smp_pe{t}", x, data["perm"], one),
            ops.smp_e(oracle, f"smp_pe{t}", x, data["perm"], one))


def test_default_permute_wider_destination(gpu, oracle, data):
    # N values into 2N + 5 places: windows span the destination, not the source
    nd = 2 * N + 5
    r = W.rng(99)
    idx = r.permutation(nd)[:N].astype(np.int32)
    dflt = np.full(nd, -7, dtype=np.int32)
    compare("exact", ops.dpe_u(gpu, "dpe_puz", data["xi"], idx, dflt),
            ops.dpe_u(oracle, "dpe_puz", data["xi"], idx, dflt))


@pytest.mark.parametrize("kind", ["lognormal", "few_long"])
def test_segmented_reductions_many_chunks(gpu, oracle, kind):
    """Reductions over more than 1024 tiles with segments that span tiles
    and chunks of tiles: the second pass's chunked look-back."""
    from cases import seg_abs_total
    r = W.rng(77)
    n = (1 << 22) + 77
    if kind == "lognormal":
        lens = W.lognormal_lengths(r, n, 5.0, 2.0, 1 << 20)
    else:
        lens = np.array([1 << 21, 5, (1 << 21) - 5, 77], dtype=np.int32)
    lens = W.with_empty(r, lens, 0.05)
    xd = W.float64_normal(r, n)
    xi = r.integers(-1000, 1000, size=n).astype(np.int32)
    fl = (r.random(n) < 0.5).astype(np.int32)
    got = ops.reduce_e(gpu, "add_red", xd, lens)
    compare("sum", got, ops.reduce_e(oracle, "add_red", xd, lens), seg_abs_total(xd, lens))
    for name, x in (("add_rez", xi), ("max_rez", xi), ("min_red", xd)):
        compare("exact", ops.reduce_e(gpu, name, x, lens), ops.reduce_e(oracle, name, x, lens))
    compare("exact", ops.pk1_e(gpu, fl, lens), ops.pk1_e(oracle, fl, lens))
