"""Sizes past the point where rank, permute and gather switch from direct
random accesses to partitioned ones (index/value pairs grouped by window of
the output or the source, then scattered or gathered window by window):
results must stay bit-identical to the oracle there too.  Also the
destination-longer-than-source case of the default permute, whose windows
follow the destination, and the segmented reductions' tile, ring and
per-warp-range forms."""
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


def test_default_permute_ascending_indices(gpu, oracle, data):
    """Ascending indices (the interleave of a flattened three-way split):
    the partitioned scatter's device-side check sends them to one streaming
    scatter instead of the window partition."""
    nd = 3 * N
    idx = (3 * np.arange(N, dtype=np.int64) + 1).astype(np.int32)
    dflt = np.full(nd, -3, dtype=np.int32)
    compare("exact", ops.dpe_u(gpu, "dpe_puz", data["xi"], idx, dflt),
            ops.dpe_u(oracle, "dpe_puz", data["xi"], idx, dflt))
    ident = np.arange(N, dtype=np.int32)
    compare("exact", ops.smp_u(gpu, "smp_pud", data["xd"], ident), ops.smp_u(oracle, "smp_pud", data["xd"], ident))
    # one descent breaks the order: the partitioned path again
    idx2 = ident.copy()
    idx2[N // 2], idx2[N // 2 + 1] = idx2[N // 2 + 1], idx2[N // 2]
    compare("exact", ops.smp_u(gpu, "smp_puz", data["xi"], idx2), ops.smp_u(oracle, "smp_puz", data["xi"], idx2))


@pytest.mark.parametrize("t", ["z", "d"])
def test_pack_two_pass(gpu, oracle, data, t):
    """Packs long enough for the two-pass form (flag mask and tile counts,
    then placement at scanned tile offsets), unsegmented and segmented,
    sparse and dense flags."""
    x = data["xi"] if t == "z" else data["xd"]
    r = W.rng(17)
    for p in (0.5, 0.01, 0.999):
        fl = (r.random(N) < p).astype(np.int32)
        compare("exact", ops.pack_u(gpu, f"pk2_lu{t}", x, fl), ops.pack_u(oracle, f"pk2_lu{t}", x, fl))
    fl = (r.random(N) < 0.3).astype(np.int32)
    g, gl = ops.pack_e(gpu, f"pk2_le{t}", x, fl, data["lens"])
    o, ol = ops.pack_e(oracle, f"pk2_le{t}", x, fl, data["lens"])
    compare("exact", gl, ol)
    compare("exact", g, o)


@pytest.mark.parametrize("t", ["z", "d"])
def test_segmented_permute_many_segments(gpu, oracle, data, t):
    """PERMUTE within every segment (the coalesced segmented scatter), short
    and empty segments included."""
    x = data["xi"] if t == "z" else data["xd"]
    r = W.rng(23)
    lens = W.with_empty(r, W.geometric_lengths(r, N, 3.0), 0.1)
    # a random permutation of every segment: rank of a random key within the segment
    seg = np.repeat(np.arange(len(lens)), lens)
    start = np.concatenate([[0], np.cumsum(lens, dtype=np.int64)[:-1]])
    order = np.lexsort((r.random(N), seg))
    idx = np.empty(N, dtype=np.int32)
    idx[order] = (np.arange(N) - start[seg[order]]).astype(np.int32)
    compare("exact", ops.smp_e(gpu, f"smp_pe{t}", x, idx, lens), ops.smp_e(oracle, f"smp_pe{t}", x, idx, lens))


@pytest.mark.parametrize("mean", [1.0, 1.7, 2.5, 3.5])
def test_reductions_tiny_segments(gpu, oracle, mean):
    """Segmented reductions whose tiles hold as many segments as elements
    (the shared-memory offsets window) or more (empty segments: global
    offsets)."""
    from cases import seg_abs_total
    r = W.rng(int(mean * 10))
    n = (1 << 21) + 3
    lens = W.with_empty(r, W.geometric_lengths(r, n, mean), 0.2)
    xi = r.integers(-1000, 1000, size=n).astype(np.int32)
    xd = W.float64_normal(r, n)
    for name, x in (("min_rez", xi), ("max_rez", xi), ("add_rez", xi), ("max_red", xd)):
        compare("exact", ops.reduce_e(gpu, name, x, lens), ops.reduce_e(oracle, name, x, lens))
    compare("sum", ops.reduce_e(gpu, "add_red", xd, lens), ops.reduce_e(oracle, "add_red", xd, lens),
            seg_abs_total(xd, lens))


@pytest.mark.parametrize("n", [64 * 4096 - 1, 64 * 4096, 64 * 4096 + 1, 1 << 22])
def test_pack_two_pass_edges(gpu, oracle, n):
    """Around the size where pack switches to two passes (64 tiles of 4096),
    with all-false, all-true and alternating flags."""
    r = W.rng(n % 1000)
    x = r.integers(-2 ** 31, 2 ** 31, size=n, dtype=np.int64).astype(np.int32)
    for fl in (np.zeros(n, np.int32), np.ones(n, np.int32), (np.arange(n) % 2).astype(np.int32)):
        compare("exact", ops.pack_u(gpu, "pk2_luz", x, fl), ops.pack_u(oracle, "pk2_luz", x, fl))


# The gather from a source larger than 64 MB takes the partitioned path
# (indices split by source window, each window gathered while it sits in
# L2, results put back in destination order); ascending indices take one
# plain gather, decided on the device.
NG = (1 << 24) + 77  # int32 source of 64 MB + 308 bytes


@pytest.mark.parametrize("t,n_src,n_dst,kind", [
    ("z", NG, NG, "perm"), ("d", (1 << 23) + 5, (1 << 23) + 5, "perm"), ("b", NG, NG, "dups"),
    ("z", NG, NG, "ascending"), ("z", 1 << 25, (1 << 21) + 3, "dups"), ("d", 1 << 24, 3 << 22, "dups"),
    ("z", NG, 1 << 20, "perm"), ("z", NG, NG, "window-edges"),
])
def test_gather_partitioned(gpu, oracle, t, n_src, n_dst, kind):
    r = W.rng(n_src + n_dst)
    if t == "d":
        x = W.float64_normal(r, n_src)
    elif t == "b":
        x = r.integers(0, 2, size=n_src).astype(np.int32)
    else:
        x = r.integers(-(2 ** 31), 2 ** 31, size=n_src, dtype=np.int64).astype(np.int32)
    if kind == "perm":
        idx = r.permutation(n_src)[:n_dst].astype(np.int32)
    elif kind == "ascending":
        idx = np.sort(r.integers(0, n_src, size=n_dst)).astype(np.int32)
    elif kind == "window-edges":  # the first and last element of every source window, and 0 and n-1
        w = 1 << max(0, int(n_src - 1).bit_length() - 8)
        edges = np.concatenate([np.arange(0, n_src, w), np.minimum(np.arange(w - 1, n_src + w, w), n_src - 1)])
        idx = edges[r.integers(0, len(edges), size=n_dst)].astype(np.int32)
    else:
        idx = r.integers(0, n_src, size=n_dst).astype(np.int32)
    got = ops.bck_u(gpu, f"bck_pu{t}", x, idx)
    compare("exact", got, ops.bck_u(oracle, f"bck_pu{t}", x, idx))
    # the same gather as a segmented one with one source segment
    if n_src == n_dst:
        one = np.array([n_src], dtype=np.int32)
        compare("exact", ops.bck_e(gpu, f"bck_pe{t}", x, idx, one, one), got)


def test_gather_partitioned_with_caller_scratch(gpu, oracle):
    """As vinterp calls it: scratch sized by bck_puz_scratch, from the heap."""
    c = gpu.cvl
    r = W.rng(5)
    x = r.integers(-(2 ** 31), 2 ** 31, size=NG, dtype=np.int64).astype(np.int32)
    idx = r.permutation(NG).astype(np.int32)
    units = c.bck_puz_scratch(NG, NG)
    assert units > 0  # the partitioned path needs scratch
    a, ix, d, scr = gpu.vec(x, "z"), gpu.vec(idx, "z"), gpu.out(NG, "z"), gpu.units(units)
    c.bck_puz(d.ptr, a.ptr, ix.ptr, NG, NG, scr.ptr)
    got = gpu.get(d, NG)
    gpu.done()
    compare("exact", got, ops.bck_u(oracle, "bck_puz", x, idx))


# Scatters with a default or flags and repeated destinations: the serial CVL
# writes element by element, so the last element aimed at a place wins
# (nesl/cvl/serial/vecops.c); NESL's remove_duplicates, union and
# intersection rely on that, and the reference's test suite checks it.
@pytest.mark.parametrize("n,nd", [(1000, 700), (300_001, 100_003), ((1 << 23) + 4099, (1 << 23) + 4099)])
@pytest.mark.parametrize("t", ["z", "d"])
def test_default_permute_last_writer_wins(gpu, oracle, n, nd, t):
    r = W.rng(n + nd)
    x = W.float64_normal(r, n) if t == "d" else r.integers(-1000, 1000, size=n).astype(np.int32)
    idx = r.integers(0, nd, size=n).astype(np.int32)  # many repeats
    dflt = (np.full(nd, -7.5) if t == "d" else np.full(nd, -7, dtype=np.int32))
    compare("exact", ops.dpe_u(gpu, f"dpe_pu{t}", x, idx, dflt), ops.dpe_u(oracle, f"dpe_pu{t}", x, idx, dflt))
    flags = (r.random(n) < 0.6).astype(np.int32)
    compare("exact", ops.fpm_u(gpu, f"fpm_pu{t}", x, idx, flags, nd), ops.fpm_u(oracle, f"fpm_pu{t}", x, idx, flags, nd))


def test_segmented_default_permute_last_writer_wins(gpu, oracle):
    r = W.rng(31)
    lens = W.geometric_lengths(r, 400_000, 50.0)
    n = int(lens.sum())
    x = r.integers(-1000, 1000, size=n).astype(np.int32)
    idx = (r.random(n) * np.repeat(lens, lens)).astype(np.int32)  # local indices, repeats within segments
    dflt = np.full(n, -9, dtype=np.int32)
    compare("exact", ops.dpe_e(gpu, "dpe_pez", x, idx, dflt, lens, lens),
            ops.dpe_e(oracle, "dpe_pez", x, idx, dflt, lens, lens))
    flags = (r.random(n) < 0.5).astype(np.int32)
    compare("exact", ops.fpm_e(gpu, "fpm_pez", x, idx, flags, lens, lens),
            ops.fpm_e(oracle, "fpm_pez", x, idx, flags, lens, lens))


@pytest.mark.parametrize("kind", ["perm", "dups"])
def test_partitioned_paths_unaligned_indices(gpu, oracle, kind):
    """Index vectors 8 bytes off a 16-byte boundary: the window histogram
    reads them one key at a time instead of four (gather and scatter)."""
    from neslgpu_gb300.cvl import load
    from neslgpu_gb300.ops import DeviceRunner
    R = DeviceRunner(load(), offset=1)
    c = R.cvl
    r = W.rng(808)
    x = r.integers(-(2 ** 31), 2 ** 31, size=NG, dtype=np.int64).astype(np.int32)
    idx = (r.permutation(NG) if kind == "perm" else r.integers(0, NG, size=NG)).astype(np.int32)
    a, ix, d = R.vec(x, "z"), R.vec(idx, "z"), R.out(NG, "z")
    c.bck_puz(d.ptr, a.ptr, ix.ptr, NG, NG, None)
    compare("exact", R.get(d, NG), ops.bck_u(oracle, "bck_puz", x, idx))
    if kind == "perm":
        c.smp_puz(d.ptr, a.ptr, ix.ptr, NG, None)
        compare("exact", R.get(d, NG), ops.smp_u(oracle, "smp_puz", x, idx))
    R.done()


@pytest.mark.parametrize("n", [5000, (1 << 23) + 4099])
def test_default_permute_ascending_with_repeats(gpu, oracle, n):
    """Sorted destinations with repeats are not strictly ascending: the
    last-writer pass must still run (a strictly ascending index vector
    skips it), unsegmented and segmented."""
    r = W.rng(n + 1)
    x = r.integers(-1000, 1000, size=n).astype(np.int32)
    idx = np.sort(r.integers(0, n, size=n)).astype(np.int32)
    dflt = np.full(n, -7, dtype=np.int32)
    compare("exact", ops.dpe_u(gpu, "dpe_puz", x, idx, dflt), ops.dpe_u(oracle, "dpe_puz", x, idx, dflt))
    lens = W.geometric_lengths(r, n, 40.0)
    # local indices sorted within each segment, with repeats
    loc = np.concatenate([np.sort(r.integers(0, L, size=L)) for L in lens]).astype(np.int32)
    compare("exact", ops.dpe_e(gpu, "dpe_pez", x, loc, dflt, lens, lens),
            ops.dpe_e(oracle, "dpe_pez", x, loc, dflt, lens, lens))
    # strictly ascending within each segment: no repeats, the bitmap pass skipped
    strict = np.concatenate([np.arange(L) for L in lens]).astype(np.int32)
    compare("exact", ops.dpe_e(gpu, "dpe_pez", x, strict, dflt, lens, lens),
            ops.dpe_e(oracle, "dpe_pez", x, strict, dflt, lens, lens))


@pytest.mark.parametrize("shape", ["chunk-aligned", "empties", "ragged"])
def test_reductions_per_warp_ranges(gpu, oracle, shape):
    """4-byte segmented reductions with segments averaging 32 elements or
    more run along per-warp ranges of 1024-element chunks: segment ends on
    chunk boundaries, runs of empty segments longer than one 32-segment
    round (and leading and trailing ones), a length off every chunk and row
    boundary, every operator, against the oracle."""
    r = W.rng({"chunk-aligned": 1, "empties": 2, "ragged": 3}[shape])
    if shape == "chunk-aligned":
        lens = np.full(3000, 1024, dtype=np.int32)
        lens[::7] = 2048
    elif shape == "empties":
        base = W.geometric_lengths(r, 1_500_000, 300.0)
        lens = np.concatenate([np.zeros(5, np.int32), base[:100], np.zeros(40, np.int32), base[100:],
                               np.zeros(37, np.int32)]).astype(np.int32)
    else:
        lens = W.with_empty(r, W.geometric_lengths(r, 1024 * 777 + 29, 64.0), 0.1)
    n = int(lens.sum())
    xi = r.integers(-1000, 1000, size=n).astype(np.int32)
    xb = (r.random(n) < 0.7).astype(np.int32)
    for name in ("add_rez", "mul_rez", "min_rez", "max_rez", "and_rez", "ior_rez", "xor_rez"):
        compare("exact", ops.reduce_e(gpu, name, xi, lens), ops.reduce_e(oracle, name, xi, lens))
    for name in ("and_reb", "ior_reb", "xor_reb"):
        compare("exact", ops.reduce_e(gpu, name, xb, lens), ops.reduce_e(oracle, name, xb, lens))
    compare("exact", ops.pk1_e(gpu, xb, lens), ops.pk1_e(oracle, xb, lens))


@pytest.mark.parametrize("shape", ["geometric", "empties", "one", "ragged"])
@pytest.mark.parametrize("t", ["z", "b", "d"])
def test_distribute_per_warp_ranges(gpu, oracle, shape, t):
    """DIST (dis_ve*) at large sizes: runs of empty segments, a single
    huge segment, a ragged length, an output off a 16-byte boundary,
    against the oracle."""
    r = W.rng({"geometric": 11, "empties": 12, "one": 13, "ragged": 14}[shape])
    if shape == "geometric":
        lens = W.with_empty(r, W.geometric_lengths(r, 1 << 21, 64.0), 0.1)
    elif shape == "empties":
        base = W.geometric_lengths(r, 1 << 20, 200.0)
        lens = np.concatenate([np.zeros(3, np.int32), base[:50], np.zeros(70, np.int32), base[50:],
                               np.zeros(45, np.int32)]).astype(np.int32)
    elif shape == "one":
        lens = np.array([(1 << 20) + 3], dtype=np.int32)
    else:
        lens = W.geometric_lengths(r, 1024 * 333 + 7, 20.0)
    m = len(lens)
    vals = {"z": r.integers(-2 ** 31, 2 ** 31, size=m, dtype=np.int64).astype(np.int32),
            "b": (r.random(m) < 0.5).astype(np.int32), "d": W.float64_normal(r, m)}[t]
    want = ops.dis_e(oracle, f"dis_ve{t}", vals, lens)
    compare("exact", ops.dis_e(gpu, f"dis_ve{t}", vals, lens), want)
    if shape == "geometric":
        from neslgpu_gb300.cvl import load
        from neslgpu_gb300.ops import DeviceRunner
        compare("exact", ops.dis_e(DeviceRunner(load(), offset=1), f"dis_ve{t}", vals, lens), want)
