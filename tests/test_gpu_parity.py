"""libcvl_gb300.so against the oracle, primitive by primitive, through the
C ABI.  Integer, boolean and index results must be bit-identical; float64
sums agree within |a - b| <= 1e-12 * max(|b|, S) (S = sum of |x| over the
same prefix or segment), float64 products within 1e-12 relative, and CUDA
transcendentals within 1e-13 relative of libm."""
import numpy as np
import pytest

from cases import compare, make_cases

pytestmark = pytest.mark.gpu

SIZES = [0, 1, 7, 4097, 100_003]
KINDS = ["geo", "tiny", "empty", "bimodal", "one", "long"]


def _run_all(gpu, oracle, n, kind, seed):
    failures = []
    for cid, fn, cmp, ctx in make_cases(n=n, seed=seed, lengths_kind=kind):
        want = fn(oracle)
        try:
            got = fn(gpu)
            compare(cmp, got, want, ctx)
        except Exception as e:  # collect every mismatch of the sweep
            failures.append(f"{cid}: {e}")
    assert not failures, f"n={n} kind={kind}:\n" + "\n".join(failures[:40])


@pytest.mark.parametrize("n", SIZES)
def test_parity_sizes(gpu, oracle, n):
    _run_all(gpu, oracle, n, "geo", seed=100 + n)


@pytest.mark.parametrize("kind", KINDS)
def test_parity_segment_shapes(gpu, oracle, kind):
    _run_all(gpu, oracle, 60_001, kind, seed=5)


def test_parity_large(gpu, oracle):
    # several tiles per segment and several segments per tile at once
    _run_all(gpu, oracle, (1 << 20) + 13, "long", seed=9)


@pytest.mark.parametrize("kind", ["geo", "long", "empty"])
def test_parity_unaligned_vectors(oracle, kind):
    """Every vector 8 bytes past a 16-byte boundary, as vinterp's 8-byte
    sub-allocation can place it: the kernels' non-TMA paths."""
    from neslgpu_gb300.cvl import load
    from neslgpu_gb300.ops import DeviceRunner
    from conftest import _has_gpu
    if not _has_gpu():
        pytest.skip("no GPU")
    _run_all(DeviceRunner(load(), offset=1), oracle, 70_001, kind, seed=21)


@pytest.mark.parametrize("kind", ["long", "tiny"])
def test_parity_unaligned_two_million(oracle, kind):
    """The non-TMA paths past 2^21 elements: segmented reductions there
    complete the results that span tiles in a second pass over more than
    one chunk of tile aggregates."""
    from neslgpu_gb300.cvl import load
    from neslgpu_gb300.ops import DeviceRunner
    from conftest import _has_gpu
    if not _has_gpu():
        pytest.skip("no GPU")
    _run_all(DeviceRunner(load(), offset=1), oracle, (1 << 22) + 13, kind, seed=41)


@pytest.mark.parametrize("kind", ["long", "tiny", "empty", "one"])
def test_parity_two_million(gpu, oracle, kind):
    """Every primitive past 2^21 elements (a thousand tiles and more):
    segments spanning many tiles, tiny and empty segments, one segment."""
    _run_all(gpu, oracle, (1 << 21) + 13, kind, seed=31)
