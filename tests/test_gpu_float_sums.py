"""Float64 +-scans and +-reductions on inputs that stress the fixed-point
folds: magnitudes spread over 2^-60 .. 2^60 within segments, zeros,
subnormals, a few values near 1e290, and (second set) infinities and NaNs in
some warps only.  Finite results must agree with the oracle within
|a - b| <= 1e-12 * max(|b|, S), S the sum of magnitudes over the same prefix
or segment; non-finite results must be the same infinity or a NaN."""
import numpy as np
import pytest

from neslgpu_gb300 import ops
from neslgpu_gb300 import workloads as W

pytestmark = pytest.mark.gpu

N = 300_003


def _values(r, n, specials):
    x = r.standard_normal(n) * np.exp2(r.integers(-60, 61, n).astype(np.float64))
    x[r.random(n) < 0.01] = 0.0
    tiny = r.random(n) < 0.005
    x[tiny] *= 2.0 ** -1070  # subnormal or zero
    x[r.random(n) < 0.001] *= 2.0 ** 900
    if specials:
        for v in (np.inf, -np.inf, np.nan):
            x[r.choice(n, size=6, replace=False)] = v
    return x


def _lengths(r, n, kind):
    if kind == "geo":
        return W.geometric_lengths(r, n, 64)
    if kind == "tiny":
        return W.geometric_lengths(r, n, 1.5)
    return W.lognormal_lengths(r, n, 9.0, 2.0, n)


def _seg_abs(x, lens, exclusive):
    """S per element (exclusive prefix) or per segment, summed segment by
    segment so that large values elsewhere do not swamp it."""
    a = np.abs(x)
    out = []
    k = 0
    for L in lens.tolist():
        c = np.cumsum(a[k:k + L])
        if exclusive:
            out.append(np.concatenate([[0.0], c[:-1]]) if L else c)
        else:
            out.append([c[-1] if L else 0.0])
        k += L
    return np.concatenate(out) if out else np.zeros(0)


def _check(got, want, S):
    got = np.atleast_1d(np.asarray(got, dtype=np.float64))
    want = np.atleast_1d(np.asarray(want, dtype=np.float64))
    fin = np.isfinite(want)
    bad = ~fin & ~((got == want) | (np.isnan(got) & np.isnan(want)))
    assert not bad.any(), f"non-finite mismatch at {np.flatnonzero(bad)[:8]}"
    tol = 1e-12 * np.maximum(np.abs(want[fin]), S[fin]) + 1e-300
    err = np.abs(got[fin] - want[fin])
    ok = err <= tol
    if not ok.all():
        i = int(np.argmax(err / tol))
        raise AssertionError(f"got {got[fin][i]!r} want {want[fin][i]!r} tol {tol[i]:.3g}")


@pytest.mark.parametrize("specials", [False, True])
@pytest.mark.parametrize("kind", ["geo", "tiny", "long"])
def test_segmented_sums(gpu, oracle, kind, specials):
    r = W.rng(900 + 7 * specials + len(kind))
    x = _values(r, N, specials)
    lens = _lengths(r, N, kind)
    for name, fn, exclusive in (("add_sed", ops.scan_e, True), ("add_red", ops.reduce_e, False)):
        got = fn(gpu, name, x, lens)
        want = fn(oracle, name, x, lens)
        _check(got, want, _seg_abs(x, lens, exclusive))


@pytest.mark.parametrize("specials", [False, True])
def test_unsegmented_sums(gpu, oracle, specials):
    r = W.rng(950 + specials)
    x = _values(r, N, specials)
    one = np.array([N], dtype=np.int32)
    _check(ops.scan_u(gpu, "add_sud", x), ops.scan_u(oracle, "add_sud", x), _seg_abs(x, one, True))
    _check(ops.reduce_u(gpu, "add_rud", x), ops.reduce_u(oracle, "add_rud", x), _seg_abs(x, one, False))
