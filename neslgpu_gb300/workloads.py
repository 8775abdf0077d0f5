"""Seeded synthetic inputs for the CVL benchmark configurations.

All generation is host-side numpy from fixed seeds, so the GPU library and
the CPU oracle see identical inputs.  The distributions restate the
benchmark configurations: uniform full-range int32 values, N(0,1)
float64 values, and segment lengths that are geometric, log-normal (capped),
power-law or bimodal.
"""
from __future__ import annotations

import numpy as np


def rng(seed: int) -> np.random.Generator:
    return np.random.Generator(np.random.PCG64(seed))


def int32_uniform(r: np.random.Generator, n: int) -> np.ndarray:
    return r.integers(-(2 ** 31), 2 ** 31, size=n, dtype=np.int64).astype(np.int32)


def float64_normal(r: np.random.Generator, n: int) -> np.ndarray:
    return r.standard_normal(n)


def _fit(lengths: np.ndarray, n: int) -> np.ndarray:
    """Cut a length sequence so that it sums exactly to n (last one truncated)."""
    c = np.cumsum(lengths, dtype=np.int64)
    k = int(np.searchsorted(c, n))
    out = lengths[: k + 1].astype(np.int64).copy()
    out[-1] -= int(c[k]) - n if k < len(c) else 0
    if out.sum() != n:  # ran out of draws: pad with one last segment
        out = np.append(out, n - out.sum())
    return out[out >= 0].astype(np.int32)


def geometric_lengths(r: np.random.Generator, n: int, mean: float) -> np.ndarray:
    """Geometric(p = 1/mean) on {1, 2, ...}, cut to sum to n."""
    if n == 0:
        return np.zeros(0, dtype=np.int32)
    est = int(n / mean * 1.2) + 16
    out = []
    total = 0
    while total < n:
        g = r.geometric(1.0 / mean, size=est)
        out.append(g)
        total += int(g.sum())
    return _fit(np.concatenate(out), n)


def lognormal_lengths(r: np.random.Generator, n: int, mu: float, sigma: float,
                      cap: int) -> np.ndarray:
    """round(LogNormal(mu, sigma)) clipped to [1, cap], cut to sum to n."""
    if n == 0:
        return np.zeros(0, dtype=np.int32)
    out = []
    total = 0
    while total < n:
        g = np.clip(np.rint(r.lognormal(mu, sigma, size=max(1024, n // 500))), 1, cap).astype(np.int64)
        out.append(g)
        total += int(g.sum())
    return _fit(np.concatenate(out), n)


def powerlaw_lengths(r: np.random.Generator, m: int, alpha: float, lo: int, hi: int) -> np.ndarray:
    """m draws of a discrete power law p(k) ~ k^-alpha on [lo, hi]."""
    k = np.arange(lo, hi + 1, dtype=np.float64)
    p = k ** (-alpha)
    p /= p.sum()
    return r.choice(np.arange(lo, hi + 1), size=m, p=p).astype(np.int32)


def bimodal_lengths(r: np.random.Generator, n: int, big: int = 4) -> np.ndarray:
    """A few very long segments plus many of length 1-4, summing to n."""
    if n == 0:
        return np.zeros(0, dtype=np.int32)
    long_total = n // 2
    longs = np.full(big, long_total // big, dtype=np.int64)
    longs[-1] += long_total - longs.sum()
    short = []
    total = 0
    rest = n - long_total
    while total < rest:
        g = r.integers(1, 5, size=max(16, rest // 2))
        short.append(g)
        total += int(g.sum())
    short = _fit(np.concatenate(short), rest).astype(np.int64)
    segs = np.concatenate([short, longs])
    r.shuffle(segs)
    return segs.astype(np.int32)


def with_empty(r: np.random.Generator, lengths: np.ndarray, frac: float) -> np.ndarray:
    """Insert empty segments (about frac * m of them) at random places."""
    m = len(lengths)
    k = int(m * frac) + 1
    pos = np.sort(r.integers(0, m + 1, size=k))
    return np.insert(lengths, pos, 0).astype(np.int32)


def permutation(r: np.random.Generator, n: int) -> np.ndarray:
    return r.permutation(n).astype(np.int32)


def seg_permutation(r: np.random.Generator, lengths: np.ndarray) -> np.ndarray:
    """Per-segment local permutations (indices relative to segment start)."""
    n = int(np.sum(lengths, dtype=np.int64))
    keys = r.random(n)
    seg = np.repeat(np.arange(len(lengths)), lengths)
    order = np.lexsort((keys, seg))
    lengths = np.asarray(lengths, dtype=np.int64)
    starts = np.cumsum(lengths) - lengths
    out = np.empty(n, dtype=np.int32)
    out[order] = (np.arange(n) - np.repeat(starts, lengths)).astype(np.int32)
    return out


def seg_indices(r: np.random.Generator, len_src: np.ndarray, len_dst: np.ndarray) -> np.ndarray:
    """For each destination element, a random index into the matching
    source segment (len_src[g] must be > 0 wherever len_dst[g] > 0)."""
    reps = np.repeat(len_src.astype(np.int64), len_dst)
    return (r.random(len(reps)) * reps).astype(np.int64).astype(np.int32)
