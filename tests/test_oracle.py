"""The oracle (oracle/cvl_oracle.c) against the reference's own serial CVL,
compiled from its sources here, on the shared parity cases: every result
must be bit-identical, float64 sums included, because the oracle folds in
the serial CVL's order."""
import numpy as np
import pytest

from cases import make_cases, compare

KINDS = ["geo", "tiny", "empty", "bimodal", "one", "long"]


@pytest.mark.parametrize("kind", KINDS)
def test_oracle_matches_serial_cvl(oracle, reference, kind):
    for cid, fn, cmp, ctx in make_cases(n=3000, seed=11, lengths_kind=kind):
        got = fn(oracle)
        want = fn(reference)
        try:
            compare("exact", got, want)
        except AssertionError as e:
            raise AssertionError(f"{cid} ({kind}): {e}") from None


@pytest.mark.parametrize("n", [0, 1, 2, 33])
def test_oracle_small_sizes(oracle, reference, n):
    for cid, fn, cmp, ctx in make_cases(n=n, seed=3, lengths_kind="geo", include_ulp=False):
        compare("exact", fn(oracle), fn(reference))
