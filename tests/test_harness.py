"""The parity checks themselves: a non-finite value anywhere is an error, never a
pass (Python's max() ignores a NaN placed second)."""
import numpy as np

from harness import relerr


def test_relerr_flags_non_finite():
    ref = np.ones(10)
    got = ref.copy()
    assert relerr(ref, got) == 0.0
    got[3] = np.nan
    assert relerr(ref, got) == float("inf")
    got[3] = np.inf
    assert relerr(ref, got) == float("inf")
    assert max(0.0, relerr(ref, got)) == float("inf")
    bad_ref = ref.copy()
    bad_ref[0] = np.nan
    assert relerr(bad_ref, ref) == float("inf")
