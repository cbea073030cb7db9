"""The FP64 adjudication of end-to-end label mismatches (tests/parity.py) on
the CPU: the derived near-tie bound accepts mismatches the FP32 arithmetic
and the measured centroid drift explain, and rejects a label planted in the
oracle's output that no rounding can produce."""
import numpy as np
import pytest

import parity
from conftest import blobs


def test_identical_runs_have_nothing_to_adjudicate(oracle):
    n, d, k = 5000, 4, 6
    P = blobs(n, d, k, seed=1)
    C0 = oracle.first_x_f32(P, n, d, k)
    C, _, L = oracle.lloyd_f32(P, n, d, k, 3, C0)
    out = parity.adjudicate(P, n, d, k, L, L, C, C)
    assert out["mismatches"] == 0 and out["max_drift"] == 0.0


def test_planted_far_label_is_rejected(oracle):
    """A label moved to a cluster far from the point (planted in the oracle's
    labels) is outside the bound."""
    n, d, k = 5000, 4, 6
    P = blobs(n, d, k, seed=2)
    C = oracle.first_x_f32(P, n, d, k)
    L = oracle.label_f32(P, n, d, k, C)
    bad = L.copy()
    _, gap, best = oracle.label_gap_f64(P, n, d, k, C)
    p = int(np.argmax(gap / np.maximum(best, 1e-30)))    # the clearest point
    bad[p] = (bad[p] + 1) % k
    with pytest.raises(AssertionError, match="outside the derived near-tie bound"):
        parity.adjudicate(P, n, d, k, bad, L, C, C)


def test_exact_tie_is_accepted_and_drift_widens_the_bound(oracle):
    """A point equidistant from two centroids may take either label; a point
    slightly off the tie is accepted only when the measured drift between the
    two runs' centroids covers its gap."""
    d, k = 2, 2
    C = np.array([-1.0, 1.0, 0.0, 0.0], np.float32)      # centroids (-1, 0) and (1, 0)
    P = np.array([0.0, 1e-3, 0.5, 0.5], np.float32)      # points (0, .5) and (1e-3, .5)
    n = 2
    ours = np.array([1, 0], np.uint32)                   # the tie flipped, and the near tie
    ref = np.array([0, 1], np.uint32)
    with pytest.raises(AssertionError):
        parity.adjudicate(P, n, d, k, ours, ref, C, C)    # no drift: the 1e-3 offset is too large
    C_ours = C.copy()
    C_ours[0] += 2e-3                                    # our first centroid drifted by 2e-3
    out = parity.adjudicate(P, n, d, k, ours, ref, C_ours, C)
    assert out["mismatches"] == 2 and out["worst_gap_over_bound"] <= 1.0


def test_rho_matches_the_kernels():
    assert parity.rho(4) == 8 * 2.0 ** -24
    assert parity.rel_centroid_error(np.array([1.0, np.nan, 3.0]), np.array([1.0, 2.0, 3.0 + 3e-6])) == \
        pytest.approx(3e-6 / (3.0 + 3e-6), rel=1e-9)
