"""The DLIST rebuild trigger (nl_check, nblist.c:607-647) restated in the
oracle: thresholds, the per-axis image rule and the site range."""
import numpy as np

from oracle import oracle as O

L = np.array([30.0, 30.0, 30.0])
RCLIST, RC = 12.0, 10.0  # rcut = 0.5 A


def _pos(n=20, seed=1):
    rng = np.random.default_rng(seed)
    return (rng.random((n, 3)) - 0.5) * L


def test_below_and_above_threshold():
    p0 = _pos()
    p = p0.copy()
    p[3, 0] += 0.49
    assert O.nl_check(p, p0, L, RCLIST, RC) == 0
    p[3, 0] += 0.02
    assert O.nl_check(p, p0, L, RCLIST, RC) == 1


def test_distance_test_beyond_the_axis_tests():
    p0 = _pos()
    p = p0.copy()
    p[5] += np.array([0.3, 0.3, 0.3])  # every axis below 0.5, distance 0.52
    assert O.nl_check(p, p0, L, RCLIST, RC) == 1


def test_image_rule_for_a_site_that_wrapped():
    p0 = _pos()
    p0[7] = [14.9, 0.0, 0.0]
    p = p0.copy()
    p[7, 0] = -14.9  # moved 0.2 A across the boundary: |d| = 29.8 > L/2 -> -0.2
    assert O.nl_check(p, p0, L, RCLIST, RC) == 0


def test_range_limits_the_sites_checked():
    p0 = _pos()
    p = p0.copy()
    p[15, 1] += 1.0
    assert O.nl_check(p, p0, L, RCLIST, RC, 0, 10) == 0
    assert O.nl_check(p, p0, L, RCLIST, RC, 10, 20) == 1
