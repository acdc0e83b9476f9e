"""The DLIST rebuild trigger (nl_check, nblist.c:607-647) restated in the
oracle: thresholds, the per-axis image rule and the site range, pinned to
the reference's own nl_check on golden cases."""
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


def test_restatement_matches_the_reference_golden_cases():
    """oracle.nl_check against the reference's own nl_check (nblist.c built
    with -DDLIST, tests/golden/nlcheck600.npz): below, at and above the
    threshold, the distance test, boundary crossings, site ranges."""
    import os
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "nlcheck600.npz"))
    got = [O.nl_check(d["pos_cases"][c], d["pos0"], d["L"], float(d["rclist"]), float(d["rc"]),
                      int(d["lb"][c]), int(d["ub"][c])) for c in range(len(d["flags"]))]
    assert got == [int(f) for f in d["flags"]]
    assert 0 in got and 1 in got
