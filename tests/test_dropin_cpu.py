"""Host pieces of the drop-in boundary (no GPU): the oracle's drift() pinned
to the reference's own (fixture tests/golden/drift600.npz made by running
drift.c), and the engine's host B-spline routine fe_bspline (the shim's
fillspline, pme_spline.c:10-49) against the oracle's restatement, bit for
bit."""
import ctypes as C
import os

import numpy as np
import pytest

from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_oracle_drift_bit_exact():
    from thecodecombo_7_gb300 import systems
    g = np.load(os.path.join(GOLDEN, "drift600.npz"))
    s = systems.water_box(200, L=25.0, seed=7, grid=(24, 25, 27), helper=False)
    np.testing.assert_array_equal(s.mass, g["mass"])
    v = O.Oracle(s).drift(g["vel0"])
    np.testing.assert_array_equal(v, g["vel"])
    p0 = (g["vel0"] * g["mass"][:, None]).sum(0)
    p = (g["vel"] * g["mass"][:, None]).sum(0)
    assert np.abs(p).max() < 1e-14 * np.abs(p0).max()  # the net momentum is gone


@pytest.mark.parametrize("order", [3, 4, 5, 6, 8])
def test_fe_bspline_matches_oracle(order):
    from thecodecombo_7_gb300 import engine
    lib = engine.load_library()
    lib.fe_bspline.argtypes = [C.c_int, C.c_double, C.c_void_p, C.c_void_p]
    for w in (0.0, 0.125, 0.3, 0.5, 0.77, 0.999):
        a = np.zeros(order + 1)
        d = np.zeros(order + 1)
        assert lib.fe_bspline(order, w, a.ctypes.data, d.ctypes.data) == 0
        ra, rd = O.fillspline(order, w)
        np.testing.assert_array_equal(a[1:], ra[1:])
        np.testing.assert_array_equal(d[1:], rd[1:])
        assert abs(a[1:].sum() - 1.0) < 1e-14  # partition of unity
    assert lib.fe_bspline(2, 0.5, a.ctypes.data, d.ctypes.data) == engine.FE_ERR_ARG
