"""Pins the oracle's classic-Ewald Monte Carlo energies to the reference's
own -DMC build (fixture tests/golden/mc.npz, made by oracle/ref_harness.c
driving enbnd_mc / ewald_kspace_mc / ewald_rspace_mc, ewald_mc.c:42-641):

* the k-space energy of the whole box and its change under each trial move,
  bit for bit (same operation order);
* on the cluster box, where no pair needs a periodic image, the real-space
  and LJ parts of each move's energy change to 1e-10 (the reference sums
  over its half list, the oracle over all partners);
* on the periodic box the reference's real space differs from the oracle's
  for moves whose pairs cross the box edge: ewald_mc.c:432-437 assigns
  dx = -lx instead of subtracting lx.  The engine and the oracle keep the
  correct minimum image; the test shows the reference's slip is the only
  difference (LJ, computed with the correct image by enbnd_mc, agrees).
"""
import numpy as np

from oracle import oracle as O
from tests.helpers import mc_case, mc_reference_parts


def test_kspace_energy_bit_exact(golden_mc):
    for which in ("per", "clu"):
        s, kmax, mks, moves, e = mc_case(golden_mc, which)
        o = O.Oracle(s)
        assert o.ewald_kspace_energy(s.pos, kmax, mks) == e[0, 4], which
        for (lb, ub, new), r in zip(moves, e[1:]):
            pn = s.pos.copy()
            pn[lb:ub] = new
            assert o.ewald_kspace_energy(pn, kmax, mks) == r[12], (which, lb)


def test_mc_delta_parts_match_reference_on_cluster(golden_mc):
    s, kmax, mks, moves, e = mc_case(golden_mc, "clu")
    want = mc_reference_parts(e)
    o = O.Oracle(s)
    for (lb, ub, new), w in zip(moves, want):
        pn = s.pos.copy()
        pn[lb:ub] = new
        de, parts = o.mc_delta_energy(s.pos, pn, lb, ub, kmax=kmax, max_k_square=mks)
        np.testing.assert_allclose(parts, w, rtol=1e-10, atol=1e-10)
        assert abs(de - w.sum()) <= 1e-10 * max(1.0, abs(de))


def test_periodic_box_differs_only_by_the_reference_image_slip(golden_mc):
    s, kmax, mks, moves, e = mc_case(golden_mc, "per")
    want = mc_reference_parts(e)
    o = O.Oracle(s)
    slips = 0
    for (lb, ub, new), w in zip(moves, want):
        pn = s.pos.copy()
        pn[lb:ub] = new
        _, parts = o.mc_delta_energy(s.pos, pn, lb, ub, kmax=kmax, max_k_square=mks)
        assert parts[0] == w[0]  # k-space: bit for bit
        assert abs(parts[2] - w[2]) <= 1e-10 * max(1.0, abs(w[2]))  # LJ: same image rule
        slips += abs(parts[1] - w[1]) > 1e-6
    assert slips > 0  # the 600-site box is small: its moves reach across the edge
