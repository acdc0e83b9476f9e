"""The engine calls the drop-in shim issues (thecodecombo_7_gb300/dropin/
fe_dropin.c), driven in the same order on the GPU and checked against the
reference's own outputs and the oracle:

* drift(): fe_drift against the reference's drift.c (fixture drift600.npz);
* one Monte Carlo move as forces_mc(lb, ub, 0|1) issues it: fe_mc_site_energy
  before, fe_mc_delta_terms for the trial, assembled into enbnd_mc's
  energy[8] -- the change of every entry against the reference's -DMC
  enbnd_mc around the same move (fixture mc.npz, cluster box), then the
  accepted move committed and the next move measured from it;
* one replica swap as swap_box(k) issues it: the two boxes' engine states
  exchanged, each keeping its temperature (fe_box_set_temperature), the
  velocities rescaled by sqrt(T_k / T_k+1) and uploaded; the Nose-Hoover
  steps that follow match the oracle started from the swapped states.
"""
import os

import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import mc_case

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _box(s, **kw):
    from thecodecombo_7_gb300 import engine
    return engine.Box(s, precision=engine.FE_PREC_FP64, **kw)


def test_drift_matches_reference():
    from thecodecombo_7_gb300 import systems
    g = np.load(os.path.join(GOLDEN, "drift600.npz"))
    s = systems.water_box(200, L=25.0, seed=7, grid=(24, 25, 27), helper=False)
    s.vel = g["vel0"]
    with _box(s) as b:
        b.drift()
        v, u = b.get_velocities()
    np.testing.assert_allclose(v, g["vel"], rtol=0, atol=1e-13 * np.abs(g["vel"]).max())
    np.testing.assert_array_equal(u, g["uu"])  # uu untouched, as drift.c


def _energy8(t, sew):
    """enbnd_mc energy[8] from the six engine terms (the shim's energy8)."""
    e0 = t[1] + t[3] - t[5] + (t[0] - sew)
    return np.array([e0, e0 - t[2], t[3] + (t[0] - sew) - t[5], t[4], t[0], sew, t[5], t[3]])


def test_mc_move_sequence_matches_reference(golden_mc):
    s, kmax, mks, moves, e = mc_case(golden_mc, "clu")
    sew = e[0, 5]
    with _box(s) as b:
        b.mc_setup(kmax=kmax, max_k_square=mks)
        for (lb, ub, new), ref in zip(moves, e[1:]):
            t_old = b.mc_site_energy(lb, ub)              # forces_mc(lb, ub, 0, k)
            d = b.mc_delta_terms(lb, ub, new)             # forces_mc(lb, ub, 1, k)
            got = _energy8(t_old + d, sew) - _energy8(t_old, sew)
            want = ref[8:] - ref[:8]
            np.testing.assert_allclose(got, want, rtol=1e-9, atol=1e-9)
            # the k-space energy is absolute in both: compare it directly
            assert abs(t_old[0] - ref[4]) <= 1e-10 * abs(ref[4])
        # a kept move is committed; the next evaluation starts from it
        lb, ub, new = moves[0]
        b.mc_delta_terms(lb, ub, new)
        b.mc_accept()
        pn = s.pos.copy()
        pn[lb:ub] = new
        o = O.Oracle(s)
        assert abs(b.mc_kspace_energy() - o.ewald_kspace_energy(pn, kmax, mks)) <= \
            1e-10 * abs(b.mc_kspace_energy())
        lb2, ub2, new2 = moves[1]
        d = b.mc_delta_terms(lb2, ub2, new2)
        pn2 = pn.copy()
        pn2[lb2:ub2] = new2
        want, parts = o.mc_delta_energy(pn, pn2, lb2, ub2, kmax=kmax, max_k_square=mks)
        assert abs((d[0] + d[1] - d[2] + d[3] - d[5]) - want) <= 1e-8 * max(1.0, abs(want))


def test_swap_sequence_matches_oracle():
    from thecodecombo_7_gb300 import systems
    T = (300.0, 330.0)
    sa = systems.water_box(200, L=25.0, seed=7, grid=(24, 25, 27), T=T[0])
    sb = systems.water_box(200, L=25.0, seed=8, grid=(24, 25, 27), T=T[1])
    sa.nlist_freq = sb.nlist_freq = 5
    boxes = [_box(sa), _box(sb)]
    try:
        for b in boxes:
            b.nblist()
            b.forces()
            b.kinet()
            b.run_md(3, use_nhc=True, record=False)
        st = [dict(pos=b.get_positions(), nop=b.get_positions_nopbc(),
                   vel=b.get_velocities()[0], zeta=b.get_nhc_state()) for b in boxes]
        # swap_box(0): configurations trade boxes, temperatures and chains stay
        boxes.reverse()
        scale = np.sqrt(T[0] / T[1])
        vel = [st[1]["vel"] * scale, st[0]["vel"] / scale]
        for k, b in enumerate(boxes):
            b.set_temperature(T[k])
            b.set_velocities(vel[k])
            b.set_nhc_state(st[k]["zeta"])
            b.nblist()
        recs = [b.run_md(4, use_nhc=True, first_step=1) for b in boxes]
        for k in range(2):
            other = 1 - k
            s = (sa, sb)[k]
            o = O.Oracle(s)
            md = o.run_md(4, use_nhc=True, pos=st[other]["pos"], vel=vel[k],
                          zeta=st[k]["zeta"], pos_nopbc=st[other]["nop"], T=T[k])
            want = md["en"][1:]
            rel = np.abs(recs[k][:, :want.shape[1]] - want).max() / np.abs(want).max()
            assert rel < 1e-10, (k, rel)
            np.testing.assert_allclose(boxes[k].get_positions(), md["pos"], rtol=0, atol=1e-10)
    finally:
        for b in boxes:
            b.close()


def _pinned_copies(arrs):
    import torch
    out = []
    for a in arrs:
        t = torch.empty(a.shape, dtype=torch.float64, pin_memory=True).numpy()
        t[:] = a
        out.append(t)
    return out


def test_integrate_vverlet_host_equals_separate_calls(golden600):
    """fe_integrate_vverlet_host with pinned arrays (copies and kernels of
    the step in one graph per set of host arrays, replayed; a new set midway
    is captured anew) and with plain numpy arrays (the separate upload /
    step / download calls) gives the results of the separate calls:
    bit for bit in mixed precision (fixed-point force sums), and to the
    run-to-run spread of the FP64 atomic force sums in FP64."""
    from thecodecombo_7_gb300 import engine
    from tests.helpers import system_from_golden
    s = system_from_golden(golden600, 200)
    for prec in (engine.FE_PREC_FP64, engine.FE_PREC_MIXED):
        outs = []
        for mode in ("pinned", "numpy", "calls"):
            with engine.Box(s, precision=prec) as b:
                b.nblist()
                b.forces()
                arrs = [b.get_positions(), b.get_positions_nopbc(), *b.get_velocities(),
                        b.get_forces()]
                if mode == "pinned":
                    arrs = _pinned_copies(arrs)
                for i in range(1, 7):
                    if i % s.nlist_freq == 0:
                        b.nblist()
                    if mode == "pinned" and i == 4:
                        # other host arrays: the step's graph is captured anew
                        arrs = _pinned_copies(arrs)
                    if mode == "calls":
                        b.set_positions(arrs[0])
                        b.set_positions_nopbc_array(arrs[1])
                        b.set_velocities(arrs[2], arrs[3])
                        b.set_forces(arrs[4])
                        en = b.integrate_vverlet()
                        arrs = [b.get_positions(), b.get_positions_nopbc(), *b.get_velocities(),
                                b.get_forces()]
                    else:
                        en = b.integrate_vverlet_host(*arrs)
                outs.append(([a.copy() for a in arrs], en))
        for other in outs[1:]:
            for k, (a, c) in enumerate(zip(outs[0][0], other[0])):
                if prec == engine.FE_PREC_MIXED:
                    assert np.array_equal(a, c), k
                else:
                    assert np.abs(a - c).max() <= 1e-10 * max(1.0, np.abs(a).max()), k
            for key, v in outs[0][1].items():
                if prec == engine.FE_PREC_MIXED:
                    assert v == other[1][key], key
                else:
                    assert abs(v - other[1][key]) <= 1e-10 * max(1.0, abs(v)), key
