"""The LJ switch (CHARMM form, r_switch..rc) of the oracle, checked against
the mathematics rather than against another restatement: the force is minus
the derivative of the energy (central finite differences), the energy and
the force are continuous at r_switch, and both vanish at rc.  The reference
has no switch (cnonbond_nblist.c:284-319 truncates with an energy shift), so
these properties are what pins the oracle's switched pair term, which the FP64
and mixed kernels are then compared with on the GPU."""
import numpy as np
import pytest

from oracle import oracle as O

RC, RON = 10.0, 8.0


def _pair_system(r, q=(0.0, 0.0), r_switch=RON):
    from thecodecombo_7_gb300 import systems
    s = systems.water_box(2, L=40.0, seed=3, r_switch=r_switch)
    # two oxygen-type sites on the x axis, no topology
    s.pos = np.array([[-0.5 * r, 0.1, -0.2], [0.5 * r, 0.1, -0.2]])
    s.vel = np.zeros((2, 3))
    s.q = np.array(q, dtype=np.float64)
    s.mass = np.array([16.0, 16.0])
    s.type = np.array([0, 0], dtype=np.int32)
    e = np.zeros((0, 2), np.int32)
    s.bonds, s.bends, s.excl = e, np.zeros((0, 3), np.int32), e
    s.bond_req = s.bond_k = s.bend_theta0 = s.bend_k = np.zeros(0)
    s.excl_flag = np.zeros(0, np.int32)
    return s


def _lj(r, r_switch=RON):
    """(LJ energy, x-force on site 1) of the pair at separation r."""
    s = _pair_system(r, r_switch=r_switch)
    o = O.Oracle(s)
    lst = (np.array([1, 0], np.int32), np.array([1], np.int32), np.array([0], np.int32))
    ff, e5 = o.pair_forces(s.pos, lst)
    return e5[0] - e5[1], ff[1, 0]  # enonbond minus the shift term (zero when switched)


@pytest.mark.parametrize("r", [3.3, 5.0, 7.9, 8.05, 8.7, 9.3, 9.97])
def test_switched_force_is_minus_energy_gradient(r):
    h = 1e-5
    ep, _ = _lj(r + h)
    em, _ = _lj(r - h)
    _, f = _lj(r)
    fd = -(ep - em) / (2.0 * h)  # site 1 sits at +r/2: dE/dx1 = dE/dr
    assert abs(f - fd) <= 1e-6 * max(1.0, abs(f)), (r, f, fd)


def test_switch_continuous_at_r_switch_and_zero_at_rc():
    d = 1e-7
    e_lo, f_lo = _lj(RON - d)
    e_hi, f_hi = _lj(RON + d)
    # across 2d both move by their slopes only (a jump would be ~1e-3 here)
    assert abs(e_hi - e_lo) <= 1.5 * 2 * d * abs(f_lo), (e_lo, e_hi, f_lo)
    assert abs(f_hi - f_lo) <= 1e-8, (f_lo, f_hi)
    e_rc, f_rc = _lj(RC - 1e-6)
    assert abs(e_rc) <= 1e-12 and abs(f_rc) <= 1e-8, (e_rc, f_rc)  # E ~ d^2, F ~ d
    e_out, f_out = _lj(RC + 1e-6)
    assert e_out == 0.0 and f_out == 0.0


def test_switch_off_is_the_reference_shift():
    """Below r_switch the switched energy is the plain LJ; with the switch
    off the reference's shifted form (energy minus its value at rc, reported
    in the shift term) is kept."""
    r = 6.0
    e_sw, f_sw = _lj(r)
    e_ref, f_ref = _lj(r, r_switch=0.0)
    s = _pair_system(r)
    eps, sig = (x[0, 0] for x in s.lj_tables())
    sr6 = (sig / r) ** 6
    sr6c = (sig / RC) ** 6
    assert abs(e_sw - eps * (sr6 * sr6 - 2 * sr6)) <= 1e-12
    assert abs(e_ref - eps * ((sr6 * sr6 - 2 * sr6) - (sr6c * sr6c - 2 * sr6c))) <= 1e-12
    assert f_sw == f_ref
