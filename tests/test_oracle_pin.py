"""Pins the CPU oracle (oracle/fe_oracle.c) to the reference.

(1) against golden fixtures made by running the reference's own routines
    (tests/golden/make_golden.py) -- bit for bit;
(2) against the reference built from source right now, when its sources are
    present (development machine only);
(3) the oracle's FFT against numpy's DFT.
"""
import hashlib
import os

import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import system_from_golden


def _pair_hash(cnt, idx):
    rows = np.repeat(np.arange(cnt.shape[0], dtype=np.int64), cnt)
    key = rows * (1 << 32) + idx.astype(np.int64)
    return hashlib.sha256(np.sort(key).tobytes()).hexdigest()


def test_oracle_lists_bit_exact(golden600):
    s = system_from_golden(golden600, 200)
    orc = O.Oracle(s)
    cnt, idx, flg, ce, ie, fe = orc.nblist(s.pos, with_ew=True)
    np.testing.assert_array_equal(cnt, golden600["nblist_nl_cnt"])
    np.testing.assert_array_equal(idx, golden600["nblist_nl_idx"])
    np.testing.assert_array_equal(flg, golden600["nblist_nl_flg"])
    np.testing.assert_array_equal(ce, golden600["nblist_nlew_cnt"])
    np.testing.assert_array_equal(ie, golden600["nblist_nlew_idx"])
    np.testing.assert_array_equal(fe, golden600["nblist_nlew_flg"])


def test_oracle_forces_bit_exact(golden600):
    g = golden600
    s = system_from_golden(g, 200)
    orc = O.Oracle(s)
    lst = orc.nblist(s.pos)
    ff, en = orc.forces(s.pos, lst)
    np.testing.assert_array_equal(ff.ravel(), g["forces_f_total"])
    ref_en = dict(zip(O.EN_KEYS, g["forces_en"]))
    for k, v in en.items():
        assert v == ref_en[k], k
    grid = orc.charge_grid(s.pos)
    np.testing.assert_array_equal(grid.ravel(), g["forces_qgrid"])
    fp, e3 = orc.pme(s.pos)
    np.testing.assert_array_equal(fp.ravel(), g["forces_f_pme"])
    np.testing.assert_array_equal(e3, g["forces_e_pme"])
    fb, eb, ea = orc.bonded(s.pos)
    np.testing.assert_array_equal(fb.ravel(), g["forces_f_bonded"])
    assert (eb, ea) == tuple(g["forces_e_bonded"])


@pytest.mark.parametrize("mode", ["nve", "nhc"])
def test_oracle_trajectory_bit_exact(golden600, mode):
    g = golden600
    s = system_from_golden(g, 200)
    orc = O.Oracle(s)
    o = orc.run_md(12, use_nhc=(mode == "nhc"))
    np.testing.assert_array_equal(o["en"].ravel(), g[mode + "_en_steps"])
    np.testing.assert_array_equal(o["pos"].ravel(), g[mode + "_pos"])
    np.testing.assert_array_equal(o["pos_nopbc"].ravel(), g[mode + "_pos_nopbc"])
    np.testing.assert_array_equal(o["vel"].ravel(), g[mode + "_vel"])
    np.testing.assert_array_equal(o["force"].ravel(), g[mode + "_force"])
    if mode == "nhc":
        np.testing.assert_array_equal(o["zeta"].ravel(), g["nhc_zeta"])


def test_oracle_4095_box(golden4095):
    g = golden4095
    s = system_from_golden(g, 1365)
    orc = O.Oracle(s)
    cnt, idx, flg = orc.nblist(s.pos)
    np.testing.assert_array_equal(cnt, g["nl_cnt"])
    assert _pair_hash(cnt, idx) == str(g["nl_hash"])
    np.testing.assert_array_equal([(flg == f).sum() for f in range(5)], g["nl_nflag"])
    ff, en = orc.forces(s.pos, (cnt, idx, flg))
    np.testing.assert_array_equal(ff.ravel(), g["forces_f_total"])
    ref_en = dict(zip(O.EN_KEYS, g["forces_en"]))
    for k, v in en.items():
        assert v == ref_en[k], k


@pytest.mark.skipif(O.reference_dir() is None, reason="reference sources not present")
def test_oracle_against_live_reference(tmp_path):
    from thecodecombo_7_gb300 import systems
    assert O.build_reference()
    s = systems.water_box(150, L=24.5, seed=99, grid=(20, 24, 30))
    s.nlist_freq = 3
    ref = O.run_reference("forces", s, str(tmp_path))
    orc = O.Oracle(s)
    ff, en = orc.forces(s.pos)
    np.testing.assert_array_equal(ff.ravel(), ref["f_total"])
    traj = O.run_reference("nhc", s, str(tmp_path), nsteps=7)
    o = orc.run_md(7, use_nhc=True)
    np.testing.assert_array_equal(o["en"].ravel(), traj["en_steps"])
    np.testing.assert_array_equal(o["vel"].ravel(), traj["vel"])


@pytest.mark.parametrize("shape", [(8, 9, 10), (24, 25, 27), (7, 1, 13)])
def test_oracle_fft_matches_dft(shape):
    import ctypes as C
    lib = C.CDLL(O.build())
    rng = np.random.default_rng(3)
    x = rng.normal(size=shape) + 1j * rng.normal(size=shape)
    for sign in (-1, 1):
        buf = np.ascontiguousarray(np.stack([x.real, x.imag], -1))
        lib.fe_fft3d(buf.ctypes.data_as(C.c_void_p), *shape, sign)
        got = buf[..., 0] + 1j * buf[..., 1]
        want = np.fft.fftn(x) if sign == -1 else np.fft.ifftn(x) * x.size
        np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-11 * np.abs(want).max())


def test_oracle_chain_terms_bit_exact(golden_chain):
    """Urey-Bradley, torsions (with a series that stops at a zero term) and
    impropers: the oracle's restatements equal the reference's curey,
    ctorsion and cimproper bit for bit, torsion angles included; the
    non-bonded forces with 1-4 pairs (xflag 4) too; the full forces() to
    rounding (the oracle sums the terms in another order)."""
    from helpers import chain_from_golden
    g = golden_chain
    s = chain_from_golden(g)
    orc = O.Oracle(s)
    x = orc.bonded_ext(s.pos)
    for k in ("f_urey", "f_tors", "f_impr"):
        np.testing.assert_array_equal(x[k].ravel(), g["forces_" + k], err_msg=k)
    assert (x["e_urey"], x["e_tors"], x["e_impr"]) == tuple(g["forces_e_ext"])
    np.testing.assert_array_equal(x["tau"], g["forces_tau"])
    np.testing.assert_array_equal(g["forces_en_ext"], g["forces_e_ext"])
    lst = orc.nblist(s.pos)
    ff, en = orc.forces(s.pos, lst)
    fb, eb, ea = orc.bonded(s.pos)
    np.testing.assert_array_equal(fb.ravel(), g["forces_f_bonded"])
    # cnonbondnl: the pair loop and pme_calc adding into one force array
    import ctypes as C
    cnt, idx, flg = lst
    pos = np.ascontiguousarray(s.pos)
    fnb, e5, e3 = np.zeros((s.n, 3)), np.zeros(5), np.zeros(3)
    orc.lib.or_cnonbond_pairs(orc.sp, O._p(pos), O._p(cnt), O._p(idx), O._p(flg), O._p(fnb),
                              O._p(e5))
    orc.lib.or_pme_calc(orc.sp, O._p(pos), C.c_double(orc.ewald_self()), O._p(fnb), O._p(e3))
    np.testing.assert_array_equal(fnb.ravel(), g["forces_f_nonbond"])
    total = ff + x["f_urey"] + x["f_tors"] + x["f_impr"]
    scale = np.abs(g["forces_f_total"]).max()
    assert np.abs(total.ravel() - g["forces_f_total"]).max() < 1e-12 * scale
    ref_en = dict(zip(O.EN_KEYS, g["forces_en"]))
    for k in ("nbond", "nbonds", "coulomb", "rewald", "rewalds", "kewald", "sewald", "iewald"):
        assert en[k] == ref_en[k], k


def test_respa_fixtures_semantics(golden_chain, golden_mts600):
    """The reference's RESPA runs (integrate_mts.c) as committed: ff ends as
    force_long's forces (ff_long = ff, force_long.c:139-143), uu = vv after
    the last kick (integrate_mts.c:133-135), and the water box's total energy
    stays within 1 % over 8 long steps of 2 fs."""
    for g, nlong in ((golden_chain, 6), (golden_mts600, 8)):
        assert np.array_equal(g["mts_force"], g["mts_f_long"])
        assert np.array_equal(g["mts_vel"], g["mts_vel_uu"])
        assert g["mts_en_steps"].shape == (15 * (nlong + 1),)
    e = golden_mts600["mts_en_steps"].reshape(-1, 15)
    tot = e[:, 0] + e[:, 1] + e[:, 2] + e[:, 3] + e[:, 12] + e[:, 13] + e[:, 14]
    assert np.abs(tot - tot[0]).max() < 0.01 * abs(tot[0])


def test_oracle_bgo_pair_form_bit_exact(golden_bgo600):
    """The BGO build's pair form (cnonbond_nblist.c:294-307: eps [13 (R/r)^12
    - 18 (R/r)^10 + 4 (R/r)^6]) against the reference's own -DBGO build
    (oracle/_ref/ref_harness_bgo, fixture tests/golden/bgo600.npz): the full
    forces() and every energy term bit for bit."""
    g = golden_bgo600
    s = system_from_golden(g, 200)
    s.lj_form = 2
    orc = O.Oracle(s)
    ff, en = orc.forces(s.pos, orc.nblist(s.pos))
    np.testing.assert_array_equal(ff.ravel(), g["forces_f_total"])
    ref_en = dict(zip(O.EN_KEYS, g["forces_en"]))
    for k, v in en.items():
        assert v == ref_en[k], k
