"""FP64 drop-in parity: the CUDA path (through the C ABI) against the
reference's own outputs (golden fixtures) and the pinned CPU oracle.

Tolerances: pair sets bit-exact; forces and energies agree to 1e-10 of the
force scale (the only differences are CUDA's exp vs glibc's and the order of
the final FP64 sums)."""
import hashlib

import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import system_from_golden

pytestmark = pytest.mark.gpu

FTOL = 1e-10  # relative to max |F|
ETOL = 1e-10  # relative, energies


def _box(s, **kw):
    from thecodecombo_7_gb300 import engine
    return engine.Box(s, precision=engine.FE_PREC_FP64, **kw)


def _hash(cnt, idx):
    rows = np.repeat(np.arange(cnt.shape[0], dtype=np.int64), cnt)
    key = rows * (1 << 32) + idx.astype(np.int64)
    return hashlib.sha256(np.sort(key).tobytes()).hexdigest()


def _close_f(got, want):
    scale = np.abs(want).max()
    err = np.abs(got - want).max()
    assert err <= FTOL * scale, f"max force error {err:.3e} (scale {scale:.3e})"


def _close_e(got, want, key=""):
    assert abs(got - want) <= ETOL * max(1.0, abs(want)), f"{key}: {got!r} vs {want!r}"


def test_nblist_bit_exact_600(golden600):
    g = golden600
    s = system_from_golden(g, 200)
    with _box(s) as b:
        b.nblist()
        cnt, idx, flg = b.nblist_download()
    np.testing.assert_array_equal(cnt, g["nblist_nl_cnt"])
    np.testing.assert_array_equal(idx, g["nblist_nl_idx"])
    np.testing.assert_array_equal(flg, g["nblist_nl_flg"])


def test_nblist_bit_exact_4095(golden4095):
    g = golden4095
    s = system_from_golden(g, 1365)
    with _box(s) as b:
        b.nblist()
        cnt, idx, flg = b.nblist_download()
    np.testing.assert_array_equal(cnt, g["nl_cnt"])
    assert _hash(cnt, idx) == str(g["nl_hash"])
    np.testing.assert_array_equal([(flg == f).sum() for f in range(5)], g["nl_nflag"])


def test_forces_fp64_vs_reference(golden600):
    g = golden600
    s = system_from_golden(g, 200)
    with _box(s) as b:
        b.nblist()
        en = b.forces()
        f = b.get_forces()
    _close_f(f.ravel(), g["forces_f_total"])
    ref = dict(zip(O.EN_KEYS, g["forces_en"]))
    for k in ("bond", "bend", "nbond", "nbonds", "coulomb", "rewald", "rewalds", "kewald",
              "sewald", "iewald", "tewald"):
        _close_e(en[k], ref[k], k)


def test_forces_fp64_4095(golden4095):
    g = golden4095
    s = system_from_golden(g, 1365)
    with _box(s) as b:
        b.nblist()
        en = b.forces()
        f = b.get_forces()
    _close_f(f.ravel(), g["forces_f_total"])
    ref = dict(zip(O.EN_KEYS, g["forces_en"]))
    for k in ("nbond", "nbonds", "rewald", "kewald", "iewald", "tewald"):
        _close_e(en[k], ref[k], k)


def test_spme_pieces(golden600):
    g = golden600
    s = system_from_golden(g, 200)
    with _box(s) as b:
        grid = b.charge_grid()
        np.testing.assert_allclose(grid.ravel(), g["forces_qgrid"], rtol=0, atol=1e-13)
        b.zero_forces()
        e3 = b.pme_calc()
        f = b.get_forces()
    _close_f(f.ravel(), g["forces_f_pme"])
    for k in range(3):
        _close_e(e3[k], g["forces_e_pme"][k])


def test_cnonbondnl_and_bonded(golden600):
    g = golden600
    s = system_from_golden(g, 200)
    with _box(s) as b:
        b.nblist()
        b.zero_forces()
        e8 = b.cnonbondnl()
        f = b.get_forces()
        _close_f(f.ravel(), g["forces_f_nonbond"])
        for k in range(8):
            _close_e(e8[k], g["forces_e_nonbond"][k], f"energy[{k}]")
        b.zero_forces()
        eb = b.bonded()
        fb = b.get_forces()
    np.testing.assert_allclose(fb.ravel(), g["forces_f_bonded"], rtol=0, atol=1e-9)
    np.testing.assert_allclose(eb, g["forces_e_bonded"], rtol=0, atol=1e-12)


@pytest.mark.parametrize("mode", ["nve", "nhc"])
def test_trajectory_fp64(golden600, mode):
    g = golden600
    s = system_from_golden(g, 200)
    with _box(s) as b:
        b.nblist()
        b.forces()
        b.kinet()
        rec = b.run_md(12, nlist_freq=s.nlist_freq, use_nhc=(mode == "nhc"))
        pos = b.get_positions()
        nop = b.get_positions_nopbc()
        vel, _ = b.get_velocities()
        f = b.get_forces()
    want = g[mode + "_en_steps"].reshape(-1, 12)[1:]
    for k in range(12):
        for i in range(12):
            _close_e(rec[i, k], want[i, k], f"step {i + 1} {O.EN_KEYS[k]}")
    np.testing.assert_allclose(pos.ravel(), g[mode + "_pos"], rtol=0, atol=1e-11)
    np.testing.assert_allclose(nop.ravel(), g[mode + "_pos_nopbc"], rtol=0, atol=1e-11)
    np.testing.assert_allclose(vel.ravel(), g[mode + "_vel"], rtol=0, atol=1e-9)
    _close_f(f.ravel(), g[mode + "_force"])


def test_reference_record_layout(golden600):
    """Positions read from and written to `struct atoms` records (64 B, x at 16)."""
    g = golden600
    s = system_from_golden(g, 200)
    rec = np.zeros(s.n, dtype=np.dtype({"names": ["t", "name", "x", "y", "z", "q", "n", "molec",
                                                  "atomid"],
                                        "formats": ["S5", "S5", "<f8", "<f8", "<f8", "<f8", "<i4",
                                                    "<i4", "<i4"],
                                        "offsets": [0, 5, 16, 24, 32, 40, 48, 52, 56],
                                        "itemsize": 64}))
    rec["x"], rec["y"], rec["z"] = s.pos[:, 0], s.pos[:, 1], s.pos[:, 2]
    rec["q"] = s.q
    with _box(s) as b:
        b.set_positions(np.zeros_like(s.pos))
        b.set_positions_records(rec, 64, 16)
        b.nblist()
        b.forces()
        f = b.get_forces()
        out = np.zeros_like(rec)
        b.get_positions_records(out, 64, 16)
    _close_f(f.ravel(), g["forces_f_total"])
    np.testing.assert_array_equal(out["x"], rec["x"])
    np.testing.assert_array_equal(out["z"], rec["z"])


def test_list_overflow_reports_code_5(golden600):
    from thecodecombo_7_gb300 import engine
    s = system_from_golden(golden600, 200)
    with _box(s, max_neighbors=16) as b:
        with pytest.raises(engine.FeError) as ei:
            b.nblist()
    assert ei.value.code == engine.FE_ERR_OVERFLOW


def test_forces_before_list_is_an_error(golden600):
    from thecodecombo_7_gb300 import engine
    s = system_from_golden(golden600, 200)
    with _box(s) as b:
        with pytest.raises(engine.FeError) as ei:
            b.forces()
    assert ei.value.code == engine.FE_ERR_STATE


def test_mc_delta_matches_oracle():
    from thecodecombo_7_gb300 import systems
    s = systems.water_box(300, L=26.0, seed=5, grid=(24, 24, 24))
    orc = O.Oracle(s)
    rng = np.random.default_rng(11)
    with _box(s) as b:
        b.mc_setup(kmax=5)
        ek0 = b.mc_kspace_energy()
        assert abs(ek0 - orc.ewald_kspace_energy(s.pos, 5, 25)) <= 1e-9 * abs(ek0)
        pos = s.pos.copy()
        for trial in range(6):
            m = int(rng.integers(0, 300))
            lb, ub = 3 * m, 3 * m + 3
            new = pos[lb:ub] + rng.uniform(-0.3, 0.3, size=3)
            new -= s.L * np.floor(new / s.L + 0.5)
            de, parts = b.mc_delta(lb, ub, new)
            pn = pos.copy()
            pn[lb:ub] = new
            want, wparts = orc.mc_delta_energy(pos, pn, lb, ub, kmax=5, max_k_square=25)
            assert abs(de - want) <= 1e-8 * max(1.0, abs(want)), (de, want)
            np.testing.assert_allclose(parts, wparts, rtol=1e-8, atol=1e-8)
            if trial % 2 == 0:
                b.mc_accept()
                pos = pn
        ek = b.mc_kspace_energy()
        assert abs(ek - orc.ewald_kspace_energy(pos, 5, 25)) <= 1e-9 * abs(ek)


def test_fp64_switch_matches_oracle():
    """The FP64 pair kernel with the LJ switch (8 -> 10 A) against the
    oracle's switched pair term (itself checked by finite differences and
    continuity in tests/test_switch_cpu.py)."""
    from thecodecombo_7_gb300 import systems
    s = systems.water_box(1365, density=0.1, seed=9, r_switch=8.0)
    o = O.Oracle(s)
    f_ref, en_ref = o.forces(s.pos)
    with _box(s) as b:
        b.nblist()
        en = b.forces()
        f = b.get_forces()
    _close_f(f, f_ref)
    for k in ("nbond", "nbonds", "rewald", "kewald", "iewald", "tewald"):
        _close_e(en[k], en_ref[k], k)
    assert en["nbonds"] == en["nbond"]  # no shift term under the switch


def test_mc_delta_with_switch_matches_oracle():
    from thecodecombo_7_gb300 import systems
    s = systems.water_box(300, L=26.0, seed=6, grid=(24, 24, 24), r_switch=8.0)
    orc = O.Oracle(s)
    rng = np.random.default_rng(12)
    with _box(s) as b:
        b.mc_setup(kmax=5)
        for trial in range(6):
            m = int(rng.integers(0, 300))
            lb, ub = 3 * m, 3 * m + 3
            new = s.pos[lb:ub] + rng.uniform(-0.3, 0.3, size=3)
            new -= s.L * np.floor(new / s.L + 0.5)
            de, parts = b.mc_delta(lb, ub, new)
            pn = s.pos.copy()
            pn[lb:ub] = new
            want, wparts = orc.mc_delta_energy(s.pos, pn, lb, ub, kmax=5, max_k_square=25)
            assert abs(de - want) <= 1e-8 * max(1.0, abs(want)), (de, want)
            np.testing.assert_allclose(parts, wparts, rtol=1e-8, atol=1e-8)


def test_mc_delta_matches_reference_fixture(golden_mc):
    """fe_mc_delta (the drop-in's forces_mc energy change) against the
    reference's own -DMC enbnd_mc before and after the same trial moves
    (tests/golden/mc.npz): every part on the cluster box, where no pair
    needs an image; k-space and LJ on the periodic box (the reference's
    real space there carries its minimum-image slip, ewald_mc.c:432-437)."""
    from tests.helpers import mc_case, mc_reference_parts
    for which in ("clu", "per"):
        s, kmax, mks, moves, e = mc_case(golden_mc, which)
        want = mc_reference_parts(e)
        with _box(s) as b:
            b.mc_setup(kmax=kmax, max_k_square=mks)
            assert abs(b.mc_kspace_energy() - e[0, 4]) <= 1e-10 * abs(e[0, 4])
            for (lb, ub, new), w in zip(moves, want):
                de, parts = b.mc_delta(lb, ub, new)
                cols = [0, 1, 2] if which == "clu" else [0, 2]
                np.testing.assert_allclose(parts[cols], w[cols], rtol=1e-9, atol=1e-9)


def test_pme_force_alone(golden600):
    """pme_force (pme_calc.c:122) after pme_calc: the same reciprocal forces
    from the grid pme_calc left, which are the reference's own f_pme."""
    g = golden600
    s = system_from_golden(g, 200)
    with _box(s) as b:
        b.zero_forces()
        b.pme_calc()
        f1 = b.get_forces()
        b.zero_forces()
        b.pme_force()
        f2 = b.get_forces()
    assert np.array_equal(f1, f2)
    _close_f(f2.ravel(), g["forces_f_pme"])



def test_bgo_pair_form_vs_reference(golden_bgo600):
    """The pair loop's BGO form (fe_box_set_lj_form 2) against the
    reference's own -DBGO build (tests/golden/bgo600.npz): forces and every
    energy term to 1e-10."""
    g = golden_bgo600
    s = system_from_golden(g, 200)
    with _box(s) as b:
        b.set_lj_form(2)
        b.nblist()
        en = b.forces()
        f = b.get_forces()
    _close_f(f.ravel(), g["forces_f_total"])
    ref = dict(zip(O.EN_KEYS, g["forces_en"]))
    for k in ("bond", "bend", "nbond", "nbonds", "coulomb", "rewald", "rewalds", "kewald",
              "sewald", "iewald", "tewald"):
        _close_e(en[k], ref[k])


def _slab_box(n_mol, Lxyz, seed):
    """Whole molecules of a cubic water box cut to an orthorhombic box, with a
    1.5 A gap left at every face (no close contacts across the new faces),
    then four molecules moved so that one site sits exactly on -L/2 of each
    axis (and one on -L/2 of all three): the wrap edges of the cell walk."""
    from thecodecombo_7_gb300 import systems
    Lxyz = np.asarray(Lxyz, dtype=float)
    s = systems.water_box(n_mol, density=0.1, seed=seed, L=float(Lxyz.max()))
    o = s.pos[0::3]
    keep = np.all(np.abs(o) < Lxyz / 2 - 1.5, axis=1)
    keep[:4] = True
    m = np.flatnonzero(keep)
    sites = (3 * m[:, None] + np.arange(3)).ravel()
    t = systems.water_box(len(m), density=0.1, seed=seed, L=float(Lxyz.max()))
    pos = s.pos[sites].copy()
    for k, axes in enumerate(([0], [1], [2], [0, 1, 2])):
        for a in axes:
            pos[3 * k:3 * k + 3, a] += -Lxyz[a] / 2 - pos[3 * k, a]
    pos -= Lxyz * np.floor(pos / Lxyz + 0.5)
    t.pos = pos
    t.L = Lxyz
    t.grid = (40, 48, 36)
    return t


@pytest.mark.parametrize("case", ["cubic_3cells", "orthorhombic_faces"])
def test_nblist_and_forces_on_larger_grids(case):
    """The golden boxes (L = 25 and 34.5 A, list radius 12 A) have two cells
    per axis; these boxes have three and more (9,000 sites, L = 44.8 A; and
    an orthorhombic 40 x 52 x 37 A box with sites exactly on -L/2): the pair
    lists bit-exact against the pinned oracle, forces and energies to 1e-10
    (the Coulomb total to 1e-10 of the Ewald terms it is summed from)."""
    from thecodecombo_7_gb300 import systems
    if case == "cubic_3cells":
        s = systems.water_box(3000, density=0.1, seed=31)
    else:
        s = _slab_box(2600, (40.0, 52.0, 37.0), seed=17)
    orc = O.Oracle(s)
    wcnt, widx, wflg = orc.nblist(s.pos)
    wf, wen = orc.forces(s.pos, (wcnt, widx, wflg))
    with _box(s) as b:
        b.nblist()
        cnt, idx, flg = b.nblist_download()
        en = b.forces()
        f = b.get_forces()
    np.testing.assert_array_equal(cnt, wcnt)
    np.testing.assert_array_equal(idx, widx)
    np.testing.assert_array_equal(flg, wflg)
    _close_f(f.ravel(), wf.ravel())
    for k in ("bond", "bend", "nbond", "nbonds", "rewald", "rewalds", "kewald", "sewald",
              "iewald"):
        _close_e(en[k], wen[k], k)
    # the Coulomb total is what is left of Ewald terms of 1e5-1e6 kJ/mol
    # that nearly cancel (-7 kJ/mol on the 9,000-site box): its bar scales
    # with the terms it is summed from
    parts = sum(abs(wen[k]) for k in ("rewald", "kewald", "sewald", "iewald"))
    for k in ("coulomb", "tewald"):
        assert abs(en[k] - wen[k]) <= ETOL * parts, (k, en[k], wen[k], parts)
