"""Urey-Bradley, proper and improper torsions on the device (curey.c,
ctorsion.c, cimproper.c) against the reference's own outputs for the 900-site
chain box (tests/golden/chain900.npz): every bonded term of forces(), 1-4
pairs, torsion series that stop at a zero term.

Bars: FP64 drop-in forces and energies to 1e-10 of their scale (CUDA's acos,
sin and cos against glibc's, and the order of the atomic force sums); the
torsion angles to 1e-12 rad; the mixed precision's forces to 1e-5 rms of the
FP64 forces (its pair and PME math is FP32) and its extra bonded energies to
1e-10 (they are computed in FP64 there too, summed exactly in fixed point)."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import chain_from_golden

pytestmark = pytest.mark.gpu

FTOL = 1e-10
ETOL = 1e-10


def _box(s, precision):
    from thecodecombo_7_gb300 import engine
    return engine.Box(s, precision=precision)


def _close_f(got, want, tol=FTOL):
    scale = np.abs(want).max()
    err = np.abs(got - want).max()
    assert err <= tol * scale, f"max force error {err:.3e} (scale {scale:.3e})"


def _close_e(got, want, key=""):
    assert abs(got - want) <= ETOL * max(1.0, abs(want)), f"{key}: {got!r} vs {want!r}"


def test_ext_terms_alone_fp64(golden_chain):
    from thecodecombo_7_gb300 import engine
    g = golden_chain
    s = chain_from_golden(g)
    with _box(s, engine.FE_PREC_FP64) as b:
        b.zero_forces()
        e3 = b.bonded_ext()
        f = b.get_forces()
        tau = b.torsion_angles()
    want = g["forces_f_urey"] + g["forces_f_tors"] + g["forces_f_impr"]
    _close_f(f.ravel(), want)
    for k, name in enumerate(("urey", "tors", "impr")):
        _close_e(e3[k], g["forces_e_ext"][k], name)
    np.testing.assert_allclose(tau, g["forces_tau"], rtol=0, atol=1e-12)


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_chain_forces_vs_reference(golden_chain, prec):
    """The full forces() of the chain box: every term at once."""
    from thecodecombo_7_gb300 import engine
    g = golden_chain
    s = chain_from_golden(g)
    p = engine.FE_PREC_FP64 if prec == "fp64" else engine.FE_PREC_MIXED
    with _box(s, p) as b:
        b.nblist()
        en = b.forces()
        f = b.get_forces()
        tau = b.torsion_angles()
    want = g["forces_f_total"]
    ref = dict(zip(O.EN_KEYS, g["forces_en"]))
    for k, name in enumerate(("urey", "tors", "impr")):
        _close_e(en[name], g["forces_en_ext"][k], name)
    np.testing.assert_allclose(tau, g["forces_tau"], rtol=0, atol=1e-12)
    if prec == "fp64":
        _close_f(f.ravel(), want)
        for k in ("bond", "bend", "nbond", "nbonds", "coulomb", "rewald", "rewalds", "kewald",
                  "sewald", "iewald", "tewald"):
            _close_e(en[k], ref[k], k)
    else:
        d = f.ravel() - want
        rms = np.sqrt((d * d).mean() / (want * want).mean())
        assert rms < 1e-5, rms
        for k in ("bond", "bend"):
            assert abs(en[k] - ref[k]) <= 1e-6 * max(1.0, abs(ref[k])), (k, en[k], ref[k])


def test_chain_trajectory_fp64(golden_chain):
    """12 NVE steps with every bonded term: positions, velocities, forces and
    the energy record against the reference's own run."""
    from thecodecombo_7_gb300 import engine
    g = golden_chain
    s = chain_from_golden(g)
    with _box(s, engine.FE_PREC_FP64) as b:
        b.nblist()
        b.forces()
        b.kinet()
        rec = b.run_md(12, nlist_freq=s.nlist_freq, use_nhc=False)
        pos = b.get_positions()
        vel, _ = b.get_velocities()
        f = b.get_forces()
    want = g["nve_en_steps"].reshape(-1, 12)[1:]
    for i in range(12):
        for k in range(12):
            assert abs(rec[i, k] - want[i, k]) <= 1e-9 * max(1.0, abs(want[i, k])), \
                (i, O.EN_KEYS[k], rec[i, k], want[i, k])
    np.testing.assert_allclose(pos.ravel(), g["nve_pos"], rtol=0, atol=1e-10)
    np.testing.assert_allclose(vel.ravel(), g["nve_vel"], rtol=0, atol=1e-8)
    _close_f(f.ravel(), g["nve_force"], 1e-9)


def test_ext_terms_replace_and_clear(golden_chain):
    """Each fe_set_* call replaces that kind of term; an empty set removes it
    and its energy, and the step graphs are recaptured."""
    from thecodecombo_7_gb300 import engine
    g = golden_chain
    s = chain_from_golden(g)
    with _box(s, engine.FE_PREC_FP64) as b:
        b.nblist()
        b.forces()
        b.kinet()
        b.run_md(2, nlist_freq=s.nlist_freq)
        s2 = s.copy()
        s2.tors = np.zeros((0, 4), np.int32)
        s2.tors_kphi = s2.tors_nphi = s2.tors_delphi = np.zeros((0, 6))
        b.set_ext_bonded(s2)
        en = b.forces()
        assert en["tors"] == 0.0 and en["impr"] != 0.0 and en["urey"] != 0.0
        rec = b.run_md(2, nlist_freq=s.nlist_freq)
        assert np.all(rec[:, 13] == 0.0) and np.all(rec[:, 14] != 0.0)
