"""RESPA multiple time stepping on the FP64 engine (integrate_mts.c,
integrate_mts_nhc.c, force_short.c, force_long.c) against the reference's
own runs: the 900-site chain box (every bonded kind: bonds, bends and
Urey-Bradley terms fast; torsions, impropers and the non-bonded terms with
SPME slow; 6 long steps of 4 short steps) and the 600-site water box (8 long
steps of 4, plain and with the Nose-Hoover chain at either placement).

Bars as for the velocity-Verlet trajectories: energies of every long step to
1e-9 of their size, positions to 1e-10 A, velocities to 1e-8 A/ps, the
forces to 1e-9 of their scale (CUDA's acos/sin/cos against glibc's and the
order of the atomic force sums are the only differences)."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import chain_from_golden, system_from_golden

pytestmark = pytest.mark.gpu

ETOL = 1e-9


def _close_f(got, want, tol=1e-9):
    scale = np.abs(want).max()
    err = np.abs(got - want).max()
    assert err <= tol * scale, f"max force error {err:.3e} (scale {scale:.3e})"


def _run(s, g, nlong, nshort, xrespa=None):
    """nve_md.c:298-304 before the loop, then its RESPA branch (:400-418), or
    nvt_md.c's integrate_mts_nhc branch (:552) when xrespa is 0 or 1."""
    from thecodecombo_7_gb300 import engine
    rec = np.zeros((nlong + 1, 15))
    with engine.Box(s, precision=engine.FE_PREC_FP64) as b:
        b.nblist()
        b.force_short()
        b.force_long()
        en = b.forces()
        rec[0] = [b.kinet()[0]] + [en[k] for k in O.EN_KEYS[1:12]] + [
            en["urey"], en["tors"], en["impr"]]
        for i in range(1, nlong + 1):
            if i % s.nlist_freq == 0:
                b.nblist()
            en = (b.integrate_mts(nshort) if xrespa is None
                  else b.integrate_mts_nhc(nshort, xrespa))
            rec[i] = [b.kinet()[0]] + [en[k] for k in O.EN_KEYS[1:12]] + [
                en["urey"], en["tors"], en["impr"]]
        out = dict(rec=rec, pos=b.get_positions(), pos_nopbc=b.get_positions_nopbc(),
                   force=b.get_forces())
        out["vel"], out["uu"] = b.get_velocities()
        out["f_short"], out["f_long"] = b.forces_mts()
        out["zeta"] = b.get_nhc_state()
    return out


def _check(out, g, nlong, pre="mts_"):
    g = {k[len(pre):]: v for k, v in g.items() if k.startswith(pre)}
    want = g["en_steps"].reshape(-1, 15)
    assert want.shape[0] == nlong + 1
    keys = list(O.EN_KEYS[:12]) + ["urey", "tors", "impr"]
    for i in range(nlong + 1):
        for k in range(15):
            assert abs(out["rec"][i, k] - want[i, k]) <= ETOL * max(1.0, abs(want[i, k])), \
                (i, keys[k], out["rec"][i, k], want[i, k])
    np.testing.assert_allclose(out["pos"].ravel(), g["pos"], rtol=0, atol=1e-10)
    np.testing.assert_allclose(out["pos_nopbc"].ravel(), g["pos_nopbc"], rtol=0, atol=1e-10)
    np.testing.assert_allclose(out["vel"].ravel(), g["vel"], rtol=0, atol=1e-8)
    np.testing.assert_allclose(out["uu"].ravel(), g["vel_uu"], rtol=0, atol=1e-8)
    _close_f(out["force"].ravel(), g["force"])
    _close_f(out["f_short"].ravel(), g["f_short"])
    _close_f(out["f_long"].ravel(), g["f_long"])
    if "zeta" in g:
        z = g["zeta"].reshape(-1, 3)
        np.testing.assert_allclose(out["zeta"][:len(z)], z, rtol=1e-9, atol=1e-15)


def test_respa_chain_vs_reference(golden_chain):
    g = golden_chain
    _check(_run(chain_from_golden(g), g, 6, 4), g, 6)


def test_respa_water_vs_reference(golden_mts600):
    g = golden_mts600
    _check(_run(system_from_golden(g, 200), g, 8, 4), g, 8)


@pytest.mark.parametrize("xrespa", [0, 1])
def test_respa_nhc_water_vs_reference(golden_mts600, xrespa):
    """integrate_mts_nhc.c with the chain per long step (xRESPA 0) or per
    short step (xRESPA 1): trajectory, energies and the chain's state."""
    g = golden_mts600
    _check(_run(system_from_golden(g, 200), g, 8, 4, xrespa), g, 8, f"mtsnhc{xrespa}_")


def test_respa_one_short_step_is_velocity_verlet(golden600):
    """With one short step per long step RESPA is velocity Verlet on the sum
    of the two force classes: the same trajectory up to the rounding of the
    split kicks."""
    from thecodecombo_7_gb300 import engine
    s = system_from_golden(golden600, 200)
    out = []
    for mts in (True, False):
        with engine.Box(s, precision=engine.FE_PREC_FP64) as b:
            b.nblist()
            if mts:
                b.force_short()
                b.force_long()
            b.forces()
            for i in range(1, 9):
                if i % s.nlist_freq == 0:
                    b.nblist()
                en = b.integrate_mts(1) if mts else b.integrate_vverlet()
            out.append((b.get_positions(), b.get_velocities()[0], en))
    np.testing.assert_allclose(out[0][0], out[1][0], rtol=0, atol=1e-11)
    np.testing.assert_allclose(out[0][1], out[1][1], rtol=0, atol=1e-9)
    for k in ("bond", "bend", "nbond", "kewald", "rewald"):
        assert abs(out[0][2][k] - out[1][2][k]) <= 1e-9 * max(1.0, abs(out[1][2][k])), k


def test_respa_refused_on_mixed(golden600):
    from thecodecombo_7_gb300 import engine
    s = system_from_golden(golden600, 200)
    with engine.Box(s, precision=engine.FE_PREC_MIXED) as b:
        b.nblist()
        with pytest.raises(engine.FeError) as e:
            b.integrate_mts(4)
        assert e.value.code == engine.FE_ERR_STATE and "FP64" in str(e.value)
