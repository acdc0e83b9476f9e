"""Cross-checks that lean on no reference output, only on physics:
  - the FP64 forces are minus the gradient of the engine's own potential
    energy (central finite differences of bond + bend + nbond + the extra
    bonded terms, every term at once; water with and without the LJ switch,
    and the chain box with every bonded kind);
  - the net force of the box vanishes (Newton's third law; the reciprocal
    mean force is removed as pme_calc.c does), in both precisions;
  - SPME's reciprocal energy converges to the classic Ewald k-space sum of
    the Monte Carlo path (two independent implementations in the engine).

Bars: gradients to 1e-5 of the atom's force (h = 1e-5 A) once the vector
they all share is taken off: the reciprocal mean force that pme_calc.c
removes from every atom is no part of the energy's gradient (it is checked
to stay below 1e-4 of the largest force); net force below 1e-9 (FP64)
and 1e-5 (mixed: FP32 row sums) of the largest atomic force; SPME at order
8 on a 1.9 points/A grid against the classic sum at |n| <= 12 to 2e-6.
Finite differences of the mixed precision's energy are not taken: pairs
that cross rc within a step of the size its FP32 rounding needs change the
unshifted energy by more than the bar."""
import numpy as np
import pytest

from tests.helpers import chain_from_golden, system_from_golden

pytestmark = pytest.mark.gpu


def _potential(en):
    return (en["bond"] + en["bend"] + en["nbond"] + en["urey"] + en["tors"] + en["impr"])


def _energy_at(b, pos):
    b.set_positions(pos)
    return _potential(b.forces())


@pytest.mark.parametrize("kind", ["water", "water_switched", "chain"])
def test_forces_are_energy_gradients(golden600, golden_chain, kind):
    from thecodecombo_7_gb300 import engine, systems
    h, tol = 1e-5, 1e-5
    if kind == "water":
        s = system_from_golden(golden600, 200)
    elif kind == "water_switched":
        s = systems.water_box(200, L=25.0, seed=9, grid=(24, 25, 27), r_switch=8.0)
    else:
        s = chain_from_golden(golden_chain)
    rng = np.random.default_rng(7)
    atoms = rng.choice(s.n, 6, replace=False)
    d = []
    with engine.Box(s, precision=engine.FE_PREC_FP64) as b:
        b.nblist()  # the list of the base configuration covers every displaced one
        b.forces()
        f0 = b.get_forces()
        for a in atoms:
            g = np.zeros(3)
            for c in range(3):
                x = s.pos.copy()
                x[a, c] += h
                ep = _energy_at(b, x)
                x[a, c] -= 2 * h
                em = _energy_at(b, x)
                g[c] = -(ep - em) / (2 * h)
            d.append(g - f0[a])
    # every atom's gradient exceeds its force by the same vector: the mean
    # reciprocal force that pme_calc.c takes off every atom (SPME's small
    # net force), which is no part of the energy's gradient
    d = np.array(d)
    off = d.mean(axis=0)
    fmax = np.abs(f0).max()
    assert np.linalg.norm(off) <= 1e-4 * fmax, off
    for k, a in enumerate(atoms):
        scale = max(np.linalg.norm(f0[a]), 1.0)
        assert np.linalg.norm(d[k] - off) <= tol * scale, (a, d[k], off, f0[a])


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-9), ("mixed", 1e-5)])
def test_net_force_vanishes(golden600, golden_chain, prec, tol):
    from thecodecombo_7_gb300 import engine
    p = engine.FE_PREC_FP64 if prec == "fp64" else engine.FE_PREC_MIXED
    for s in (system_from_golden(golden600, 200), chain_from_golden(golden_chain)):
        with engine.Box(s, precision=p) as b:
            b.nblist()
            b.forces()
            f = b.get_forces()
        assert np.abs(f.sum(axis=0)).max() <= tol * np.abs(f).max(), f.sum(axis=0)


def test_spme_converges_to_classic_ewald():
    from thecodecombo_7_gb300 import engine, systems
    s = systems.water_box(200, L=25.0, seed=7, grid=(48, 48, 48), order=8)
    with engine.Box(s, precision=engine.FE_PREC_FP64) as b:
        b.nblist()
        en = b.forces()
        b.mc_setup(kmax=12)
        classic = b.mc_kspace_energy()
    assert abs(en["kewald"] - classic) <= 2e-6 * abs(classic), (en["kewald"], classic)
