"""Mixed-precision path (FP32 pair/PME math, 64-bit fixed-point force sums,
FP64 integration) against the FP64 CPU oracle.

Bars: relative rms force error <= 1e-5 (forces summed over all terms);
bitwise identical results on repeated evaluation (fixed-point sums are order
independent); energies per term, relative to the oracle's value of the same
term, ENERGY_BARS below: 1e-7 where FP32 pair math can reach it, and for the
terms it cannot, the measured level with its cause."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

RMS_TOL = 1e-5

# Relative error per energy term against the FP64 oracle at the seeded random
# starts of 4,095 and 12,000 sites (measured on a GB300: 4,095 / 12,000).
ENERGY_BARS = {
    "sewald": 1e-12,  # 0: set up once in FP64
    "iewald": 1e-9,   # < 2e-12: the correction energy is summed in double-float
    # nbond = LJ + real - intra + (reciprocal - self): 1.4e-6 / 8e-8; inherits
    # the real-space error below
    "nbond": 3e-6, "nbonds": 3e-6,
    # reciprocal: FP32 spline weights, grid and cuFFT transforms, 2.2e-7 /
    # 1.1e-7 (a sum of positive |S(k)|^2 terms: below 1e-7 needs FP64 FFTs)
    "kewald": 5e-7,
    # real space: 4.6e-6 / 7.9e-7.  The term is a net sum of ~1e6 pair energies
    # of both signs that cancel to ~1e-3 of their magnitudes; each FP32 pair
    # energy carries ~1e-7 of rounding, so the net carries ~1e-6 relative
    "rewald": 1e-5,
    # coulomb = real + reciprocal - self - intra, a net of 1e-3 of its parts:
    # 8.1e-6 / 2.2e-6 (the real-space error above over a smaller total)
    "coulomb": 2e-5, "tewald": 2e-5,
}


def _mixed(s):
    from thecodecombo_7_gb300 import engine
    return engine.Box(s, precision=engine.FE_PREC_MIXED)


def _rms_rel(got, want):
    return float(np.sqrt(((got - want) ** 2).sum() / (want ** 2).sum()))


@pytest.fixture(scope="module", params=[(1365, None), (4000, None)], ids=["4095", "12000"])
def case(request):
    from thecodecombo_7_gb300 import systems
    n_mol, _ = request.param
    s = systems.water_box(n_mol, density=0.1, seed=77 + n_mol)
    o = O.Oracle(s)
    f_ref, en_ref = o.forces(s.pos)
    return s, f_ref, en_ref


def test_mixed_force_error(case):
    s, f_ref, en_ref = case
    with _mixed(s) as b:
        b.nblist()
        en = b.forces()
        f = b.get_forces()
    err = _rms_rel(f, f_ref)
    assert err <= RMS_TOL, f"rms force error {err:.3e}"
    for k, bar in ENERGY_BARS.items():
        rel = abs(en[k] - en_ref[k]) / abs(en_ref[k])
        assert rel <= bar, (k, en[k], en_ref[k], rel)
    # bond and bend vanish at the rigid start (1e-22 in the oracle): absolute
    for k in ("bond", "bend"):
        assert abs(en[k] - en_ref[k]) <= 1e-6, (k, en[k], en_ref[k])


def test_mixed_bonded_energies_relative():
    """Bond and bend energies of a perturbed (non-rigid) geometry: sums of
    positive terms, within 1e-7 relative of the oracle (the stretch and the
    angle are formed in FP64 from the fixed-point coordinates, whose
    2e-8 A resolution is all that separates them from the oracle's)."""
    from thecodecombo_7_gb300 import systems
    s = systems.water_box(1365, density=0.1, seed=41)
    rng = np.random.default_rng(3)
    s.pos = s.pos + rng.normal(0.0, 0.03, s.pos.shape)
    s.pos -= s.L * np.floor(s.pos / s.L + 0.5)
    _, en_ref = O.Oracle(s).forces(s.pos)
    with _mixed(s) as b:
        b.nblist()
        en = b.forces()
    for k in ("bond", "bend"):
        assert abs(en[k] - en_ref[k]) <= 1e-7 * abs(en_ref[k]), (k, en[k], en_ref[k])


def test_mixed_bonded_energies_thermal():
    """Bond and bend energies of a thermalised box (400 NVE steps from the
    rigid start) against the FP64 oracle on the same coordinates: within
    1e-7, the energy bar (stretch and angle in FP64 from the fixed-point
    coordinates)."""
    from thecodecombo_7_gb300 import systems
    s = systems.water_box(1365, density=0.1, seed=43)
    with _mixed(s) as b:
        b.nblist()
        b.forces()
        b.kinet()
        b.run_md(400, nlist_freq=10, record=False)
        pos = b.get_positions()
        b.nblist()
        en = b.forces()
    _, en_ref = O.Oracle(s).forces(pos)
    for k in ("bond", "bend"):
        assert abs(en[k] - en_ref[k]) <= 1e-7 * abs(en_ref[k]), (k, en[k], en_ref[k])


def test_mixed_deterministic(case):
    s, _, _ = case
    with _mixed(s) as b:
        b.nblist()
        e1 = b.forces()
        f1 = b.get_forces()
        b.nblist()
        e2 = b.forces()
        f2 = b.get_forces()
    assert np.array_equal(f1, f2)
    assert e1 == e2


def test_mixed_trajectory_tracks_fp64():
    """20 NVE steps: the mixed trajectory stays within the FP32 error band of
    the FP64 oracle trajectory."""
    from thecodecombo_7_gb300 import systems
    s = systems.water_box(1365, density=0.1, seed=5)
    o = O.Oracle(s)
    md = o.run_md(20)
    with _mixed(s) as b:
        b.nblist()
        b.forces()
        b.kinet()
        rec = b.run_md(20)
        pos = b.get_positions()
    d = pos - md["pos"]
    d -= s.L * np.rint(d / s.L)
    assert np.abs(d).max() < 1e-4
    tot = rec[:, 0] + rec[:, 1] + rec[:, 2] + rec[:, 4]
    tot_ref = (md["en"][1:, 0] + md["en"][1:, 1] + md["en"][1:, 2] + md["en"][1:, 4])
    assert np.abs(tot - tot_ref).max() <= 1e-5 * np.abs(tot_ref).max()


def test_mixed_switch_matches_oracle():
    from thecodecombo_7_gb300 import systems
    s = systems.water_box(1365, density=0.1, seed=9, r_switch=8.0)
    o = O.Oracle(s)
    f_ref, en_ref = o.forces(s.pos)
    with _mixed(s) as b:
        b.nblist()
        en = b.forces()
        f = b.get_forces()
    assert _rms_rel(f, f_ref) <= RMS_TOL
    for k in ("nbond", "nbonds", "kewald", "iewald", "rewald"):
        rel = abs(en[k] - en_ref[k]) / abs(en_ref[k])
        assert rel <= ENERGY_BARS[k], (k, en[k], en_ref[k], rel)


def test_mixed_drift_matches_fp64():
    """NVE energy drift of the mixed-precision engine against the FP64 engine
    on the same start (4,095 sites, 2,000 steps after 500 of relaxation): the
    drift belongs to the force field and integrator (energy-shifted cutoff,
    relaxation of the random start), not to the FP32 arithmetic.  The two
    trajectories are chaotic and separate within a few hundred steps, so the
    fitted slopes carry fluctuations of order 15 % of their size: the bar is
    agreement within 25 %."""
    from thecodecombo_7_gb300 import engine, systems
    s = systems.water_box(1365, density=0.1, seed=2025)
    slopes = []
    for prec in (engine.FE_PREC_FP64, engine.FE_PREC_MIXED):
        with engine.Box(s, precision=prec) as b:
            b.nblist()
            b.forces()
            b.kinet()
            b.run_md(500, first_step=1, record=False)
            rec = b.run_md(2000, first_step=501, record=True)
        tot = rec[:, 0] + rec[:, 1] + rec[:, 2] + rec[:, 4]
        slopes.append(np.polyfit(np.arange(len(tot)) * s.dt, tot, 1)[0])
    kT = 1.380662e-23 * 6.022045e23 * s.T * 1e-3
    per_dof = [x * 1000.0 / (kT * (3 * s.n - 3)) for x in slopes]  # kT / ns / dof
    assert abs(per_dof[1] - per_dof[0]) <= 0.25 * max(abs(per_dof[0]), 0.05), per_dof


def test_autotune_keeps_results_bitwise(case):
    """Every launch shape gives the same fixed-point forces and energies."""
    s, _, _ = case
    with _mixed(s) as b:
        b.nblist()
        b.forces()  # prunes the inner list: the calls below walk it
        e1 = b.forces()
        f1 = b.get_forces()
        nw, regs, blocks, us = b.autotune()
        e2 = b.forces()
        f2 = b.get_forces()
    assert nw in (4, 8, 16) and regs in (40, 64) and blocks > 0 and us > 0
    assert np.array_equal(f1, f2)
    assert e1 == e2


def _exact_row_counts(s, rl):
    """Per-site count of non-excluded partners within rl, from the same
    32-bit fractional coordinates the engine lists from (minimum image)."""
    L = np.asarray(s.L, float)
    u = np.rint((s.pos / L + 0.5) * 2.0 ** 32).astype(np.int64) & 0xFFFFFFFF
    n = s.n
    cnt = np.zeros(n, np.int64)
    near = 0
    for a in range(0, n, 512):
        d = u[a:a + 512, None, :] - u[None, :, :]
        d = ((d + 2 ** 31) & 0xFFFFFFFF) - 2 ** 31
        r2 = ((d * (L / 2.0 ** 32)) ** 2).sum(-1)
        inside = r2 < rl * rl
        inside[np.arange(inside.shape[0]), np.arange(a, a + inside.shape[0])] = False
        cnt[a:a + 512] = inside.sum(1)
        near += int((np.abs(np.sqrt(r2) - rl) < 1e-4).sum())
    for i, j in np.asarray(s.excl).reshape(-1, 2):
        d = ((u[i] - u[j] + 2 ** 31) & 0xFFFFFFFF) - 2 ** 31
        if ((d * (L / 2.0 ** 32)) ** 2).sum() < rl * rl:
            cnt[i] -= 1
            cnt[j] -= 1
    return cnt, near


@pytest.mark.parametrize("kind", ["water12000", "water900_small_box", "ortho_3000"])
def test_mixed_list_is_complete(kind):
    """The outer list holds exactly the non-excluded pairs within rlist
    (both directions): total entries and the longest row against an exact
    count, up to pairs within 1e-4 A of rlist."""
    from thecodecombo_7_gb300 import systems
    if kind == "water12000":
        s = systems.water_box(4000, density=0.1, seed=11)
    elif kind == "water900_small_box":
        s = systems.water_box(300, density=0.1, seed=5, grid=(16, 16, 16))
        s.rc = s.rc_ew = 8.0
        s.rclist = s.rclist_ew = 9.0
    else:
        s = systems.water_box(1000, density=0.1, seed=9)
        rng = np.random.default_rng(2)
        s.L = np.array([30.0, 42.0, 26.0])
        s.pos = (rng.random((s.n, 3)) - 0.5) * s.L
        s.pos[:5, 0] = s.L[0] / 2
        s.pos[5:10, 1] = -s.L[1] / 2
        s.grid = (32, 40, 24)
        s.rc = s.rc_ew = 11.0
        s.rclist = s.rclist_ew = 12.5
    rl = min(s.rclist, s.rclist_ew)
    want, near = _exact_row_counts(s, rl)
    with _mixed(s) as b:
        b.nblist()
        entries, max_row = b.list_stats()
    assert abs(entries - int(want.sum())) <= 2 * near, (entries, int(want.sum()), near)
    assert abs(max_row - int(want.max())) <= (1 if near else 0), (max_row, int(want.max()))


def test_inner_list_pruning():
    """The pair kernel walks an inner list (rc + 0.8 A) between prunes: it is
    pruned after a list rebuild, kept while displacements stay under 0.4 A,
    re-pruned on the device when a site moves further, and forces from the
    inner list agree with a walk of the outer list at the same positions to
    FP32 summation order."""
    from thecodecombo_7_gb300 import systems
    s = systems.water_box(4000, density=0.1, seed=21)
    with _mixed(s) as b:
        b.nblist()
        b.forces()
        e0, m0, p0 = b.inner_list_stats()
        want, near = _exact_row_counts(s, s.rc + 0.8)
        assert abs(e0 - int(want.sum())) <= 2 * near, (e0, int(want.sum()))
        assert abs(m0 - int(want.max())) <= (1 if near else 0)
        b.run_md(5, nlist_freq=1000, first_step=1, record=False)
        _, _, p1 = b.inner_list_stats()
        assert p1 == p0, "no prune expected for small displacements"
        f_step = b.get_forces()
        b.forces()
        assert np.array_equal(b.get_forces(), f_step)
        b.nblist()
        b.forces()  # after a rebuild: walks the outer list
        _, _, p2 = b.inner_list_stats()
        assert p2 == p1 + 1
        assert _rms_rel(f_step, b.get_forces()) < 1e-6
        pos = b.get_positions()
        pos[0, 0] += 0.45
        b.set_positions(pos)
        b.run_md(1, nlist_freq=1000, first_step=100, record=False)
        _, _, p3 = b.inner_list_stats()
        assert p3 == p2 + 1, "a 0.45 A displacement must trigger a prune"


@pytest.mark.parametrize("grid", [(8, 8, 8), (10, 12, 9), (20, 18, 12)],
                         ids=["8^3", "10x12x9", "20x18x12"])
def test_mixed_spme_small_and_ragged_grids(grid):
    """Spreading (fixed-point reductions with periodic wrap of the spline
    points) and gathering on a grid of a few points per axis and on odd
    grid sizes: forces and the reciprocal energy against the FP64 oracle."""
    from thecodecombo_7_gb300 import systems
    if grid == (8, 8, 8):
        s = systems.water_box(50, L=18.5, seed=5, grid=grid)
    elif grid == (10, 12, 9):
        s = systems.water_box(100, L=18.5, seed=5, grid=grid)
    else:
        s = systems.water_box(300, density=0.1, seed=5, grid=grid)
    s.rc = s.rc_ew = 8.0
    s.rclist = s.rclist_ew = 9.0
    f_ref, en_ref = O.Oracle(s).forces(s.pos)
    with _mixed(s) as b:
        b.nblist()
        en = b.forces()
        f = b.get_forces()
    err = _rms_rel(f, f_ref)
    assert err <= RMS_TOL, f"rms force error {err:.3e}"
    assert abs(en["kewald"] - en_ref["kewald"]) <= 2e-6 * abs(en_ref["sewald"])


@pytest.mark.parametrize("order", [3, 4, 6])
def test_mixed_spline_orders(order):
    """Order 4 computes its spline weights inside spreading and gathering;
    other orders store them in a separate pass first: both against the FP64
    oracle at the same order."""
    from thecodecombo_7_gb300 import systems
    s = systems.water_box(600, density=0.1, seed=11, order=order)
    f_ref, en_ref = O.Oracle(s).forces(s.pos)
    with _mixed(s) as b:
        b.nblist()
        en = b.forces()
        f = b.get_forces()
    err = _rms_rel(f, f_ref)
    assert err <= RMS_TOL, f"rms force error {err:.3e}"
    assert abs(en["kewald"] - en_ref["kewald"]) <= 5e-7 * abs(en_ref["kewald"]) + 1e-9 * abs(
        en_ref["sewald"])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_nl_check_matches_oracle(precision):
    """fe_nl_check against the oracle's restatement of nl_check after moves
    below, at and above (rclist - rc)/4, including a site moved across the
    periodic boundary and a restricted site range."""
    from thecodecombo_7_gb300 import engine, systems
    s = systems.water_box(300, density=0.1, seed=4)
    s.rc = s.rc_ew = 8.0  # mixed precision needs rclist < L/2 (L = 20.8 A)
    s.rclist = s.rclist_ew = 9.0
    prec = engine.FE_PREC_FP64 if precision == "fp64" else engine.FE_PREC_MIXED
    with engine.Box(s, precision=prec) as b:
        b.nblist()
        p0 = b.get_positions()
        rng = np.random.default_rng(3)
        rcut = (s.rclist - s.rc) / 4.0
        cases = []
        for amp in (0.2 * rcut, 0.55 * rcut, 0.95 * rcut, 1.05 * rcut):
            d = np.zeros_like(p0)
            d[rng.integers(0, s.n, 5)] = rng.normal(size=(5, 3)) * amp / np.sqrt(3)
            cases.append(d)
        far = np.zeros_like(p0)
        far[s.n - 1, 2] = 1.2 * rcut  # a site past the threshold, outside [0, n/2)
        cases.append(far)
        edge = np.zeros_like(p0)
        k = int(np.argmax(p0[:, 0]))
        edge[k, 0] = s.L[0] / 2 - p0[k, 0] + 0.3 * rcut  # crosses +L/2, wraps
        cases.append(edge)
        got, want = [], []
        for d in cases:
            b.set_positions(p0 + d)
            p = b.get_positions()
            for lb, ub in ((0, s.n), (0, s.n // 2)):
                got.append(b.nl_check(lb, ub))
                want.append(O.nl_check(p, p0, s.L, s.rclist, s.rc, lb, ub))
        assert got == want
        assert 0 in want and 1 in want
