"""Go-model chain workload without a GPU: the generated chains and the
oracle's forces (finite differences) and Langevin integrator."""
import numpy as np

from oracle import oracle as O
from thecodecombo_7_gb300 import systems


def _small(n_rep=3, seed=5):
    return systems.go_chains(n_rep, nmin=40, nmax=90, seed=seed)


def test_go_chains_shapes():
    g = _small()
    st = g.start
    assert len(g.nbeads) == 3 and np.all((g.nbeads >= 40) & (g.nbeads <= 90))
    assert g.pos.shape == (st[-1], 3) and g.nat_start[-1] == len(g.nat_j)
    assert np.all(g.T[1:] > g.T[:-1]) and abs(g.T[0] - 280) < 1e-9 and abs(g.T[-1] - 450) < 1e-9
    pairs = set()
    for i in range(st[-1]):
        r = np.searchsorted(st, i, side="right") - 1
        for q in range(g.nat_start[i], g.nat_start[i + 1]):
            j = g.nat_j[q]
            assert st[r] <= j < st[r + 1] and abs(i - j) >= 4
            d = np.linalg.norm(g.pos[i] - g.pos[j])
            assert abs(d - g.nat_r0[q]) < 1e-12 and d < 6.5
            pairs.add((i, j))
    assert all((j, i) in pairs for i, j in pairs)  # symmetric
    for r in range(3):
        b = np.linalg.norm(np.diff(g.pos[st[r]:st[r + 1]], axis=0), axis=1)
        assert np.all(np.abs(b - 3.8) < 0.9)
        # self-avoiding: no two beads closer than the lattice minus the jitter
        x = g.pos[st[r]:st[r + 1]]
        d = np.sqrt(((x[:, None] - x[None]) ** 2).sum(-1)) + np.eye(len(x)) * 99
        assert d.min() > 3.8 - 2 * np.sqrt(3) * 0.25


def test_go_oracle_forces_are_energy_gradient():
    g = _small()
    x = g.pos[:g.nbeads[0]].copy()
    x += np.random.default_rng(1).normal(0, 0.1, x.shape)
    f, e = O.go_forces(g, 0, x)
    rng = np.random.default_rng(2)
    for _ in range(20):
        i, a = rng.integers(len(x)), rng.integers(3)
        h = 1e-6
        xp, xm = x.copy(), x.copy()
        xp[i, a] += h
        xm[i, a] -= h
        fd = -(O.go_forces(g, 0, xp)[1] - O.go_forces(g, 0, xm)[1]) / (2 * h)
        assert abs(fd - f[i, a]) <= 1e-5 * max(1.0, abs(fd)), (i, a, fd, f[i, a])


def test_go_oracle_verlet_limit_is_second_order():
    """gamma = 0 turns BAOAB into velocity Verlet: the energy error over a
    fixed time falls as dt^2."""
    g = _small()
    g.gamma = 0.0

    def ke(v):
        return 0.5 * g.mass * (v ** 2).sum() / 100.0  # amu A^2/ps^2 -> kJ/mol

    v0 = g.vel[g.start[1]:g.start[2]]
    errs = []
    for dt in (0.002, 0.001):
        g.dt = dt
        e0 = O.go_baoab(g, 1, 0, seed=1)[2] + ke(v0)
        x, v, e1 = O.go_baoab(g, 1, int(round(0.2 / dt)), seed=1)
        errs.append(abs(e1 + ke(v) - e0))
    assert errs[1] < errs[0] / 3.0, errs


def test_reference_go_model_pinned(golden_go_hc):
    """The restatement of the reference's own Go model (or_go_hc_term:
    cbb_golik, cba_golik, cda_golik, cnbnd_golik of cgolik.c) against the
    reference's routines run on the same chains (tests/golden/go_hc.npz):
    forces and energies of every term bit for bit."""
    from oracle import oracle as O
    from tests.helpers import go_from_golden
    g = golden_go_hc
    chains, pos, hc = go_from_golden(g)
    for r in range(len(chains.nbeads)):
        a, b = int(chains.start[r]), int(chains.start[r + 1])
        mine = O.go_hc_terms(chains, r, hc, pos=pos[a:b])
        for name in ("bond", "bend", "tors", "nb"):
            np.testing.assert_array_equal(mine["f_" + name].ravel(), g[f"r{r}_f_{name}"])
        en = g[f"r{r}_en"]
        assert mine["e_bond"] == en[0] and mine["e_bend"] == en[1] and mine["e_tors"] == en[2]
        assert mine["e_nb2"][0] == en[3] and mine["e_nb2"][1] == en[4]
        assert np.abs(g[f"r{r}_f_bond"]).max() > 0 and np.abs(g[f"r{r}_f_bend"]).max() > 0
