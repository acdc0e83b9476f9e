"""Batched Go-model replicas on the device against the oracle: FP32 forces
and energies, BAOAB trajectories with the same Philox draws, the exchange
decisions, and reproducibility."""
import numpy as np
import pytest

from oracle import oracle as O
from thecodecombo_7_gb300 import replicas

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def chains():
    from thecodecombo_7_gb300 import systems
    return systems.go_chains(6, nmin=60, nmax=300, seed=77)


def test_go_forces_match_oracle(chains):
    from thecodecombo_7_gb300 import engine
    g = chains
    b = engine.GoBatch(g, seed=1)
    try:
        f, e = b.forces()
    finally:
        b.close()
    st = g.start
    for r in range(len(g.nbeads)):
        fr, er = O.go_forces(g, r)
        fg = f[st[r]:st[r + 1]]
        rms = np.sqrt(((fg - fr) ** 2).sum() / (fr ** 2).sum())
        assert rms <= 1e-5, (r, rms)
        assert abs(e[r] - er) <= 1e-5 * g.eps * g.nbeads[r], (r, e[r], er)


def test_go_trajectory_matches_oracle(chains):
    from thecodecombo_7_gb300 import engine
    g = chains
    b = engine.GoBatch(g, seed=11)
    try:
        b.run(25)
        s = b.state()
    finally:
        b.close()
    assert s["steps"] == 25
    st = g.start
    for r in range(len(g.nbeads)):
        x, v, e = O.go_baoab(g, r, 25, seed=11)
        assert np.abs(s["pos"][st[r]:st[r + 1]] - x).max() < 1e-4, r
        assert np.abs(s["vel"][st[r]:st[r + 1]] - v).max() < 1e-2, r
        assert abs(s["epot"][r] - e) <= 1e-4 * g.eps * g.nbeads[r]


def test_go_exchange_decisions(chains):
    from thecodecombo_7_gb300 import engine
    g = chains
    seed = 5
    b = engine.GoBatch(g, seed=seed)
    try:
        slot = np.arange(len(g.nbeads), dtype=np.int32)
        for a in range(4):
            b.run(10, swap_freq=10)
            s = b.state()
            slot, vmode, vfac = replicas.exchange_decision(g.T, s["epot"], slot, a, seed)
            assert np.array_equal(s["slot_rep"], slot), (a, s["slot_rep"], slot)
            for q in range(len(slot)):
                assert s["T"][slot[q]] == g.T[q]
        assert s["steps"] == 40 and int(s["attempted"].sum()) > 0
    finally:
        b.close()


def test_go_reproducible(chains):
    from thecodecombo_7_gb300 import engine
    out = []
    for _ in range(2):
        b = engine.GoBatch(chains, seed=3)
        try:
            b.run(30, swap_freq=10)
            out.append(b.state())
        finally:
            b.close()
    assert np.array_equal(out[0]["pos"], out[1]["pos"])
    assert np.array_equal(out[0]["slot_rep"], out[1]["slot_rep"])


def test_go_split_plan_and_forces():
    """48 chains of 20-120 beads: the plan mixes chains on one CTA with chains
    split over several CTAs of a cluster; every kind matches the oracle's
    forces and a short trajectory."""
    from thecodecombo_7_gb300 import engine, systems
    g = systems.go_chains(48, nmin=20, nmax=120, seed=19)
    b = engine.GoBatch(g, seed=2)
    try:
        lay = b.layout()
        f, e = b.forces()
        b.run(10)
        s = b.state()
    finally:
        b.close()
    parts = lay["parts"]
    assert lay["ncta"] % 4 == 0 and parts.sum() <= lay["ncta"]
    assert set(parts.tolist()) <= {1, 2, 3, 4}
    assert len(set(parts.tolist())) > 1, parts
    assert lay["ncta"] <= lay["slots"] or parts.max() == 1
    st = g.start
    for r in range(len(g.nbeads)):
        fr, er = O.go_forces(g, r)
        fg = f[st[r]:st[r + 1]]
        rms = np.sqrt(((fg - fr) ** 2).sum() / (fr ** 2).sum())
        assert rms <= 1e-5, (r, parts[r], rms)
        assert abs(e[r] - er) <= 1e-5 * g.eps * g.nbeads[r], (r, parts[r], e[r], er)
        x, v, eo = O.go_baoab(g, r, 10, seed=2)
        assert np.abs(s["pos"][st[r]:st[r + 1]] - x).max() < 1e-4, (r, parts[r])
        assert np.abs(s["vel"][st[r]:st[r + 1]] - v).max() < 1e-2, (r, parts[r])


@pytest.mark.parametrize("nrep,nb", [(1, 1024), (3, 2), (2, 5)])
def test_go_extreme_chain_lengths(nrep, nb):
    """The limits of the batch: one chain of the maximum 1,024 beads (split
    over the CTAs of a cluster, the largest shared-memory rows), chains of two
    beads (a bond and nothing else) and of five (one non-native pair)."""
    from thecodecombo_7_gb300 import engine, systems
    g = systems.go_chains(nrep, nmin=nb, nmax=nb, seed=23)
    b = engine.GoBatch(g, seed=4)
    try:
        f, e = b.forces()
        b.run(10)
        s = b.state()
    finally:
        b.close()
    st = g.start
    for r in range(nrep):
        fr, er = O.go_forces(g, r)
        fg = f[st[r]:st[r + 1]]
        scale = np.sqrt((fr ** 2).sum())
        assert np.sqrt(((fg - fr) ** 2).sum()) <= 1e-5 * max(scale, 1e-3), r
        assert abs(e[r] - er) <= 1e-5 * g.eps * max(g.nbeads[r], 10), (r, e[r], er)
        x, v, eo = O.go_baoab(g, r, 10, seed=4)
        assert np.abs(s["pos"][st[r]:st[r + 1]] - x).max() < 1e-4, r
        assert np.abs(s["vel"][st[r]:st[r + 1]] - v).max() < 1e-2, r



def test_reference_form_vs_reference(golden_go_hc):
    """The reference's own Go model on the device (fe_go_set_reference_form)
    against the reference's cgolik.c routines run on the same chains at the
    same perturbed coordinates (tests/golden/go_hc.npz): forces (FP32) to
    1e-5 rms, energy to 1e-5."""
    import dataclasses
    from thecodecombo_7_gb300 import engine
    from tests.helpers import go_from_golden
    g = golden_go_hc
    chains, pos, hc = go_from_golden(g)
    moved = dataclasses.replace(chains, pos=pos)
    b = engine.GoBatch(moved, seed=1)
    try:
        b.set_reference_form(d_rep=hc[1], rc=hc[2], native=chains.pos)
        f, e = b.forces()
    finally:
        b.close()
    st = chains.start
    for r in range(len(chains.nbeads)):
        want = sum(g[f"r{r}_f_{t}"] for t in ("bond", "bend", "tors", "nb")).reshape(-1, 3)
        got = f[st[r]:st[r + 1]]
        rms = np.sqrt(((got - want) ** 2).sum() / (want ** 2).sum())
        assert rms <= 1e-5, (r, rms)
        en = g[f"r{r}_en"]
        e_ref = en[0] + en[1] + en[2] + en[4]
        assert abs(e[r] - e_ref) <= 1e-5 * max(abs(e_ref), 1.0), (r, e[r], e_ref)


def test_reference_form_trajectory_matches_oracle():
    """10 BAOAB steps under the reference's Go model against the oracle's
    (pinned to cgolik.c) with the same Philox draws (measured: positions
    within 1.8e-5 A, velocities 3.8e-4 A/ps, energies 4e-7).  Over 25 steps
    one of these chains passes a nearly straight torsion, where the FP32
    torsion force (~3e-5 of the force elsewhere) departs further and moves
    the chain 3e-3 A from the FP64 trajectory; the other chains stay within
    4e-5 A."""
    from thecodecombo_7_gb300 import engine, systems
    g = systems.go_chains(5, nmin=40, nmax=160, seed=12)
    hc = (g.eps, 4.0, 12.0)
    b = engine.GoBatch(g, seed=6)
    try:
        b.set_reference_form(d_rep=hc[1], rc=hc[2])
        b.run(10)
        s = b.state()
    finally:
        b.close()
    st = g.start
    for r in range(len(g.nbeads)):
        x, v, e = O.go_hc_baoab(g, r, hc, 10, seed=6)
        assert np.abs(s["pos"][st[r]:st[r + 1]] - x).max() < 1e-4, r
        assert np.abs(s["vel"][st[r]:st[r + 1]] - v).max() < 2e-3, r
        assert abs(s["epot"][r] - e) <= 1e-5 * max(abs(e), 1.0), (r, s["epot"][r], e)
