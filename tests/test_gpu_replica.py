"""Replicas stepped together in one graph, with exchange on the device.

FP64 boxes against the oracle: every box runs the reference's NHC step
(integrate_nhc / integrate_vverlet / integrate_nhc), and every exchange
attempt is replayed on the CPU with the oracle's swap_box restatement and the
same Philox draws -- same slots, same velocity rescales, same trajectories.
Mixed-precision boxes: stepping them box by box in one graph changes
nothing (bitwise equal to running each box alone) when no exchange is
attempted; the fused step (one launch per kernel for all boxes) agrees with
box by box to the rounding of the batched FFTs."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

SEED = 20241
TEMPS = [300.0, 302.0, 304.0, 306.0]


def _systems():
    from thecodecombo_7_gb300 import systems
    out = []
    for k, (n_mol, seed) in enumerate([(200, 11), (200, 12), (160, 13), (200, 14)]):
        s = systems.water_box(n_mol, L=25.0, seed=seed, T=TEMPS[k])
        s.nlist_freq = 5
        out.append(s)
    return out


def _potens(en_row):
    # calcvalue.c:43: bond + bend + nbonds (rec columns kinet, bond, bend, nbond, nbonds, ..)
    return en_row[1] + en_row[2] + en_row[4]


def test_batch_exchange_matches_oracle():
    from thecodecombo_7_gb300 import engine
    ss = _systems()
    R = len(ss)
    nseg, seg = 4, 5
    boxes = [engine.Box(s, precision=engine.FE_PREC_FP64) for s in ss]
    try:
        for b in boxes:
            b.nblist()
            b.forces()
        batch = engine.Batch(boxes, seed=SEED)
        batch.run(nseg * seg, nlist_freq=5, swap_freq=seg, first_step=1, use_nhc=True)
        st = batch.state()
        got = [(b.get_positions(), b.get_velocities()[0], b.get_nhc_state()) for b in boxes]
        launches = batch.step_launches()
        batch.close()
    finally:
        for b in boxes:
            b.close()

    # oracle replay
    ors = [O.Oracle(s) for s in ss]
    state = [dict(pos=s.pos.copy(), nop=s.pos.copy(), vel=s.vel.copy(), zeta=None) for s in ss]
    T_slot = np.array(TEMPS)
    slot_box = np.arange(R, dtype=np.int32)
    T_box = np.array(TEMPS)
    zeta_slot = [None] * R
    n_acc = 0
    for a in range(nseg):
        U = np.zeros(R)
        for r in range(R):
            out = ors[r].run_md(seg, use_nhc=True, pos=state[r]["pos"], vel=state[r]["vel"],
                                zeta=state[r]["zeta"], pos_nopbc=state[r]["nop"], T=T_box[r])
            state[r] = dict(pos=out["pos"], nop=out["pos_nopbc"], vel=out["vel"],
                            zeta=out["zeta"].reshape(-1))
            U[r] = _potens(out["en"][-1])
        new_slot, vmode, vfac, n = O.rex_attempt(T_slot, U, slot_box, a, SEED)
        n_acc += n
        for s in range(R):
            if new_slot[s] != slot_box[s]:
                r = new_slot[s]
                T_box[r] = T_slot[s]
        # chain states follow the slots: box now in slot s takes the chain of slot s
        old_z = {slot_box[s]: state[slot_box[s]]["zeta"] for s in range(R)}
        for s in range(R):
            state[new_slot[s]]["zeta"] = old_z[slot_box[s]]
        for r in range(R):
            if vmode[r] == 1:
                state[r]["vel"] = state[r]["vel"] * vfac[r]
            elif vmode[r] == 2:
                state[r]["vel"] = state[r]["vel"] / vfac[r]
        slot_box = new_slot

    assert st["attempts"] == nseg
    assert np.array_equal(st["slot_box"], slot_box), (st["slot_box"], slot_box)
    assert np.allclose(st["T_box"], T_box, rtol=0, atol=0)
    assert int(st["accepted"].sum()) == n_acc
    assert n_acc > 0, "the test temperatures should give some accepted swaps"
    for r in range(R):
        pos, vel, zeta = got[r]
        L = ss[r].L[0]
        d = pos - state[r]["pos"]
        d -= L * np.round(d / L)
        assert np.abs(d).max() < 1e-8, (r, np.abs(d).max())
        assert np.abs(vel - state[r]["vel"]).max() < 1e-8 * max(1.0, np.abs(vel).max())
        assert np.allclose(zeta.reshape(-1), state[r]["zeta"], rtol=1e-8, atol=1e-14)
    assert launches[0] > 0 and launches[3] > launches[1]


def test_batch_mixed_equals_single_boxes():
    from thecodecombo_7_gb300 import engine, systems
    ss = [systems.water_box(n, density=0.1, seed=40 + n) for n in (1365, 2000, 2600)]
    for s in ss:
        s.nlist_freq = 10
    alone = []
    for s in ss:
        with engine.Box(s, precision=engine.FE_PREC_MIXED) as b:
            b.nblist()
            b.forces()
            b.run_md(25, use_nhc=True, first_step=1, record=False)
            alone.append((b.get_positions(), b.get_velocities()[0]))
    boxes = [engine.Box(s, precision=engine.FE_PREC_MIXED) for s in ss]
    try:
        for b in boxes:
            b.nblist()
            b.forces()
        batch = engine.Batch(boxes, seed=3)
        batch.set_fused(False)
        batch.run(25, nlist_freq=10, swap_freq=0, first_step=1, use_nhc=True)
        together = [(b.get_positions(), b.get_velocities()[0]) for b in boxes]
        batch.close()
    finally:
        for b in boxes:
            b.close()
    for (p1, v1), (p2, v2) in zip(alone, together):
        assert np.array_equal(p1, p2)
        assert np.array_equal(v1, v2)


def test_fused_batch_matches_box_by_box():
    """The fused step (each kernel once for every box, batched FFTs per grid
    shape) against the box-by-box graph on the same mixed-precision boxes of
    uneven sizes and grids: Nose-Hoover steps with list rebuilds and replica
    exchanges; the same slots and temperatures, positions to 1e-6 A (the
    batched FFT may round differently in the last bit; forces are fixed-point
    sums either way)."""
    from thecodecombo_7_gb300 import engine, systems
    specs = [(1365, 300.0, None), (2000, 310.0, None), (1365, 320.0, None),
             (2600, 330.0, (45, 45, 45)), (2600, 340.0, (45, 45, 45)), (2000, 350.0, (27, 36, 25))]
    # odd grids (45^3, 27 x 36 x 25) exercise the padded, aligned slots of the
    # batched FFT buffers; two boxes share each grid shape
    ss = [systems.water_box(n, density=0.1, seed=60 + k, T=T, r_switch=8.0, grid=g)
          for k, (n, T, g) in enumerate(specs)]
    for s in ss:
        s.nlist_freq = 10
    out = {}
    for fused in (False, True):
        boxes = [engine.Box(s, precision=engine.FE_PREC_MIXED) for s in ss]
        try:
            for b in boxes:
                b.nblist()
                b.forces()
            batch = engine.Batch(boxes, seed=5)
            batch.set_fused(fused)
            batch.run(40, nlist_freq=10, swap_freq=10, first_step=1, use_nhc=True)
            st = batch.state()
            out[fused] = (st, [(b.get_positions(), b.get_velocities()[0]) for b in boxes],
                          batch.step_launches())
            batch.close()
        finally:
            for b in boxes:
                b.close()
    (s0, x0, l0), (s1, x1, l1) = out[False], out[True]
    assert np.array_equal(s0["slot_box"], s1["slot_box"])
    assert np.array_equal(s0["T_box"], s1["T_box"])
    assert s1["attempts"] == 4
    for (p0, v0), (p1, v1), s in zip(x0, x1, ss):
        d = p1 - p0
        d -= s.L * np.round(d / s.L)
        assert np.abs(d).max() < 1e-6
        assert np.abs(v1 - v0).max() < 1e-4 * np.abs(v0).max()
    # one launch per kernel for all boxes: far fewer than box by box; the
    # list rebuild adds six launches and the exchange two (list steps here
    # are exchange steps too)
    assert 0 < l1[0] <= 14 and l1[0] < l0[0]
    assert 0 < l1[3] <= 22 and l1[3] < l0[3]
