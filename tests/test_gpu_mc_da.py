"""Delayed-acceptance Monte Carlo with the trained surrogate.

1. Exact-mode chains collect (descriptors, exact dE_k) samples; the network
   is trained on them on the device; on held-out samples its prediction
   error is below that of the method without it (a zero estimate of dE_k).
2. The in-kernel surrogate (FP32 arithmetic, bf16 weights, normalisation
   folded in) agrees with the tensor-core network on the same descriptors.
3. A delayed-acceptance chain applies both stages exactly (replayed from its
   log), evaluates the reciprocal sum only after stage 1 accepts, its exact
   dE agrees with the oracle, and replaying its accepted moves reproduces
   its final coordinates bit for bit."""
import numpy as np
import pytest

from oracle import mlp_oracle as MO
from oracle import oracle as O

pytestmark = pytest.mark.gpu

T = 300.0
BETA = 1.0 / (1.380662e-23 * 6.022045e23 * T * 1e-3)


@pytest.fixture(scope="module")
def trained():
    from thecodecombo_7_gb300 import engine, systems
    s = systems.water_box(1365, density=0.1, seed=31)
    box = engine.Box(s, precision=engine.FE_PREC_FP64)
    box.mc_chains_setup(nchains=32, kmax=7, T=T, seed=17)
    box.mc_chains_collect(1000)
    box.mc_chains_run(1000)
    train = box.mc_chains_samples()
    net = engine.Mlp(seed=3)
    hist = box.mc_chains_train_surrogate(net, epochs=25, batch=512, lr=2e-3, seed=5)
    # held-out samples from other chains (another seed)
    box.mc_chains_setup(nchains=8, kmax=7, T=T, seed=99)
    box.mc_chains_collect(500)
    box.mc_chains_run(500)
    held = box.mc_chains_samples()
    yield s, box, net, train, held, hist
    net.close()
    box.close()


def _predict(net, rows):
    B = (len(rows) // 64) * 64
    rows = rows[:B]
    _, _, out = net.grad(rows[:, :128], rows[:, 128])
    return out[B:] - out[:B], rows[:, 128]


def test_surrogate_beats_zero_estimate(trained):
    s, box, net, train, held, hist = trained
    assert len(train) == 32000 and len(held) == 4000
    assert np.isfinite(hist).all() and hist[-1] < hist[0]
    pred, y = _predict(net, held)
    mse_net = float(np.mean((pred - y) ** 2))
    mse_zero = float(np.mean(y ** 2))
    print(f"held-out dE_k: rms {np.sqrt(mse_zero):.4f} kJ/mol, "
          f"network residual rms {np.sqrt(mse_net):.4f} kJ/mol")
    assert mse_net < 0.8 * mse_zero


def test_in_kernel_surrogate_matches_network(trained):
    s, box, net, train, held, hist = trained
    box.mc_chains_setup(nchains=1, kmax=7, T=T, seed=7)
    box.mc_chains_set_surrogate(net)
    box.mc_chains_set_mode(1)
    box.mc_chains_collect(256)
    box.mc_chains_run(256)
    rows = box.mc_chains_samples()
    assert len(rows) == 256
    ghat = rows[:, 128].astype(np.float64)
    # the kernel's arithmetic: bf16 weights, fp32 normalised inputs and activations
    P, mean, istd = net.get_params()
    p = MO.unpack(P)
    W1, W2 = MO.bf16(p["W1"]).astype(np.float64), MO.bf16(p["W2"]).astype(np.float64)

    def g(x):
        x = ((x - mean) * istd).astype(np.float64)
        h1 = x @ W1.T + p["b1"]
        h1 = h1 / (1 + np.exp(-h1))
        h2 = h1 @ W2.T + p["b2"]
        return (h2 / (1 + np.exp(-h2))) @ p["w3"]

    want = g(rows[:, 64:128]) - g(rows[:, :64])
    scale = float(np.std(want)) + 1e-3
    assert np.abs(want - ghat).max() <= 1e-3 * scale, np.abs(want - ghat).max()
    # and the tensor-core network, which also rounds inputs and activations to
    # bf16: agreement to a few percent of the spread
    pred, _ = _predict(net, rows)
    assert np.abs(pred - ghat).mean() <= 0.05 * scale


def test_delayed_acceptance_chain_replay(trained):
    s, box, net, train, held, hist = trained
    n = 200
    box.mc_chains_setup(nchains=1, kmax=7, T=T, seed=4242, log_cap=n)
    pos0, _, _ = box.mc_chains_state(0)
    box.mc_chains_set_surrogate(net)
    box.mc_chains_set_mode(1)
    box.mc_chains_run(n)
    rec, fx = box.mc_chains_log(n)
    xyz, mv, acc = box.mc_chains_state(0)
    st = box.mc_chains_stats(0)
    assert st["moves"] == n and st["kspace"] == st["stage1"] < n
    o = O.Oracle(s)
    L = float(s.L[0])
    pos = pos0.copy()
    n_acc = 0
    for t in range(n):
        lb, m = int(rec[t, 0]) >> 1, int(rec[t, 1])
        de, u1, dE1, u2, s1, kev, ghat = rec[t, 5], rec[t, 6], rec[t, 7], rec[t, 8], \
            rec[t, 9], rec[t, 10], rec[t, 11]
        assert abs(dE1 - (de + ghat)) < 1e-5
        a1 = -dE1 * BETA
        want1 = a1 > 0 or np.exp(a1) > u1
        if not (a1 <= 0 and abs(np.exp(a1) - u1) < 1e-5):
            assert bool(s1) == want1
        assert kev == s1
        new = (fx[t, :m].astype(np.float64) * 2.0 ** -32 - 0.5) * L
        pos_new = pos.copy()
        pos_new[lb:lb + m] = new
        if s1:
            dE, parts = o.mc_delta_energy(pos, pos_new, lb, lb + m, kmax=7, max_k_square=49,
                                          rc_ew=10.0)
            assert abs(dE - rec[t, 3]) <= 2e-3
            a2 = -(rec[t, 4] - ghat) * BETA
            want2 = a2 > 0 or np.exp(a2) > u2
            if not (a2 <= 0 and abs(np.exp(a2) - u2) < 1e-5):
                assert bool(rec[t, 2]) == want2
        else:
            assert rec[t, 2] == 0 and np.isnan(rec[t, 3])
        if rec[t, 2]:
            n_acc += 1
            pos = pos_new
    assert acc == n_acc > 0
    assert np.array_equal(xyz, pos)


def _mc_energy(s, pos):
    """The chains' energy function at pos: classic-Ewald reciprocal (kmax 7)
    + real space + shifted LJ of all pairs minus the intramolecular
    correction, from the FP64 engine (the self energy is a constant)."""
    from thecodecombo_7_gb300 import engine
    with engine.Box(s, precision=engine.FE_PREC_FP64) as b:
        b.set_positions(pos)
        b.mc_setup(kmax=7)
        t = b.mc_site_energy(0, s.n)
    return t[0] + (t[1] - t[2]) + (t[3] - t[5])


def test_delayed_acceptance_samples_the_exact_distribution(trained):
    """64 exact-dE chains and 64 delayed-acceptance chains started from the
    same equilibrated configuration, 40,000 moves each (about 30 moves per
    molecule): the mean and the variance of the energy of their final states
    agree within their statistical errors (4 standard errors for the means,
    an F ratio inside [0.45, 2.2] for the variances).  Delayed acceptance
    keeps the Boltzmann distribution of the exact energy, only its acceptance
    per move is lower."""
    s, box, net, train, held, hist = trained
    # equilibrate one exact chain from the random start
    box.mc_chains_setup(nchains=1, kmax=7, T=T, seed=2024)
    box.mc_chains_run(300000)
    x0, _, _ = box.mc_chains_state(0)
    u = {}
    for mode, seed in ((0, 501), (1, 502)):
        box.set_positions(x0)
        box.mc_chains_setup(nchains=64, kmax=7, T=T, seed=seed)
        if mode:
            box.mc_chains_set_surrogate(net)
            box.mc_chains_set_mode(1)
        box.mc_chains_run(40000)
        u[mode] = np.array([_mc_energy(s, box.mc_chains_state(c)[0]) for c in range(64)])
    m0, m1 = u[0].mean(), u[1].mean()
    v0, v1 = u[0].var(ddof=1), u[1].var(ddof=1)
    se = np.sqrt(v0 / 64 + v1 / 64)
    print(f"<U> exact {m0:.2f} +- {np.sqrt(v0 / 64):.2f}, delayed {m1:.2f} +- "
          f"{np.sqrt(v1 / 64):.2f} kJ/mol; Var ratio {v1 / v0:.3f}")
    assert abs(m1 - m0) <= 4.0 * se
    assert 0.45 <= v1 / v0 <= 2.2
