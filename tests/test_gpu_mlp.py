"""Tensor-core (tcgen05) kernels of the Monte Carlo surrogate network
against the CPU oracle: the GEMM alone, the forward/backward gradient of a
batch (BF16 rounding emulated in the oracle), and training."""
import numpy as np
import pytest

from oracle import mlp_oracle as M

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("Mr,N,K", [(128, 64, 64), (256, 128, 64), (1024, 128, 128),
                                    (128, 128, 1024), (128, 64, 1024), (384, 256, 192)])
def test_tc_gemm_matches_numpy(Mr, N, K):
    from thecodecombo_7_gb300 import engine
    rng = np.random.default_rng(Mr + N + K)
    A = M.bf16(rng.normal(0, 1, (Mr, K)).astype(np.float32))
    B = M.bf16(rng.normal(0, 1, (N, K)).astype(np.float32))
    bias = rng.normal(0, 1, N).astype(np.float32)
    D = engine.tc_gemm_bf16(M.bf16_bits(A), M.bf16_bits(B), bias)
    want = A.astype(np.float64) @ B.astype(np.float64).T + bias
    scale = np.abs(A).astype(np.float64) @ np.abs(B).astype(np.float64).T + 1.0
    # bf16 products are exact in fp32; only the fp32 summation order differs
    assert np.all(np.abs(D - want) <= 1e-5 * scale), np.abs(D - want).max()


def _batch(rng, B):
    data = rng.normal(0, 1, (B, 2 * M.N_IN)).astype(np.float32)
    y = rng.normal(0, 0.5, B).astype(np.float32)
    return data, y


def test_mlp_gradient_matches_oracle():
    from thecodecombo_7_gb300 import engine
    rng = np.random.default_rng(11)
    net = engine.Mlp(seed=5)
    try:
        P = rng.normal(0, 0.15, net.n_params).astype(np.float32)
        mean = rng.normal(0, 0.1, M.N_IN).astype(np.float32)
        istd = rng.uniform(0.8, 1.2, M.N_IN).astype(np.float32)
        net.set_params(P, mean, istd)
        data, y = _batch(rng, 128)
        loss, G, out = net.grad(data, y)
    finally:
        net.close()
    l_ref, G_ref, out_ref = M.forward_backward(P, data, y, mean, istd)
    assert abs(loss - l_ref) <= 1e-4 * abs(l_ref)
    assert np.abs(out - out_ref).max() <= 1e-3 * (1 + np.abs(out_ref).max())
    blocks = dict(W1=(M.OFF_W1, M.OFF_B1), b1=(M.OFF_B1, M.OFF_W2), W2=(M.OFF_W2, M.OFF_B2),
                  b2=(M.OFF_B2, M.OFF_W3), w3=(M.OFF_W3, M.OFF_B3), b3=(M.OFF_B3, M.N_PARAMS))
    # b3 cancels in g(after) - g(before): its gradient is exactly zero
    assert abs(G[M.OFF_B3]) <= 1e-6 and G_ref[M.OFF_B3] == 0.0
    del blocks["b3"]
    for name, (a, b) in blocks.items():
        g, r = G[a:b].astype(np.float64), G_ref[a:b]
        rel = np.linalg.norm(g - r) / max(np.linalg.norm(r), 1e-12)
        assert rel <= 2e-3, (name, rel)


def test_mlp_training_reduces_loss():
    from thecodecombo_7_gb300 import engine
    rng = np.random.default_rng(2)
    n = 4096
    w = rng.normal(0, 0.3, M.N_IN)

    def f(x):
        return np.tanh(x @ w) + 0.1 * (x[:, 0] ** 2)

    data = rng.normal(0, 1, (n, 2 * M.N_IN)).astype(np.float32)
    y = (f(data[:, M.N_IN:].astype(np.float64)) - f(data[:, :M.N_IN].astype(np.float64)))
    y = y.astype(np.float32)
    net = engine.Mlp(seed=9)
    try:
        hist = net.train(data, y, epochs=12, batch=256, lr=2e-3, seed=4)
    finally:
        net.close()
    var = float(np.var(y))
    assert hist[-1] < 0.1 * var, (hist, var)
    assert hist[-1] < hist[0]
