"""The surrogate network's CPU oracle: BF16 rounding and the backward pass
(finite differences of the exact-arithmetic network)."""
import numpy as np

from oracle import mlp_oracle as M


def test_bf16_rounding():
    # bf16 spacing at 1 is 2^-7: 1 + 2^-7 is exact, 1 + 2^-8 is a tie -> even (1),
    # 1 + 3 * 2^-8 is a tie -> even (1 + 2^-6), 1 + 2^-8 + 2^-12 rounds up
    x = np.array([1.0, 1.0078125, 1.00390625, 1.01171875, 1.0041503906, -3.0, 0.0], np.float32)
    want = np.array([1.0, 1.0078125, 1.0, 1.015625, 1.0078125, -3.0, 0.0], np.float32)
    assert np.array_equal(M.bf16(x), want)
    assert M.bf16_bits(np.array([1.0], np.float32))[0] == 0x3F80


def test_oracle_gradient_finite_differences():
    rng = np.random.default_rng(3)
    B = 8
    P = rng.normal(0, 0.2, M.N_PARAMS)
    data = rng.normal(0, 1, (B, 2 * M.N_IN))
    y = rng.normal(0, 0.5, B)
    mean, istd = np.zeros(M.N_IN), np.ones(M.N_IN)
    loss, G, _ = M.forward_backward(P, data, y, mean, istd, round_bf16=False)
    for k in list(rng.choice(M.N_PARAMS, 40, replace=False)) + [M.OFF_B3, M.OFF_B1 + 3]:
        h = 1e-6
        Pp, Pm = P.copy(), P.copy()
        Pp[k] += h
        Pm[k] -= h
        lp = M.forward_backward(Pp, data, y, mean, istd, round_bf16=False)[0]
        lm = M.forward_backward(Pm, data, y, mean, istd, round_bf16=False)[0]
        fd = (lp - lm) / (2 * h)
        assert abs(fd - G[k]) <= 1e-6 + 1e-5 * abs(fd), (k, fd, G[k])
