"""CPU restatement of the Monte Carlo surrogate network's forward and
backward pass with BF16 rounding emulated where the device rounds.

TEST INFRASTRUCTURE ONLY: the checker for the device's tensor-core training
kernels, never the product path.  There is no counterpart in the reference
(the surrogate is a new component); the arithmetic follows the device
pipeline step by step:

    x' = bf16((x - mean) * istd)
    Z1 = x' W1b^T + b1            (bf16 operands, fp32 accumulation)
    H1 = bf16(silu(Z1))
    Z2 = H1 W2b^T + b2
    g  = w3 . silu(Z2) + b3       (fp32)
    loss = mean_s (g(after_s) - g(before_s) - y_s)^2
and the gradients by the chain rule with dZ2 and dZ1 rounded to bf16 before
the products that feed the weight gradients (as the tensor-core GEMMs see
them).  Parameters are packed W1 (128x64), b1, W2 (128x128), b2, w3, b3.
"""
import numpy as np

N_IN, N_H = 64, 128
OFF_W1 = 0
OFF_B1 = OFF_W1 + N_H * N_IN
OFF_W2 = OFF_B1 + N_H
OFF_B2 = OFF_W2 + N_H * N_H
OFF_W3 = OFF_B2 + N_H
OFF_B3 = OFF_W3 + N_H
N_PARAMS = OFF_B3 + 1


def bf16(x):
    """Round float32 values to bfloat16 (round to nearest even), returned as float32."""
    a = np.ascontiguousarray(x, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32).reshape(a.shape)


def bf16_bits(x):
    """bfloat16 bit patterns (uint16) of float32 values, round to nearest even."""
    return (bf16(x).view(np.uint32) >> 16).astype(np.uint16)


def unpack(P, dtype=np.float32):
    P = np.asarray(P, dtype)
    return dict(W1=P[OFF_W1:OFF_B1].reshape(N_H, N_IN), b1=P[OFF_B1:OFF_W2],
                W2=P[OFF_W2:OFF_B2].reshape(N_H, N_H), b2=P[OFF_B2:OFF_W3],
                w3=P[OFF_W3:OFF_B3], b3=P[OFF_B3])


def _silu(z):
    return z / (1.0 + np.exp(-z))


def _dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward_backward(P, data, y, mean, istd, round_bf16=True):
    """data: B x 128 (64 before | 64 after); returns (loss, grad[N_PARAMS], out[2B]).
    round_bf16=False gives the exact-arithmetic network (for derivative checks)."""
    rnd = bf16 if round_bf16 else (lambda a: np.asarray(a, np.float64))
    p = unpack(P, np.float32 if round_bf16 else np.float64)
    data = np.asarray(data, np.float32 if round_bf16 else np.float64)
    B = data.shape[0]
    X = np.concatenate([data[:, :N_IN], data[:, N_IN:]], axis=0)        # 2B x 64
    X = np.asarray(rnd((X - mean) * istd), np.float64)
    W1 = np.asarray(rnd(p["W1"]), np.float64)
    W2 = np.asarray(rnd(p["W2"]), np.float64)
    Z1 = X @ W1.T + p["b1"]
    H1 = np.asarray(rnd(_silu(Z1).astype(np.float32) if round_bf16 else _silu(Z1)), np.float64)
    Z2 = H1 @ W2.T + p["b2"]
    H2 = _silu(Z2)
    out = H2 @ p["w3"].astype(np.float64) + float(p["b3"])
    e = (out[B:] - out[:B]) - np.asarray(y, np.float64)
    loss = float(np.mean(e * e))
    g = 2.0 * e / B
    dout = np.concatenate([-g, g])
    dZ2 = dout[:, None] * p["w3"][None, :] * _dsilu(Z2)
    dZ2b = np.asarray(rnd(dZ2.astype(np.float32) if round_bf16 else dZ2), np.float64)
    dH1 = dZ2b @ W2
    dZ1 = dH1 * _dsilu(Z1)
    dZ1b = np.asarray(rnd(dZ1.astype(np.float32) if round_bf16 else dZ1), np.float64)
    G = np.zeros(N_PARAMS)
    G[OFF_W1:OFF_B1] = (dZ1b.T @ X).reshape(-1)
    G[OFF_B1:OFF_W2] = dZ1.sum(0)
    G[OFF_W2:OFF_B2] = (dZ2b.T @ H1).reshape(-1)
    G[OFF_B2:OFF_W3] = dZ2.sum(0)
    G[OFF_W3:OFF_B3] = dout @ H2
    G[OFF_B3] = dout.sum()
    return loss, G, out
