"""Reference of the warm-start perceptron in numpy (TEST INFRASTRUCTURE ONLY).

Mirrors clmgb.mlp's forward and backward passes with bf16 rounding applied at the
same points as the kernels (layer inputs, activations and backward signals in
bf16; products summed in float64 here, float32 on the GPU).
"""
import numpy as np

IN, HID, OUT, OUTP = 64, 128, 21, 32


def bf16(x):
    """Round float32 values to bfloat16 (round to nearest even), returned as float32."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32)
    r = ((u >> 16) & 1) + np.uint32(0x7FFF)
    return ((u + r) & np.uint32(0xFFFF0000)).view(np.float32)


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(X, W, b):
    """X [M,64] (bf16 values), W/b lists of float32 masters; weights used as bf16."""
    Wb = [bf16(w).astype(np.float64) for w in W]
    Z1 = X.astype(np.float64) @ Wb[0].T + b[0]
    H1 = bf16(silu(Z1).astype(np.float32)).astype(np.float64)
    Z2 = H1 @ Wb[1].T + b[1]
    H2 = bf16(silu(Z2).astype(np.float32)).astype(np.float64)
    Y = H2 @ Wb[2].T + b[2]
    return Y, (X.astype(np.float64), Z1, H1, Z2, H2)


def loss_and_dy(Y, T, w_dt=1.0, w_incr=1.0):
    M = Y.shape[0]
    e = Y - T
    w = np.zeros(OUTP)
    w[0] = w_dt
    w[1:OUT] = w_incr / 20.0
    L = float(np.sum(w * e * e) / M)
    dY = bf16((2.0 * w * e / M).astype(np.float32)).astype(np.float64)
    return L, dY


def backward(acts, dY, W):
    X, Z1, H1, Z2, H2 = acts
    Wb = [bf16(w).astype(np.float64) for w in W]
    dW3 = dY.T @ H2
    db3 = dY.sum(0)
    dH2 = bf16((dY @ Wb[2]).astype(np.float32)).astype(np.float64)
    dZ2 = bf16((dH2 * dsilu(Z2)).astype(np.float32)).astype(np.float64)
    dW2 = dZ2.T @ H1
    db2 = dZ2.sum(0)
    dH1 = bf16((dZ2 @ Wb[1]).astype(np.float32)).astype(np.float64)
    dZ1 = bf16((dH1 * dsilu(Z1)).astype(np.float32)).astype(np.float64)
    dW1 = dZ1.T @ X
    db1 = dZ1.sum(0)
    return [dW1, dW2, dW3], [db1, db2, db3]


def exact_gradients(X, T, W, b, w_dt=1.0, w_incr=1.0):
    """Gradient of the loss in float64 without any rounding (for derivative checks)."""
    Z1 = X @ W[0].T + b[0]
    H1 = silu(Z1)
    Z2 = H1 @ W[1].T + b[1]
    H2 = silu(Z2)
    Y = H2 @ W[2].T + b[2]
    M = X.shape[0]
    w = np.zeros(OUTP)
    w[0] = w_dt
    w[1:OUT] = w_incr / 20.0
    L = float(np.sum(w * (Y - T) ** 2) / M)
    dY = 2.0 * w * (Y - T) / M
    dW3 = dY.T @ H2
    dZ2 = (dY @ W[2]) * dsilu(Z2)
    dW2 = dZ2.T @ H1
    dZ1 = (dZ2 @ W[1]) * dsilu(Z1)
    dW1 = dZ1.T @ X
    return L, [dW1, dW2, dW3], [dZ1.sum(0), dZ2.sum(0), dY.sum(0)]
