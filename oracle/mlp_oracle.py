"""Float64 restatement of the learned-ordering MLP's forward and backward
pass, with BF16 rounding at the same points as the device (inputs,
activations and the softmax gradient fed to the GEMMs).

TEST INFRASTRUCTURE ONLY: the checker for pbg_learn_gradients.

Network: x[112] -> relu(W1 x + b1)[64] -> relu(W2 h1 + b2)[64] ->
W3 h2 + b3 [256]; loss = mean softmax cross-entropy.  Parameter layout
(pbg_learn_params_io): W1 [64 x 112], b1 [64], W2 [64 x 64], b2 [64],
W3 [256 x 64], b3 [256].
"""
from __future__ import annotations

import numpy as np

FEAT, HID, CLS = 112, 64, 256
SIZES = [HID * FEAT, HID, HID * HID, HID, CLS * HID, CLS]


def bf16(x):
    """Round float32 values to BF16 (nearest even), returned as float64."""
    u = np.ascontiguousarray(np.asarray(x, np.float32)).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) >> 16
    return (u.astype(np.uint32) << 16).view(np.float32).astype(np.float64)


def unpack(params):
    out, k = [], 0
    for n in SIZES:
        out.append(np.asarray(params[k:k + n], np.float64))
        k += n
    W1, b1, W2, b2, W3, b3 = out
    return W1.reshape(HID, FEAT), b1, W2.reshape(HID, HID), b2, W3.reshape(CLS, HID), b3


def gradients(params, x, labels):
    """Returns (flat gradients in the parameter layout, loss)."""
    W1, b1, W2, b2, W3, b3 = unpack(params)
    B = x.shape[0]
    X = bf16(x)
    W1b, W2b, W3b = bf16(W1), bf16(W2), bf16(W3)
    Z1 = X @ W1b.T + b1
    A1 = np.maximum(Z1, 0)
    H1 = bf16(A1)
    Z2 = H1 @ W2b.T + b2
    A2 = np.maximum(Z2, 0)
    H2 = bf16(A2)
    Z3 = H2 @ W3b.T + b3
    Zs = Z3 - Z3.max(1, keepdims=True)
    P = np.exp(Zs)
    P /= P.sum(1, keepdims=True)
    loss = float(-np.log(np.maximum(P[np.arange(B), labels], 1e-30)).mean())
    dZ3 = P.copy()
    dZ3[np.arange(B), labels] -= 1.0
    dZ3 /= B
    dZ3b = bf16(dZ3)
    gW3 = dZ3b.T @ H2
    gb3 = dZ3.sum(0)
    dH2 = dZ3b @ W3b
    dZ2 = dH2 * (A2 > 0)
    dZ2b = bf16(dZ2)
    gW2 = dZ2b.T @ H1
    gb2 = dZ2.sum(0)
    dH1 = dZ2b @ W2b
    dZ1 = dH1 * (A1 > 0)
    dZ1b = bf16(dZ1)
    gW1 = dZ1b.T @ X
    gb1 = dZ1.sum(0)
    flat = np.concatenate([gW1.reshape(-1), gb1, gW2.reshape(-1), gb2, gW3.reshape(-1), gb3])
    return flat, loss
