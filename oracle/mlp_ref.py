"""FP64 CPU reference of the step-size MLP (TEST INFRASTRUCTURE ONLY).

Restates the forward pass and the loss gradient of the GPU training kernel
(numbacs_gb300/csrc/mlp_train.cu) in numpy, with the same BF16 roundings of
the tensor-core operands (standardised inputs, W1, W2, layer-1 activations,
and the layer deltas dZ2 / dZ1 that enter the weight-gradient products), so
the GPU gradient can be checked to FP32-accumulation accuracy.

Parameter vector layout: W1[64][8], b1[64], W2[64][64], b2[64], w3[64], b3.
"""
import numpy as np

OFF_W1, OFF_B1, OFF_W2, OFF_B2, OFF_W3, OFF_B3, NPARAM = 0, 512, 576, 4672, 4736, 4800, 4801


EXACT = False  # set True to drop the BF16 roundings (finite-difference checks)


def bf16(x):
    """Round float values to bfloat16 (nearest even), returned as float64."""
    if EXACT:
        return np.asarray(x, np.float64)
    a = np.ascontiguousarray(np.asarray(x, np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(p):
    p = np.asarray(p, np.float64)
    return (p[OFF_W1:OFF_B1].reshape(64, 8), p[OFF_B1:OFF_W2], p[OFF_W2:OFF_B2].reshape(64, 64),
            p[OFF_B2:OFF_W3], p[OFF_W3:OFF_B3], p[OFF_B3])


def forward(p, feats, mu, inv_sigma):
    W1, b1, W2, b2, w3, b3 = unpack(p)
    x = bf16((np.asarray(feats, np.float64) - mu) * inv_sigma if EXACT else
             (np.asarray(feats, np.float32) - np.float32(mu)) * np.float32(inv_sigma))
    z1 = x @ bf16(W1).T + b1
    a1 = bf16(np.maximum(z1, 0.0))
    z2 = a1 @ bf16(W2).T + b2
    h2 = np.maximum(z2, 0.0)
    out = h2 @ w3 + b3
    return x, a1, h2, out


def predict(p, feats, mu, inv_sigma, out_mu, out_sigma):
    return out_mu + out_sigma * forward(p, feats, mu, inv_sigma)[3]


def loss_grad(p, feats, targets, mu, inv_sigma, out_mu, out_sigma):
    """(gradient of sum (net - standardised target)^2 / n, unscaled sum of squares)."""
    W1, b1, W2, b2, w3, b3 = unpack(p)
    n = len(targets)
    x, a1, h2, out = forward(p, feats, mu, inv_sigma)
    tn = (np.asarray(targets, np.float64) - out_mu) / out_sigma
    e = out - tn
    dout = 2.0 * e / n
    g = np.zeros(NPARAM)
    g[OFF_W3:OFF_B3] = h2.T @ dout
    g[OFF_B3] = dout.sum()
    dz2 = np.where(h2 > 0, dout[:, None] * w3[None, :], 0.0)
    g[OFF_B2:OFF_W3] = dz2.sum(0)
    dz2b = bf16(dz2)
    g[OFF_W2:OFF_B2] = (dz2b.T @ a1).ravel()
    da1 = dz2b @ bf16(W2)
    dz1 = np.where(a1 > 0, da1, 0.0)
    g[OFF_B1:OFF_W2] = dz1.sum(0)
    g[OFF_W1:OFF_B1] = (bf16(dz1).T @ x[:, :8]).ravel()
    return g, float((e * e).sum())
