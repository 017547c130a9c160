"""CPU oracle of the warm-start network -- TEST INFRASTRUCTURE ONLY.

The MLP of fsph_mlp (FSPH_MLP_FEATURES -> 64 -> 64 -> 3, ReLU) in numpy
FP64: forward pass and the gradient of the loss mean_i sum_k (y_ik - t_ik)^2
with respect to the parameter blob (layout of include/fsph.h).  With
bf16=True the values the GPU kernels round to BF16 before each tensor-core
product (normalised inputs, weights, hidden activations, deltas) are rounded
the same way, so the comparison isolates summation order; with bf16=False it
is the exact FP64 reference the BF16 error is reported against.
"""
from __future__ import annotations

import numpy as np

NI, NH, NO = 32, 64, 3
O_MU = 0
O_SIG = O_MU + NI
O_W1 = O_SIG + NI
O_B1 = O_W1 + NI * NH
O_W2 = O_B1 + NH
O_B2 = O_W2 + NH * NH
O_W3 = O_B2 + NH
O_B3 = O_W3 + NH * NO
O_SCALE = O_B3 + NO
BLOB = O_SCALE + 1


def bf16(a: np.ndarray) -> np.ndarray:
    """Round to the nearest BF16 (ties to even), returned as float64."""
    f = np.asarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    lsb = (u >> np.uint64(16)) & np.uint64(1)
    r = ((u + np.uint64(0x7FFF) + lsb) >> np.uint64(16)) << np.uint64(16)
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(blob):
    b = np.asarray(blob, dtype=np.float64)
    return dict(mu=b[O_MU:O_SIG], sig=b[O_SIG:O_W1], W1=b[O_W1:O_B1].reshape(NI, NH), b1=b[O_B1:O_W2],
                W2=b[O_W2:O_B2].reshape(NH, NH), b2=b[O_B2:O_W3], W3=b[O_W3:O_B3].reshape(NH, NO),
                b3=b[O_B3:O_SCALE], scale=b[O_SCALE])


def forward(blob, x, bf16_emul: bool = False):
    """Returns (y, cache): y = network output times out_scale, shape (n, 3)."""
    P = unpack(blob)
    r = bf16 if bf16_emul else (lambda a: np.asarray(a, np.float64))
    isig = np.where(P["sig"] > 1e-20, 1.0 / np.where(P["sig"] > 1e-20, P["sig"], 1.0), 0.0)
    if bf16_emul:
        isig = isig.astype(np.float32).astype(np.float64)
    xn = (np.asarray(x, np.float64) - P["mu"]) * isig
    if bf16_emul:
        xn = xn.astype(np.float32).astype(np.float64)
    a0 = r(xn)
    z1 = a0 @ r(P["W1"]) + P["b1"]
    h1 = np.maximum(z1, 0.0)
    a1 = r(h1)
    z2 = a1 @ r(P["W2"]) + P["b2"]
    h2 = np.maximum(z2, 0.0)
    a2 = r(h2)
    o = a2 @ r(P["W3"]) + P["b3"]
    cache = dict(a0=a0, h1=h1, a1=a1, h2=h2, a2=a2, o=o, P=P)
    return o * P["scale"], cache


def gradient(blob, x, t, bf16_emul: bool = False):
    """Gradient of mean_i sum_k (o_ik - t_ik / scale)^2 w.r.t. the blob
    (normalisation and scale entries are zero) and the loss."""
    n = x.shape[0]
    o_scaled, C = forward(blob, x, bf16_emul)
    P = C["P"]
    r = bf16 if bf16_emul else (lambda a: np.asarray(a, np.float64))
    tt = np.asarray(t, np.float64) / P["scale"]
    e = C["o"] - tt
    loss = float((e * e).sum() / n)
    dy = 2.0 * e / n
    ddy = r(dy)
    d2 = (ddy @ r(P["W3"]).T) * (C["h2"] > 0)
    dd2 = r(d2)
    d1 = (dd2 @ r(P["W2"]).T) * (C["h1"] > 0)
    dd1 = r(d1)
    g = np.zeros(BLOB)
    g[O_W1:O_B1] = (C["a0"].T @ dd1).ravel()
    g[O_B1:O_W2] = dd1.sum(0)
    g[O_W2:O_B2] = (C["a1"].T @ dd2).ravel()
    g[O_B2:O_W3] = dd2.sum(0)
    g[O_W3:O_B3] = (C["a2"].T @ ddy).ravel()
    g[O_B3:O_SCALE] = ddy.sum(0)
    return g, loss
