"""CPU oracle of the importance network's forward pass, backward pass and
Adam update (test infrastructure: only tests, the smoke check and the
benchmark's baseline leg use it; the product never does).

The network has no reference counterpart; this module states the same
arithmetic as the tensor-core kernels in numpy so that their gradients can
be checked: BF16 rounding of weights, activations and backpropagated
pre-activation gradients exactly where the GPU rounds them, FP64 sums where
the GPU accumulates in FP32.  With ``bf16=False`` it is plain FP64
backpropagation, which the tests check against finite differences.

Parameter layout (flat FP32, 33,793 values): W1[128][4], b1[128],
W2[128][128], b2[128], W3[128][128], b3[128], w4[128], b4.
"""
from __future__ import annotations

import numpy as np

HID = 128
SIZES = [("W1", (HID, 4)), ("b1", (HID,)), ("W2", (HID, HID)), ("b2", (HID,)),
         ("W3", (HID, HID)), ("b3", (HID,)), ("w4", (HID,)), ("b4", (1,))]
N_PARAMS = sum(int(np.prod(s)) for _, s in SIZES)


def unpack(p):
    out, k = {}, 0
    for name, shape in SIZES:
        n = int(np.prod(shape))
        out[name] = np.asarray(p[k:k + n], dtype=np.float64).reshape(shape)
        k += n
    return out


def pack(d):
    return np.concatenate([np.asarray(d[name], dtype=np.float64).ravel() for name, _ in SIZES])


def bf16(x):
    """Round to the nearest BF16 value (ties to even), returned as float64."""
    f = np.asarray(x, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    u = ((u + 0x7FFF + lsb) >> 16) << 16
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def silu(z):
    return z / (1.0 + np.exp(-z))


def silu_grad(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(p, x4, bf=True):
    """Returns (y, cache) for inputs x4 [n][4]."""
    q = unpack(p)
    r = bf16 if bf else (lambda a: np.asarray(a, dtype=np.float64))
    X0 = r(x4)
    W1, W2, W3 = r(q["W1"]), r(q["W2"]), r(q["W3"])
    Z1 = X0 @ W1.T + q["b1"]
    H1 = r(silu(Z1))
    Z2 = H1 @ W2.T + q["b2"]
    H2 = r(silu(Z2))
    Z3 = H2 @ W3.T + q["b3"]
    H3 = r(silu(Z3))
    y = H3 @ q["w4"] + q["b4"][0]
    return y, dict(X0=X0, W1=W1, W2=W2, W3=W3, Z1=Z1, Z2=Z2, Z3=Z3, H1=H1, H2=H2, H3=H3, q=q)


def loss_and_grad(p, x4, target, weight=None, bf=True):
    """Weighted mean squared error sum(w (y - t)^2) / n and its gradient."""
    n = len(target)
    w = np.ones(n) if weight is None else np.asarray(weight, dtype=np.float64)
    y, c = forward(p, x4, bf)
    r = bf16 if bf else (lambda a: a)
    e = y - target
    loss = float(np.sum(w * e * e) / n)
    dy = 2.0 * w * e / n
    q = c["q"]
    g = {"w4": c["H3"].T @ dy, "b4": np.array([dy.sum()])}
    dZ3 = r(dy[:, None] * q["w4"][None, :] * silu_grad(c["Z3"]))
    g["W3"] = dZ3.T @ c["H2"]
    g["b3"] = dZ3.sum(0)
    dZ2 = r((dZ3 @ c["W3"]) * silu_grad(c["Z2"]))
    g["W2"] = dZ2.T @ c["H1"]
    g["b2"] = dZ2.sum(0)
    dZ1 = r((dZ2 @ c["W2"]) * silu_grad(c["Z1"]))
    g["W1"] = dZ1.T @ c["X0"]
    g["b1"] = dZ1.sum(0)
    return loss, pack(g)


def adam(p, m, v, g, t, lr, beta1=0.9, beta2=0.999, eps=1e-8):
    """One bias-corrected Adam update (step t >= 1)."""
    m = beta1 * m + (1 - beta1) * g
    v = beta2 * v + (1 - beta2) * g * g
    mh = m / (1 - beta1 ** t)
    vh = v / (1 - beta2 ** t)
    return p - lr * mh / (np.sqrt(vh) + eps), m, v


def init_params(seed):
    """LeCun-uniform weights, zero biases (the same construction as the
    device network's, not the same random numbers)."""
    rng = np.random.default_rng(seed)
    d = {}
    for name, shape in SIZES:
        if name.startswith("b"):
            d[name] = np.zeros(shape)
        else:
            fan_in = shape[-1] if len(shape) == 2 else shape[0]
            a = np.sqrt(3.0 / fan_in)
            d[name] = rng.uniform(-a, a, size=shape)
    return pack(d)
