"""CPU restatement of the learned path's network for checking the tensor-core
kernels.  TEST INFRASTRUCTURE ONLY (tests/ and the benchmark's checks).

The network: 42 inputs, hidden layers of 64 with ReLU, 4 linear outputs
(irradiance RGB and an estimate e of the network's own error there);
packed parameters W1[64][42] b1[64] W2[64][64] b2[64] W3[64][64] b3[64]
W4[4][64] b4[4]; loss = mean squared error over the n x 3 irradiance
outputs + CONF_WEIGHT * mean over the n rows of (e - |y - t|)^2, with
|y - t| (the Euclidean error of the row's irradiance) held constant.

Two evaluations:
  - float64 throughout (the reference for the gradients' mathematics);
  - BF16-emulating: weights, inputs, hidden activations, dY and dZ rounded to
    BF16 (round to nearest even) where the kernels round them, products
    summed in float64 (the kernels sum in fp32); this one matches the kernels
    to accumulation-order rounding.
"""

from __future__ import annotations

import numpy as np

IN, HID, OUT = 42, 64, 4
CONF_WEIGHT = 0.5
SHAPES = [("W1", (HID, IN)), ("b1", (HID,)), ("W2", (HID, HID)), ("b2", (HID,)), ("W3", (HID, HID)), ("b3", (HID,)),
          ("W4", (OUT, HID)), ("b4", (OUT,))]
NPARAMS = sum(int(np.prod(s)) for _, s in SHAPES)


def unpack(p: np.ndarray) -> dict:
    out, o = {}, 0
    for name, shape in SHAPES:
        n = int(np.prod(shape))
        out[name] = np.asarray(p[o:o + n], dtype=np.float64).reshape(shape)
        o += n
    return out


def pack(d: dict) -> np.ndarray:
    return np.concatenate([np.asarray(d[name], dtype=np.float64).reshape(-1) for name, _ in SHAPES])


def bf16(x) -> np.ndarray:
    """Round to the nearest BF16 value (ties to even), returned as float64."""
    f = np.ascontiguousarray(x, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def forward_backward(p: np.ndarray, x: np.ndarray, y: np.ndarray | None = None, emulate_bf16: bool = False):
    """Returns (predictions (n, 4), loss, gradient (NPARAMS,)); loss and
    gradient are None without targets (n, 3)."""
    r = bf16 if emulate_bf16 else (lambda a: np.asarray(a, dtype=np.float64))
    w = unpack(p)
    W = {k: (r(v) if k.startswith("W") else v) for k, v in w.items()}
    n = x.shape[0]
    h0 = r(x)
    z1 = h0 @ W["W1"].T + W["b1"]
    h1 = r(np.maximum(z1, 0.0))
    z2 = h1 @ W["W2"].T + W["b2"]
    h2 = r(np.maximum(z2, 0.0))
    z3 = h2 @ W["W3"].T + W["b3"]
    h3 = r(np.maximum(z3, 0.0))
    out = h3 @ W["W4"].T + W["b4"]
    if y is None:
        return out, None, None
    diff = out[:, :3] - np.asarray(y, dtype=np.float64)
    err = np.sqrt((diff ** 2).sum(1))  # held constant: no gradient through it
    dc = out[:, 3] - err
    loss = float((diff ** 2).sum() / (3 * n) + CONF_WEIGHT * (dc ** 2).sum() / n)
    if emulate_bf16:
        # the kernels compute (2 / 3n) * diff and (2 w / n) * dc in fp32 and round them to BF16
        d32 = diff.astype(np.float32)
        e32 = np.sqrt((d32 * d32).sum(1, dtype=np.float32))
        dc32 = out[:, 3].astype(np.float32) - e32
        dy = np.concatenate([r(np.float32(2.0 / (3.0 * n)) * d32),
                             r(np.float32(2.0 * CONF_WEIGHT / n) * dc32)[:, None]], 1)
    else:
        dy = np.concatenate([2.0 * diff / (3 * n), (2.0 * CONF_WEIGHT / n) * dc[:, None]], 1)
    g = {"W4": dy.T @ h3, "b4": dy.sum(0)}
    dz3 = r((dy @ W["W4"]) * (z3 > 0))
    g["W3"], g["b3"] = dz3.T @ h2, dz3.sum(0)
    dz2 = r((dz3 @ W["W3"]) * (z2 > 0))
    g["W2"], g["b2"] = dz2.T @ h1, dz2.sum(0)
    dz1 = r((dz2 @ W["W2"]) * (z1 > 0))
    g["W1"], g["b1"] = dz1.T @ h0, dz1.sum(0)
    return out, loss, pack(g)


def adam(p, grad, m, v, step, lr, beta1=0.9, beta2=0.999, eps=1e-8):
    """One Adam step (Kingma & Ba 2015) in float64; returns (p, m, v)."""
    m = beta1 * m + (1 - beta1) * grad
    v = beta2 * v + (1 - beta2) * grad * grad
    mh = m / (1 - beta1 ** step)
    vh = v / (1 - beta2 ** step)
    return p - lr * mh / (np.sqrt(vh) + eps), m, v
