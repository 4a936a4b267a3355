"""CPU restatement of the learned-importance network, the checker of its GPU kernels.

TEST INFRASTRUCTURE ONLY: tests/ compare the tcgen05 forward/backward kernels with this
file; nothing in the product imports it.

The network and its arithmetic follow monki-gpu_gb300/csrc/mlp.cu: inputs padded to 64,
three hidden layers of 256 with GELU (erf form), a linear output, weighted squared-error
loss. With ``bf16=True`` the values the device keeps in BF16 (weights, inputs, hidden
activations, the hidden-layer gradients) are rounded to BF16 (round to nearest even)
exactly where the kernels round them, and everything else is carried in float64, so the
comparison isolates the FP32 accumulation order of the tensor cores.
"""

from __future__ import annotations

import math

import numpy as np

IN, HIDDEN = 64, 256
SHAPES = (("W1", (HIDDEN, IN)), ("b1", (HIDDEN,)), ("W2", (HIDDEN, HIDDEN)), ("b2", (HIDDEN,)),
          ("W3", (HIDDEN, HIDDEN)), ("b3", (HIDDEN,)), ("w4", (HIDDEN,)), ("b4", (1,)))
COUNT = sum(int(np.prod(s)) for _, s in SHAPES)

_erf = np.vectorize(math.erf, otypes=[float])


def bf16(x):
    """Round to the nearest BF16 (ties to even), returned as float64."""

    f = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    u = f.view(np.uint32).astype(np.uint64)
    rounded = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return rounded.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(params):
    out, at = {}, 0
    for name, shape in SHAPES:
        size = int(np.prod(shape))
        out[name] = np.asarray(params[at : at + size], dtype=np.float64).reshape(shape)
        at += size
    return out


def pack(parts):
    return np.concatenate([np.asarray(parts[name], dtype=np.float64).ravel() for name, _ in SHAPES])


def gelu(z):
    return 0.5 * z * (1.0 + _erf(z / math.sqrt(2.0)))


def gelu_grad(z):
    return 0.5 * (1.0 + _erf(z / math.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / math.sqrt(2.0 * math.pi)


def forward(params, x, bf16_values=True):
    """Returns (y, cache)."""

    r = bf16 if bf16_values else (lambda v: np.asarray(v, dtype=np.float64))
    p = unpack(params)
    X = np.zeros((x.shape[0], IN))
    X[:, : x.shape[1]] = x
    X = r(X)
    W1, W2, W3 = r(p["W1"]), r(p["W2"]), r(p["W3"])
    Z1 = X @ W1.T + p["b1"]
    H1 = r(gelu(Z1))
    Z2 = H1 @ W2.T + p["b2"]
    H2 = r(gelu(Z2))
    Z3 = H2 @ W3.T + p["b3"]
    H3 = r(gelu(Z3))
    y = H3 @ p["w4"] + p["b4"][0]
    return y, dict(X=X, W2=W2, W3=W3, Z1=Z1, Z2=Z2, Z3=Z3, H1=H1, H2=H2, H3=H3, p=p, r=r)


def gradients(params, x, target, weight, scale=None, bf16_values=True):
    """Loss sum w (y - t)^2 * scale and its gradient in the parameter layout;
    scale defaults to 1 / sum(w)."""

    y, c = forward(params, x, bf16_values)
    r = c["r"]
    scale = 1.0 / np.sum(weight) if scale is None else scale
    d = y - target
    loss = float(np.sum(weight * d * d) * scale)
    dy = 2.0 * weight * d * scale
    g = {}
    g["w4"] = c["H3"].T @ dy
    g["b4"] = np.array([dy.sum()])
    # The kernels keep the pre-activations in BF16 for the backward pass.
    G3 = r(np.outer(dy, c["p"]["w4"]) * gelu_grad(r(c["Z3"])))
    g["W3"] = G3.T @ c["H2"]
    g["b3"] = G3.sum(0)
    G2 = r((G3 @ c["W3"]) * gelu_grad(r(c["Z2"])))
    g["W2"] = G2.T @ c["H1"]
    g["b2"] = G2.sum(0)
    G1 = r((G2 @ c["W2"]) * gelu_grad(r(c["Z1"])))
    g["W1"] = G1.T @ c["X"]
    g["b1"] = G1.sum(0)
    return loss, pack(g)


def initial(seed: int = 0, features: int = IN):
    """He-uniform hidden weights (zero columns past ``features``), small output layer."""

    rng = np.random.default_rng(seed)
    parts = {}
    fan = {"W1": features, "W2": HIDDEN, "W3": HIDDEN}
    for name, shape in SHAPES:
        if name in fan:
            bound = math.sqrt(6.0 / fan[name])
            w = rng.uniform(-bound, bound, size=shape)
            if name == "W1":
                w[:, features:] = 0.0
            parts[name] = w
        elif name == "w4":
            parts[name] = rng.uniform(-1.0, 1.0, size=shape) / math.sqrt(HIDDEN)
        else:
            parts[name] = np.zeros(shape)
    return pack(parts).astype(np.float32)
