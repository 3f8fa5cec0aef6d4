"""TEST INFRASTRUCTURE ONLY: CPU restatement of the warm-start MLP.

8 -> 128 -> 128 -> 128 -> 2 with GELU (erf form) on the hidden layers, the
flat parameter order of include/pd.h (W1[128][8], b1, W2[128][128], b2,
W3[128][128], b3, W4[2][128], b4).  ``forward`` / ``grad`` follow the
engine's rounding sequence when ``bf16=True``: weights, inputs, hidden
activations, the loss gradient and the backward deltas are rounded to BF16
(round to nearest even), products are accumulated exactly (float64 here,
FP32 on the tensor cores), biases are added in FP32.  With ``bf16=False``
the same formulas run in float64 (used for the finite-difference check of
the oracle itself).  No reference counterpart: the reference has no learned
component; this is the oracle the tensor-core kernels are checked against.
"""
import math

import numpy as np

N_IN, N_HID, N_OUT = 8, 128, 2
SHAPES = [("W1", (N_HID, N_IN)), ("b1", (N_HID,)), ("W2", (N_HID, N_HID)), ("b2", (N_HID,)),
          ("W3", (N_HID, N_HID)), ("b3", (N_HID,)), ("W4", (N_OUT, N_HID)), ("b4", (N_OUT,))]
N_PARAMS = sum(int(np.prod(s)) for _, s in SHAPES)  # 34,434

_erf = np.vectorize(math.erf)


def bf16(a):
    """Round float32 values to BF16 (nearest even), returned as float32."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    b = a.view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32).reshape(a.shape)


def unflatten(p):
    out, o = {}, 0
    for name, shape in SHAPES:
        n = int(np.prod(shape))
        out[name] = np.asarray(p[o:o + n]).reshape(shape)
        o += n
    return out


def flatten(d):
    return np.concatenate([np.asarray(d[name]).reshape(-1) for name, _ in SHAPES])


def init_params(seed=0):
    """He-style initial parameters (biases zero)."""
    rng = np.random.default_rng(seed)
    d = {}
    for name, shape in SHAPES:
        if name.startswith("W"):
            d[name] = rng.standard_normal(shape) * math.sqrt(2.0 / shape[1])
        else:
            d[name] = np.zeros(shape)
    return flatten(d).astype(np.float32)


def gelu(z):
    return 0.5 * z * (1.0 + _erf(z / math.sqrt(2.0)))


def gelu_grad(z):
    return 0.5 * (1.0 + _erf(z / math.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / math.sqrt(2.0 * math.pi)


def forward(p, x, bf=True):
    """x: [M][8] inputs.  Returns (y [M][2], cache)."""
    w = unflatten(p)
    r = bf16 if bf else (lambda a: np.asarray(a, dtype=np.float64))
    f32 = (lambda a: np.asarray(a, dtype=np.float32)) if bf else (lambda a: a)
    h = r(x).astype(np.float64)
    cache = {"h0": h}
    for k in (1, 2, 3):
        W = r(w[f"W{k}"]).astype(np.float64)
        z = f32(f32(h @ W.T) + f32(w[f"b{k}"]))
        h = r(gelu(np.asarray(z, dtype=np.float64))).astype(np.float64)
        cache[f"z{k}"], cache[f"h{k}"] = np.asarray(z, dtype=np.float64), h
    W4 = r(w["W4"]).astype(np.float64)
    y = f32(f32(h @ W4.T) + f32(w["b4"]))
    return np.asarray(y, dtype=np.float64), cache


def grad(p, x, t, bf=True):
    """Gradient of sum((y - t)^2) / (2 M).  Returns (flat gradient, loss)."""
    w = unflatten(p)
    M = x.shape[0]
    r = bf16 if bf else (lambda a: np.asarray(a, dtype=np.float64))
    y, c = forward(p, x, bf)
    e = y - t
    loss = float((e * e).sum() / (2.0 * M))
    d = r(e / M).astype(np.float64)  # dY
    g = {}
    g["W4"] = d.T @ c["h3"]
    g["b4"] = d.sum(axis=0)
    dh = d @ r(w["W4"]).astype(np.float64)
    for k in (3, 2, 1):
        dz = r(dh * gelu_grad(c[f"z{k}"])).astype(np.float64)
        g[f"W{k}"] = dz.T @ c[f"h{k - 1}"]
        g[f"b{k}"] = dz.sum(axis=0)
        if k > 1:
            dh = dz @ r(w[f"W{k}"]).astype(np.float64)
    return flatten(g), loss
