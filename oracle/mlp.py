"""FP64 restatement of the proposal network and of its GPU training step.

TEST INFRASTRUCTURE ONLY: the gradient checks compare the engine's
tensor-core training kernel (k_mlp_train, reached through xrp_mlp_grad)
with this code; nothing in the product imports it.  The reference has no
network (its integrators are main.go:144-199); the definition restated here
is the engine's own: 64 inputs -> 64 -> 64 -> 64 (ReLU) -> 1 logit,
parameters packed as W1[64][64] (out, in), b1, W2, b2, W3, b3, w4[64], b4,
loss = (1/rows) * sum_r w_r * BCE(sigmoid(logit_r), y_r) with
w_r = pos_weight for y_r = 1, else 1.

``emulate=True`` applies the kernel's BF16 roundings at the points the
kernel applies them (weights, the two hidden activations after ReLU, and
the back-propagated signals that enter tensor-core products), with every
sum in FP64; ``emulate=False`` is the exact FP64 network.
"""
from __future__ import annotations

import numpy as np

IN = HID = 64
OFF = {}
_o = 0
for _name, _n in (("W1", HID * IN), ("b1", HID), ("W2", HID * HID), ("b2", HID),
                  ("W3", HID * HID), ("b3", HID), ("w4", HID), ("b4", 1)):
    OFF[_name] = (_o, _n)
    _o += _n
N_PARAMS = _o


def unpack(p):
    p = np.asarray(p, np.float64)
    g = {k: p[o:o + n] for k, (o, n) in OFF.items()}
    for k in ("W1", "W2", "W3"):
        g[k] = g[k].reshape(HID, -1)
    return g


def pack(g):
    out = np.zeros(N_PARAMS, np.float64)
    for k, (o, n) in OFF.items():
        out[o:o + n] = np.asarray(g[k], np.float64).ravel()
    return out


def bf16(x):
    """Round to the nearest BF16 (ties to even), via FP32 like the kernel's
    __float2bfloat16_rn of an FP32 value."""
    x32 = np.ascontiguousarray(np.asarray(x, np.float32))
    b = x32.view(np.uint32).astype(np.uint64)
    r = ((b + 0x7FFF + ((b >> 16) & 1)) >> 16) & 0xFFFF
    return (r.astype(np.uint32) << 16).view(np.float32).astype(np.float64)


def bf16_bits(x):
    """BF16 bit patterns (uint16) of x."""
    return (bf16(x).astype(np.float32).view(np.uint32) >> 16).astype(np.uint16)


def from_bf16_bits(b):
    return (np.asarray(b, np.uint32) << 16).view(np.float32).astype(np.float64)


def forward_backward(params, X, y, pos_weight=1.0, emulate=True):
    """Returns (loss, logits, grad) for feature rows X [rows][64] (values
    already BF16 when emulating) and labels y."""
    P = unpack(params)
    X = np.asarray(X, np.float64)
    y = np.asarray(y, np.float64)
    rows = X.shape[0]
    r = bf16 if emulate else (lambda a: np.asarray(a, np.float64))
    W1, W2, W3 = r(P["W1"]), r(P["W2"]), r(P["W3"])
    z1 = r(np.maximum(X @ W1.T + P["b1"], 0.0))
    z2 = r(np.maximum(z1 @ W2.T + P["b2"], 0.0))
    z3 = np.maximum(z2 @ W3.T + P["b3"], 0.0)
    logit = z3 @ P["w4"] + P["b4"][0]
    w = np.where(y > 0.5, pos_weight, 1.0)
    sp = np.maximum(logit, 0.0) + np.log1p(np.exp(-np.abs(logit)))
    loss = float(np.sum(w * (sp - y * logit)) / rows)
    sg = 1.0 / (1.0 + np.exp(-logit))
    dlog = w * (sg - y) / rows
    G = {"b4": np.array([dlog.sum()]), "w4": dlog @ z3}
    dz3 = np.where(z3 > 0, dlog[:, None] * P["w4"][None, :], 0.0)
    G["b3"] = dz3.sum(0)
    G["W3"] = r(dz3).T @ z2
    dz2 = np.where(z2 > 0, r(dz3) @ W3, 0.0)
    G["b2"] = dz2.sum(0)
    G["W2"] = r(dz2).T @ z1
    dz1 = np.where(z1 > 0, r(dz2) @ W2, 0.0)
    G["b1"] = dz1.sum(0)
    G["W1"] = r(dz1).T @ X
    return loss, logit, pack(G)


def init_params(seed=0):
    """He-uniform hidden layers, small output layer (the engine's own
    initialisation, restated for tests)."""
    rng = np.random.default_rng(seed)
    g = {"W1": rng.uniform(-1, 1, (HID, IN)) * np.sqrt(6.0 / IN),
         "W2": rng.uniform(-1, 1, (HID, HID)) * np.sqrt(6.0 / HID),
         "W3": rng.uniform(-1, 1, (HID, HID)) * np.sqrt(6.0 / HID),
         "w4": rng.uniform(-1, 1, HID) * np.sqrt(3.0 / HID),
         "b1": rng.normal(0, 0.1, HID), "b2": rng.normal(0, 0.1, HID),
         "b3": rng.normal(0, 0.1, HID), "b4": rng.normal(0, 0.1, 1)}
    return pack(g)


def segment_features(a, b):
    """The engine's positional features of a segment (a, b) in normalised
    coordinates: per coordinate c of (a, b): c, then sin/cos of pi*c*2^f for
    f = 0..3 (double-angle recurrences in the kernel); the unit direction; a
    constant 1; zeros up to 64."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    feats = []
    for c in np.concatenate([a, b], axis=-1).T:
        feats.append(c)
        for f in range(4):
            feats.append(np.sin(np.pi * c * 2 ** f))
            feats.append(np.cos(np.pi * c * 2 ** f))
    d = b - a
    n = np.linalg.norm(d, axis=-1, keepdims=True)
    d = np.where(n > 0, d / np.where(n > 0, n, 1), 0.0)
    feats.extend(list(d.T))
    feats.append(np.ones_like(a[..., 0]))
    X = np.stack(feats, axis=-1)
    pad = np.zeros(X.shape[:-1] + (IN - X.shape[-1],))
    return np.concatenate([X, pad], axis=-1)
