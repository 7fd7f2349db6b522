"""NumPy restatement of the learned-preconditioner MLP — test infrastructure only.

The network of lywell_gb300/csrc/mlf_mlp.cu: 16 -> 128 (ReLU) -> 128 (ReLU)
-> 2, parameters read in BF16, hidden activations stored in BF16, sums in
(here) float64.  `grad` returns the gradient of the mean squared error
(mean over tokens and the two outputs) in the kernel's parameter layout:
W1[16][128] b1[128] W2[128][128] b2[128] W3[128][2] b3[2].

With bf16=False every rounding is dropped, which gives a plain float64
network for a finite-difference check of the backward pass itself.
"""
from __future__ import annotations

import numpy as np

IN, H, OUT = 16, 128, 2
SHAPES = [("W1", (IN, H)), ("b1", (H,)), ("W2", (H, H)), ("b2", (H,)), ("W3", (H, OUT)), ("b3", (OUT,))]
NPARAM = sum(int(np.prod(s)) for _, s in SHAPES)


def bf16(a):
    """Round float32 values to bfloat16 (nearest, ties to even), returned as float32."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    b = a.view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32)


def unpack(P):
    out, o = {}, 0
    for name, shp in SHAPES:
        n = int(np.prod(shp))
        out[name] = np.asarray(P[o:o + n], dtype=np.float64).reshape(shp)
        o += n
    return out


def pack(d):
    return np.concatenate([np.asarray(d[name], dtype=np.float64).ravel() for name, _ in SHAPES])


def forward(P, norm, X, bf=True):
    r = (lambda a: bf16(a).astype(np.float64)) if bf else (lambda a: np.asarray(a, dtype=np.float64))
    w = {k: r(v.astype(np.float32)) if bf else v for k, v in unpack(P).items()}
    mu, sd = np.asarray(norm[:IN], np.float32), np.asarray(norm[IN:], np.float32)
    xn = ((np.asarray(X, np.float32) - mu) / sd).astype(np.float64) if bf else (np.asarray(X) - norm[:IN]) / norm[IN:]
    a1 = xn @ w["W1"] + w["b1"]
    h1 = r(np.maximum(a1, 0).astype(np.float32)) if bf else np.maximum(a1, 0)
    a2 = h1 @ w["W2"] + w["b2"]
    h2 = r(np.maximum(a2, 0).astype(np.float32)) if bf else np.maximum(a2, 0)
    out = h2 @ w["W3"] + w["b3"]
    return out, dict(w=w, xn=xn, h1=h1, h2=h2)


def grad(P, norm, X, T, bf=True):
    out, c = forward(P, norm, X, bf)
    n = out.shape[0]
    d = out - np.asarray(T, dtype=np.float64)
    loss = float(np.mean(d * d))
    dout = 2.0 * d / (n * OUT)
    w = c["w"]
    g = {"W3": c["h2"].T @ dout, "b3": dout.sum(0)}
    dh2 = (dout @ w["W3"].T) * (c["h2"] > 0)
    g["W2"] = c["h1"].T @ dh2
    g["b2"] = dh2.sum(0)
    dh1 = (dh2 @ w["W2"].T) * (c["h1"] > 0)
    g["W1"] = c["xn"].T @ dh1
    g["b1"] = dh1.sum(0)
    return loss, pack(g)


def init(seed=0):
    """Glorot-uniform weights, zero biases (the same law as the kernel's
    initialiser, not the same random stream)."""
    rng = np.random.default_rng(seed)
    d = {}
    for name, shp in SHAPES:
        if name.startswith("W"):
            a = np.sqrt(6.0 / (shp[0] + shp[1]))
            d[name] = rng.uniform(-a, a, shp)
        else:
            d[name] = np.zeros(shp)
    return pack(d)
