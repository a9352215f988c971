"""FP64 numpy forward/backward of the beam surrogate's MLP (test
infrastructure: the checker for the library's own training kernels).

Layout of the FP32 parameter vector (as vgb_surrogate_get_params returns it):
W0 [256][6], W1..W3 [256][256], W4 [8][256], b0..b3 [4][256], b4 [8],
embeddings [nsets][2]. The weights enter the products rounded to BF16 (round
to nearest even) as on the device; biases and embeddings stay FP32.
Loss: mean over the batch and the 8 outputs of the squared error.
"""
from __future__ import annotations

import numpy as np
from scipy.special import erf

H = 256


def layout(nsets: int):
    off = {}
    o = 0
    for name, shape in (("W0", (H, 6)), ("W1", (H, H)), ("W2", (H, H)), ("W3", (H, H)), ("W4", (8, H)),
                        ("b", (4, H)), ("b4", (8,)), ("emb", (nsets, 2))):
        n = int(np.prod(shape))
        off[name] = (o, shape)
        o += n
    return off, o


def unpack(p, nsets):
    off, total = layout(nsets)
    assert p.size == total
    return {k: p[o:o + int(np.prod(s))].reshape(s).astype(np.float64) for k, (o, s) in off.items()}


def pack(d, nsets):
    off, total = layout(nsets)
    out = np.zeros(total, dtype=np.float64)
    for k, (o, s) in off.items():
        out[o:o + int(np.prod(s))] = d[k].reshape(-1)
    return out


def bf16(x):
    x = np.asarray(x, dtype=np.float32)
    b = x.view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


def gelu(x):
    return 0.5 * x * (1.0 + erf(x / np.sqrt(2.0)))


def gelu_grad(x):
    return 0.5 * (1.0 + erf(x / np.sqrt(2.0))) + x * np.exp(-0.5 * x * x) / np.sqrt(2.0 * np.pi)


def forward_backward(p, nsets, feat, sets, y):
    """feat [n][4], sets [n], y [n][8] -> (loss, gradient vector, predictions)."""
    P = unpack(np.asarray(p, dtype=np.float32), nsets)
    W = [bf16(P[f"W{l}"]) for l in range(5)]
    n = feat.shape[0]
    x0 = np.concatenate([feat.astype(np.float64), P["emb"][sets]], axis=1)
    acts, pres = [x0], []
    h = x0
    for l in range(4):
        pre = h @ W[l].T + P["b"][l]
        pres.append(pre)
        h = gelu(pre)
        acts.append(h)
    out = h @ W[4].T + P["b4"]
    d = out - y
    loss = float(np.mean(d * d))
    g = {k: np.zeros_like(v) for k, v in P.items()}
    dout = 2.0 * d / (8.0 * n)
    g["W4"] = dout.T @ acts[4]
    g["b4"] = dout.sum(0)
    dh = dout @ W[4]
    for l in range(3, -1, -1):
        dp = dh * gelu_grad(pres[l])
        g[f"W{l}"] = dp.T @ acts[l]
        g["b"][l] = dp.sum(0)
        dh = dp @ W[l]
    np.add.at(g["emb"], sets, dh[:, 4:6])
    return loss, pack(g, nsets), out
