"""FP64 restatement of the warm-start MLP (TEST INFRASTRUCTURE ONLY).

Forward and backward of the network in rewl_simulator_gb300/csrc/mlp.cu in
float64 numpy, on the same padded parameter vector.  The tensors the GPU stores
in bf16 (inputs, weights, hidden activations, output gradient, backpropagated
activation gradients) are rounded to bf16 at the same points, so the GPU's
gradients must agree up to FP32-accumulation and erf differences.  With
`round_bf16=False` the arithmetic is plain FP64, which the finite-difference test
uses to pin the analytic gradients themselves.
"""
from __future__ import annotations

import math

import numpy as np

IN_PAD = 64
OUT_PAD = 64


def bf16(x: np.ndarray) -> np.ndarray:
    """Round to bfloat16 (nearest, ties to even) and return as float64."""
    f = np.asarray(x, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


_erf = np.vectorize(math.erf)


def gelu(z):
    return 0.5 * z * (1.0 + _erf(z / math.sqrt(2.0)))


def gelu_prime(z):
    return 0.5 * (1.0 + _erf(z / math.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / math.sqrt(2.0 * math.pi)


def unpack(params: np.ndarray, layout: np.ndarray):
    Ws, bs = [], []
    for din, dout, wo, bo in layout:
        Ws.append(params[wo:wo + din * dout].astype(np.float64).reshape(dout, din))
        bs.append(params[bo:bo + dout].astype(np.float64))
    return Ws, bs


def forward_backward(params, layout, X, y, round_bf16: bool = True):
    """Loss and gradient vector (same padded layout) of mean((f(X) - y)^2)."""
    R = bf16 if round_bf16 else (lambda a: np.asarray(a, dtype=np.float64))
    Ws, bs = unpack(params, layout)
    Wq = [R(W) for W in Ws]
    B = X.shape[0]
    H = np.zeros((B, IN_PAD))
    H[:, :X.shape[1]] = X
    Hs = [R(H)]
    Zs = []
    for l in range(len(Ws) - 1):
        Z = Hs[-1] @ Wq[l].T + bs[l]
        Zs.append(Z)
        Hs.append(R(gelu(Z)))
    out = Hs[-1] @ Wq[-1].T + bs[-1]
    e = out[:, 0] - y
    loss = float(np.mean(e * e))
    dOut = np.zeros_like(out)
    dOut[:, 0] = 2.0 * e / B
    dOut = R(dOut)
    grads = np.zeros_like(params, dtype=np.float64)
    L = len(Ws) - 1
    din, dout, wo, bo = layout[L]
    grads[wo:wo + din * dout] = (dOut.T @ Hs[L]).ravel()
    grads[bo:bo + dout] = dOut.sum(axis=0)
    dH = R(dOut @ Wq[L])
    for l in range(L - 1, -1, -1):
        G = R(dH * gelu_prime(Zs[l]))
        din, dout, wo, bo = layout[l]
        grads[wo:wo + din * dout] = (G.T @ Hs[l]).ravel()
        grads[bo:bo + dout] = G.sum(axis=0)
        if l > 0:
            dH = R(G @ Wq[l])
    return loss, grads


def predict(params, layout, X, round_bf16: bool = True):
    R = bf16 if round_bf16 else (lambda a: np.asarray(a, dtype=np.float64))
    Ws, bs = unpack(params, layout)
    H = np.zeros((X.shape[0], IN_PAD))
    H[:, :X.shape[1]] = X
    H = R(H)
    for l in range(len(Ws) - 1):
        H = R(gelu(H @ R(Ws[l]).T + bs[l]))
    return (H @ R(Ws[-1]).T + bs[-1])[:, 0]


def make_layout(hidden: int = 256, layers: int = 4):
    """The padded parameter layout of the GPU network (mirrors rewl_mlp_create)."""
    rows, off = [], 0
    for l in range(layers + 1):
        din = IN_PAD if l == 0 else hidden
        dout = OUT_PAD if l == layers else hidden
        wo = off
        off += din * dout
        bo = off
        off += dout
        off = (off + 7) & ~7
        rows.append((din, dout, wo, bo))
    return np.array(rows, dtype=np.int64), off
