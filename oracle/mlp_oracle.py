"""CPU restatement of the learned part's network (test infrastructure only:
the product never imports it).  It follows exadem_gb300/csrc/k_mlp.cu term for
term so the GPU gradients can be checked against it:

  x_b = bf16(x); W_b = bf16(W)            (round to nearest even)
  h1 = relu(x_b W1_b^T + b1)              h1_b = bf16(h1)
  h2 = relu(h1_b W2_b^T + b2)             h2_b = bf16(h2)
  z  = h2_b W3_b^T + b3                   rate = exp(z)
  loss = mean(exp(z) - y z)               over samples and the 4 outputs
  dz = (exp(z) - y) / (4 n)               (float32)
  dh2 = (bf16(dz) W3_b) * [h2 > 0]        dh2_b = bf16(dh2)
  dh1 = (dh2_b W2_b) * [h1 > 0]           dh1_b = bf16(dh1)
  dW3 = dz^T h2_b, db3 = sum dz;  dW2 = dh2_b^T h1_b, db2 = sum dh2_b;
  dW1 = dh1_b^T x_b, db1 = sum dh1_b
With round=False every bf16() is the identity (plain float64 network), which
the finite-difference test uses to check the backward formulas themselves.
Parameter vector: W1[64][16], b1[64], W2[64][64], b2[64], W3[4][64], b3[4].
"""
from __future__ import annotations

import numpy as np

NIN, NH, NOUT = 16, 64, 4
NPARAM = NH * NIN + NH + NH * NH + NH + NOUT * NH + NOUT


def bf16(a: np.ndarray) -> np.ndarray:
    """Round float32 values to the nearest bfloat16 (ties to even), returned as float32."""
    u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return r.astype(np.uint32).view(np.float32)


def unpack(p: np.ndarray):
    o = 0
    out = []
    for shape in ((NH, NIN), (NH,), (NH, NH), (NH,), (NOUT, NH), (NOUT,)):
        k = int(np.prod(shape))
        out.append(p[o:o + k].reshape(shape))
        o += k
    return out


def loss_grad(p: np.ndarray, x: np.ndarray, y: np.ndarray, round_bf16: bool = True):
    """Mean Poisson loss and its gradient (same layout as p)."""
    dt = np.float32 if round_bf16 else np.float64
    rnd = (lambda a: bf16(a)) if round_bf16 else (lambda a: np.asarray(a, dtype=np.float64))
    W1, b1, W2, b2, W3, b3 = (np.asarray(v, dtype=dt) for v in unpack(np.asarray(p, dtype=dt)))
    x = np.asarray(x, dtype=dt)
    y = np.asarray(y, dtype=dt)
    n = x.shape[0]
    W1b, W2b, W3b = rnd(W1), rnd(W2), rnd(W3)
    xb = rnd(x)
    h1 = np.maximum(xb @ W1b.T + b1, 0)
    h1b = rnd(h1)
    h2 = np.maximum(h1b @ W2b.T + b2, 0)
    h2b = rnd(h2)
    z = h2b @ W3b.T + b3
    lam = np.exp(z)
    loss = float(np.mean(lam - y * z))
    dz = ((lam - y) / (NOUT * n)).astype(dt)
    dh2 = (rnd(dz) @ W3b) * (h2 > 0)
    dh2b = rnd(dh2)
    dh1 = (dh2b @ W2b) * (h1 > 0)
    dh1b = rnd(dh1)
    g = [dh1b.T @ xb, dh1b.sum(0), dh2b.T @ h1b, dh2b.sum(0), dz.T @ h2b, dz.sum(0)]
    return loss, np.concatenate([v.ravel() for v in g]).astype(np.float64)


def rates(p: np.ndarray, x: np.ndarray) -> np.ndarray:
    W1, b1, W2, b2, W3, b3 = unpack(np.asarray(p, dtype=np.float32))
    h1 = bf16(np.maximum(bf16(x) @ bf16(W1).T + b1, 0))
    h2 = bf16(np.maximum(h1 @ bf16(W2).T + b2, 0))
    return np.exp(h2 @ bf16(W3).T + b3)
