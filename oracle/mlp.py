"""FP64 CPU oracle of the learned-correction network and its loss.

TEST INFRASTRUCTURE: checks the GPU training kernels (forward, loss and
gradients).  It follows the same definition as powspec_gb300/csrc/ps_mlp.cu:
inputs, weights of the three hidden layers and hidden activations are
rounded to BF16 where the GPU feeds its tensor cores; everything else is
exact (FP64 here), and gradients pass straight through the BF16 roundings.
"""
from __future__ import annotations

import numpy as np

K1, H, IN, GROUP = 16, 64, 6, 16
oW1 = 0
ob1 = oW1 + K1 * H
oW2 = ob1 + H
ob2 = oW2 + H * H
oW3 = ob2 + H
ob3 = oW3 + H * H
ow4 = ob3 + H
ob4 = ow4 + H
NPARAM = ob4 + 1


def bf16(x):
    """Round to BF16 (round to nearest even), returned as float64."""
    a = np.asarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32).astype(np.float64)


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    return dict(W1=p[oW1:ob1].reshape(K1, H), b1=p[ob1:oW2], W2=p[oW2:ob2].reshape(H, H),
                b2=p[ob2:oW3], W3=p[oW3:ob3].reshape(H, H), b3=p[ob3:ow4], w4=p[ow4:ob4],
                b4=p[ob4])


def _erf(x):
    from scipy.special import erf
    return erf(x)


def gelu(z):
    return 0.5 * z * (1 + _erf(z / np.sqrt(2)))


def gelu_grad(z):
    return 0.5 * (1 + _erf(z / np.sqrt(2))) + z * np.exp(-0.5 * z * z) / np.sqrt(2 * np.pi)


def init_params(seed=0):
    """He-style initialisation of the hidden layers; zero output layer (c = 1)."""
    rng = np.random.default_rng(seed)
    p = np.zeros(NPARAM)
    P = unpack(p)
    p[oW1:ob1] = 0
    w1 = np.zeros((K1, H))
    w1[:IN] = rng.standard_normal((IN, H)) * np.sqrt(2.0 / IN)
    p[oW1:ob1] = w1.ravel()
    p[oW2:ob2] = (rng.standard_normal((H, H)) * np.sqrt(2.0 / H)).ravel()
    p[oW3:ob3] = (rng.standard_normal((H, H)) * np.sqrt(2.0 / H)).ravel()
    del P
    return p.astype(np.float32)


def forward(p, x):
    """Rows x[n, 6] -> y[n] and the intermediate values."""
    P = unpack(p)
    xb = np.zeros((len(x), K1))
    xb[:, :IN] = bf16(x)
    W1, W2, W3 = bf16(P["W1"]), bf16(P["W2"]), bf16(P["W3"])
    z1 = xb @ W1 + P["b1"]
    h1 = bf16(gelu(z1))
    z2 = h1 @ W2 + P["b2"]
    h2 = bf16(gelu(z2))
    z3 = h2 @ W3 + P["b3"]
    h3 = bf16(gelu(z3))
    y = h3 @ P["w4"] + P["b4"]
    return y, dict(xb=xb, z1=z1, h1=h1, z2=z2, h2=h2, z3=z3, h3=h3, W1=W1, W2=W2, W3=W3)


def loss_and_grad(p, x, a, grp, idx):
    """Mean loss over the groups idx and its gradient (FP64)."""
    P = unpack(p)
    rows = (np.asarray(idx)[:, None] * GROUP + np.arange(GROUP)[None, :]).ravel()
    X, A = x[rows], a[rows].astype(np.float64)
    G = grp[idx].astype(np.float64)
    y, c = forward(p, X)
    cc = np.exp(y).reshape(len(idx), GROUP)
    Ag = A.reshape(len(idx), GROUP, 3)
    f = np.array([1.0, 5.0, 9.0])
    s = np.einsum("gj,gjl->gl", cc, Ag)
    r = f * (s - G[:, 0:3]) - G[:, 3:6]
    inv = (G[:, 6] * G[:, 7] / len(idx))[:, None]
    loss = float((r * r * inv).sum())
    dc = np.einsum("gl,gjl->gj", 2 * r * inv * f, Ag)
    dy = (dc * cc).ravel()
    g = np.zeros(NPARAM)
    dz3 = np.outer(dy, P["w4"]) * gelu_grad(c["z3"])
    g[ow4:ob4] = c["h3"].T @ dy
    g[ob4] = dy.sum()
    g[ob3:ow4] = dz3.sum(0)
    dz3b = bf16(dz3)
    g[oW3:ob3] = (c["h2"].T @ dz3b).ravel()
    dz2 = (dz3b @ c["W3"].T) * gelu_grad(c["z2"])
    g[ob2:oW3] = dz2.sum(0)
    dz2b = bf16(dz2)
    g[oW2:ob2] = (c["h1"].T @ dz2b).ravel()
    dz1 = (dz2b @ c["W2"].T) * gelu_grad(c["z1"])
    g[ob1:oW2] = dz1.sum(0)
    dz1b = bf16(dz1)
    gw1 = c["xb"].T @ dz1b
    gw1[IN:] = 0
    g[oW1:ob1] = gw1.ravel()
    return loss, g
