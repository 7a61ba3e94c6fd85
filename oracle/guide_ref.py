"""ORACLE -- test infrastructure only.

NumPy FP64 restatement of the path-guide network and its training step, used
to check the tensor-core kernels of lisa_gb300/csrc/guide.cu.  The guide has
no counterpart in the reference; its definition is the product's own
(64 -> 4 x 64 ReLU -> 40 = 8 vMF lobes, loss -w log q).  With bf16=True the
oracle rounds to BF16 exactly where the kernels do (inputs, weights,
activations and output gradients that feed a tensor-core product) and keeps
FP32/FP64 elsewhere, so the comparison isolates accumulation-order and
transcendental-function differences.
"""
from __future__ import annotations

import numpy as np

NIN, NH, NOUT = 64, 64, 40
LOBES = 8
P_W5 = 4 * 64 * 64
P_B = P_W5 + 40 * 64
P_B5 = P_B + 4 * 64
NPARAM = P_B5 + 40
KLO, KHI = -4.0, 8.0


def bf16(x):
    """Round to the nearest BF16 (ties to even), returned as float64."""
    a = np.ascontiguousarray(np.asarray(x, np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(p):
    p = np.asarray(p, np.float64)
    W = [p[l * 4096:(l + 1) * 4096].reshape(64, 64) for l in range(4)]
    W.append(p[P_W5:P_W5 + 2560].reshape(40, 64))
    b = [p[P_B + 64 * l:P_B + 64 * (l + 1)] for l in range(4)] + [p[P_B5:P_B5 + 40]]
    return W, b


def forward(p, X, bf=True):
    """Raw outputs (n, 40) and the activations [X, H1..H4] as used."""
    W, b = unpack(p)
    r = bf16 if bf else (lambda x: np.asarray(x, np.float64))
    h = r(X)
    acts = [h]
    for l in range(4):
        z = h @ r(W[l]).T + b[l]
        h = r(np.maximum(z, 0.0))
        acts.append(h)
    out = h @ r(W[4]).T + b[4]
    return out, acts


def decode(o):
    o = np.asarray(o, np.float64).reshape(-1, LOBES, 5)
    raw_mu = o[..., 0:3]
    nrm = np.maximum(np.linalg.norm(raw_mu, axis=-1, keepdims=True), 1e-6)
    mu = raw_mu / nrm
    kappa = np.exp(np.clip(o[..., 3], KLO, KHI))
    lg = o[..., 4] - o[..., 4].max(axis=-1, keepdims=True)
    w = np.exp(lg)
    w /= w.sum(axis=-1, keepdims=True)
    return mu, kappa, w, nrm[..., 0]


def vmf(mu, kappa, d):
    c = np.einsum("nkj,nj->nk", mu, d)
    return kappa / (2 * np.pi * -np.expm1(-2 * kappa)) * np.exp(kappa * (c - 1))


def log_q(o, d):
    mu, kappa, w, _ = decode(o)
    return np.log(np.maximum((w * vmf(mu, kappa, d)).sum(-1), 1e-300))


def loss_and_output_grad(o, d, wt):
    """Per-sample loss -wt log q and its gradient w.r.t. the 40 outputs."""
    o = np.asarray(o, np.float64)
    d = np.asarray(d, np.float64)
    d = d / np.linalg.norm(d, axis=1, keepdims=True)
    mu, kappa, w, nrm = decode(o)
    f = vmf(mu, kappa, d)
    q = np.maximum((w * f).sum(-1), 1e-300)
    r = w * f / q[:, None]
    c = np.einsum("nkj,nj->nk", mu, d)
    dlk = 1 / kappa - 2 / np.expm1(2 * kappa) + (c - 1)
    rawk = o.reshape(-1, LOBES, 5)[..., 3]
    dk = np.where((rawk > KLO) & (rawk < KHI), kappa, 0.0)
    g = np.zeros((o.shape[0], LOBES, 5))
    wt = np.asarray(wt, np.float64)[:, None]
    g[..., 3] = -wt * r * dlk * dk
    gm = -(wt * r * kappa)[..., None] * d[:, None, :]
    dot = (gm * mu).sum(-1, keepdims=True)
    g[..., 0:3] = (gm - dot * mu) / nrm[..., None]
    g[..., 4] = -wt * (r - w)
    return -wt[:, 0] * np.log(q), g.reshape(-1, 40)


def train_grads(p, X, dirs, weights, bf=True):
    """(mean loss, gradient of the mean loss w.r.t. all parameters)."""
    W, b = unpack(p)
    r = bf16 if bf else (lambda x: np.asarray(x, np.float64))
    n = X.shape[0]
    out, acts = forward(p, X, bf)
    loss, g = loss_and_output_grad(out, dirs, np.asarray(weights, np.float64) / n)
    grad = np.zeros(NPARAM)
    dz = np.zeros((n, 64))
    dz[:, :40] = g
    for l in range(4, -1, -1):
        rows = 40 if l == 4 else 64
        dzr = r(dz)
        dW = dzr[:, :rows].T @ acts[l]
        if l == 4:
            grad[P_W5:P_W5 + 2560] = dW.ravel()
            grad[P_B5:P_B5 + 40] = dz[:, :40].sum(0)
        else:
            grad[l * 4096:(l + 1) * 4096] = dW.ravel()
            grad[P_B + 64 * l:P_B + 64 * (l + 1)] = dz.sum(0)
        if l > 0:
            dh = dzr[:, :rows] @ r(W[l])
            dz = np.where(acts[l] > 0, dh, 0.0)
    return float(loss.sum()), grad


def adam(p, m, v, g, lr, step):
    m = 0.9 * m + 0.1 * g
    v = 0.999 * v + 0.001 * g * g
    p = p - lr * (m / (1 - 0.9 ** step)) / (np.sqrt(v / (1 - 0.999 ** step)) + 1e-8)
    return p, m, v
