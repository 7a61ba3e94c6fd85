"""The NumPy guide oracle is itself checked before it checks the GPU:
finite differences of its loss, and torch autograd in FP64 (CPU)."""
import numpy as np
import pytest

from oracle import guide_ref as G


def _problem(n=16, seed=0):
    rng = np.random.default_rng(seed)
    p = rng.normal(0, 0.15, G.NPARAM)
    X = rng.normal(0, 1, (n, 64))
    d = rng.normal(0, 1, (n, 3))
    w = rng.uniform(0.1, 2.0, n)
    return p, X, d, w


def test_finite_differences_fp64():
    p, X, d, w = _problem()
    _, g = G.train_grads(p, X, d, w, bf=False)
    rng = np.random.default_rng(1)
    idx = np.concatenate([rng.integers(0, G.P_W5, 12), rng.integers(G.P_W5, G.P_B, 6),
                          rng.integers(G.P_B, G.NPARAM, 8)])
    eps = 1e-6
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += eps
        pm[i] -= eps
        lp, _ = G.train_grads(pp, X, d, w, bf=False)
        lm, _ = G.train_grads(pm, X, d, w, bf=False)
        fd = (lp - lm) / (2 * eps)
        assert abs(fd - g[i]) <= 1e-6 + 1e-4 * abs(fd), (i, fd, g[i])


def test_torch_autograd_fp64():
    torch = pytest.importorskip("torch")
    p, X, d, w = _problem(n=32, seed=3)
    _, g = G.train_grads(p, X, d, w, bf=False)
    P = torch.tensor(p, dtype=torch.float64, requires_grad=True)
    Wl = [P[l * 4096:(l + 1) * 4096].view(64, 64) for l in range(4)] + [P[G.P_W5:G.P_W5 + 2560].view(40, 64)]
    bl = [P[G.P_B + 64 * l:G.P_B + 64 * (l + 1)] for l in range(4)] + [P[G.P_B5:G.P_B5 + 40]]
    h = torch.tensor(X)
    for l in range(4):
        h = torch.relu(h @ Wl[l].T + bl[l])
    o = (h @ Wl[4].T + bl[4]).view(-1, 8, 5)
    mu = o[..., :3] / torch.clamp(o[..., :3].norm(dim=-1, keepdim=True), min=1e-6)
    kap = torch.exp(torch.clamp(o[..., 3], G.KLO, G.KHI))
    pi = torch.softmax(o[..., 4], dim=-1)
    dd = torch.tensor(d / np.linalg.norm(d, axis=1, keepdims=True))
    c = (mu * dd[:, None, :]).sum(-1)
    f = kap / (2 * np.pi * -torch.expm1(-2 * kap)) * torch.exp(kap * (c - 1))
    loss = -(torch.tensor(w) / len(w) * torch.log((pi * f).sum(-1))).sum()
    loss.backward()
    np.testing.assert_allclose(P.grad.numpy(), g, rtol=1e-7, atol=1e-10)


def test_bf16_rounding():
    # 1 + 2^-8 and 1 + 3*2^-8 are halfway cases: ties go to the even mantissa
    x = np.array([1.0, 1.00390625, 1.01171875, 1.001953125, -2.5], np.float32)
    r = G.bf16(x)
    assert r.tolist() == [1.0, 1.0, 1.015625, 1.0, -2.5]
