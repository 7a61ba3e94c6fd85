"""Guide network on the tensor cores against the NumPy oracle.

Forward outputs, training-loss gradients (FP32 gradients from BF16
tensor-core products) and the Adam update are compared with
oracle/guide_ref.py, which rounds to BF16 at the same points, so only the
FP32 accumulation order differs (and, rarely, a BF16 rounding of an
activation that this order tips).  Tolerances, about three times the
errors measured on a GB300 (forward 5.9e-4 of the output scale, gradient
blocks 3.2e-4 relative at worst): outputs within 2e-3 of their scale;
per-block gradient cosine similarity >= 1 - 1e-6 and relative L2 error
<= 1e-3.
"""
import numpy as np
import pytest

import lisa_gb300 as L
from oracle import guide_ref as G

pytestmark = pytest.mark.gpu


def _params(seed, scale=0.15):
    rng = np.random.default_rng(seed)
    p = rng.normal(0, scale, G.NPARAM).astype(np.float32)
    return p


def _batch(n, seed):
    rng = np.random.default_rng(seed)
    X = rng.normal(0, 1, (n, 64)).astype(np.float32)
    d = rng.normal(0, 1, (n, 3)).astype(np.float32)
    w = rng.uniform(0.1, 2.0, n).astype(np.float32)
    return X, d, w


BLOCKS = [("W1", 0, 4096), ("W2", 4096, 8192), ("W3", 8192, 12288), ("W4", 12288, 16384),
          ("W5", G.P_W5, G.P_B), ("b1-4", G.P_B, G.P_B5), ("b5", G.P_B5, G.NPARAM)]


def test_forward_matches_oracle(gpu):
    g = L.Guide(seed=1)
    p = _params(2)
    g.set_params(p)
    assert np.array_equal(g.params(), p)
    X, _, _ = _batch(1000, 3)  # not a multiple of 128: a ragged last tile
    out = g.forward(X)
    ref, _ = G.forward(p, X, bf=True)
    scale = np.abs(ref).max()
    err = np.abs(out - ref).max() / scale
    assert err < 2e-3, err
    assert np.corrcoef(out.ravel(), ref.ravel())[0, 1] > 0.9999


def test_training_gradients_match_oracle(gpu):
    g = L.Guide(seed=1)
    p = _params(4)
    g.set_params(p)
    X, d, w = _batch(1024, 5)
    loss, grads = g.train_step(X, d, w, lr=0.0)
    rloss, rg = G.train_grads(p, X, d, w, bf=True)
    assert abs(loss - rloss) <= 1e-3 * abs(rloss) + 1e-4, (loss, rloss)
    for name, a, b in BLOCKS:
        x, y = grads[a:b].astype(np.float64), rg[a:b]
        cos = x @ y / (np.linalg.norm(x) * np.linalg.norm(y) + 1e-30)
        rel = np.linalg.norm(x - y) / (np.linalg.norm(y) + 1e-30)
        assert cos >= 1.0 - 1e-6 and rel <= 1e-3, (name, cos, rel)


def test_adam_update(gpu):
    g = L.Guide(seed=1)
    p = _params(6)
    g.set_params(p)
    X, d, w = _batch(256, 7)
    _, grads = g.train_step(X, d, w, lr=1e-2)
    after = g.params()
    ref, _, _ = G.adam(p.astype(np.float64), 0.0, 0.0, grads.astype(np.float64), 1e-2, 1)
    np.testing.assert_allclose(after, ref, rtol=1e-5, atol=1e-6)


def test_train_steps_equal_step_by_step_training(gpu):
    """Several Adam steps in one cooperative launch (the renderer's training
    path) against one train_step launch pair per slice: every CTA's
    gradient goes to its own slot and the slots are summed in the same
    order, so the parameters agree bit for bit.  Three slices of 1,024
    samples with eight steps asked for: the steps end with the samples."""
    p = _params(8)
    X, d, w = _batch(3 * 1024, 9)
    a = L.Guide(seed=1)
    a.set_params(p)
    loss_a = a.train_steps(X, d, w, chunk=1024, steps=8, lr=1e-2)
    b = L.Guide(seed=1)
    b.set_params(p)
    for k in range(3):
        sl = slice(1024 * k, 1024 * (k + 1))
        loss_b, _ = b.train_step(X[sl], d[sl], w[sl], lr=1e-2, want_grads=False)
    assert not np.array_equal(a.params(), p)
    assert np.array_equal(a.params(), b.params())
    # the loss of the last step (summed in another order)
    assert abs(loss_a - loss_b) <= 1e-5 * abs(loss_b) + 1e-6, (loss_a, loss_b)


def test_training_learns_a_direction_distribution(gpu):
    """Samples whose direction depends on the features: training with the
    kernels' own gradients raises the likelihood of held-out samples."""
    rng = np.random.default_rng(9)
    g = L.Guide(seed=3)

    def make(n):
        X = np.zeros((n, 64), np.float32)
        a = rng.uniform(-1, 1, n).astype(np.float32)
        X[:, 0] = a
        X[:, 1] = 1.0
        mean = np.stack([np.cos(a * 1.5), np.sin(a * 1.5), np.zeros(n)], 1)
        d = mean + 0.15 * rng.normal(size=(n, 3))
        return X, d.astype(np.float32), np.ones(n, np.float32)

    Xt, dt, wt = make(2048)

    def heldout_loss():
        out = g.forward(Xt)
        return float(-G.log_q(out, dt / np.linalg.norm(dt, axis=1, keepdims=True)).mean())

    before = heldout_loss()
    for _ in range(300):
        X, d, w = make(1024)
        g.train_step(X, d, w, lr=1e-2, want_grads=False)
    after = heldout_loss()
    assert after < before - 1.0, (before, after)
