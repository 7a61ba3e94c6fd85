"""Shared test helpers: seeded ray sets for traversal checks."""
import numpy as np


def random_rays(vertices: np.ndarray, n: int, seed: int, eye=None) -> np.ndarray:
    """n rays (ox oy oz tmin dx dy dz tmax) against a soup: a third from
    random points of the (inflated) bounding box in random directions, a
    third from random points on random triangles (tmin 1e-4, like bounce
    and shadow rays), a third from the camera through the box, with a few
    axis-aligned and unnormalised directions mixed in."""
    rng = np.random.default_rng(seed)
    v = vertices.reshape(-1, 3)
    lo, hi = v.min(0), v.max(0)
    ext = np.maximum(hi - lo, 1e-3)
    k1 = n // 3
    k2 = n // 3
    k3 = n - k1 - k2
    o1 = lo - 0.1 * ext + rng.random((k1, 3)) * 1.2 * ext
    tri = v.reshape(-1, 3, 3)
    idx = rng.integers(0, tri.shape[0], k2)
    a, b = rng.random(k2), rng.random(k2)
    flip = a + b > 1
    a[flip], b[flip] = 1 - a[flip], 1 - b[flip]
    o2 = tri[idx, 0] + a[:, None] * (tri[idx, 1] - tri[idx, 0]) + b[:, None] * (tri[idx, 2] - tri[idx, 0])
    if eye is None:
        eye = (lo + hi) / 2 + np.array([0, 0, 2.0]) * ext.max()
    o3 = np.broadcast_to(np.asarray(eye, np.float64), (k3, 3))
    d12 = rng.normal(size=(k1 + k2, 3))
    d12 /= np.linalg.norm(d12, axis=1, keepdims=True)
    targets = lo + rng.random((k3, 3)) * ext
    d3 = targets - o3
    d3 /= np.linalg.norm(d3, axis=1, keepdims=True)
    o = np.concatenate([o1, o2, o3]).astype(np.float32)
    d = np.concatenate([d12, d3])
    # some axis-aligned and some unnormalised directions
    m = rng.random(n) < 0.01
    ax = rng.integers(0, 3, n)
    d[m] = 0.0
    d[m, ax[m]] = np.where(rng.random(m.sum()) < 0.5, -1.0, 1.0)
    scale = np.where(rng.random(n) < 0.1, rng.uniform(0.1, 3.0, n), 1.0)
    d = (d * scale[:, None]).astype(np.float32)
    rays = np.empty((n, 8), np.float32)
    rays[:, 0:3] = o
    rays[:, 3] = 1e-4
    rays[:, 4:7] = d
    rays[:, 7] = 1e16
    return rays
