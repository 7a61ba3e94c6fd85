"""The oracle's physically based estimator against an analytic answer (host
only): a small square emitter above a large diffuse floor, seen through a
narrow camera.  With two radiance traces (camera -> floor -> emitter) the
pixel is the floor's direct-lighting radiance  r * rho / pi * E,  where E is
the irradiance integral of the emitter (computed here by quadrature) and r
the weight of the diffuse lobe; emitter sampling and cosine-weighted
sampling are combined by MIS, so their weights must sum to one for the mean
to come out right."""
import numpy as np
import pytest


def _quad(p0, p1, p2, p3, n):
    v = np.array([p0, p1, p2, p0, p2, p3], np.float32).reshape(2, 9)
    nn = np.tile(np.asarray(n, np.float32), 6).reshape(2, 9)
    return v, nn


def _scene(oracle, roughness, spp, seed=1, bounces=2):
    floor_v, floor_n = _quad((-5, 0, -5), (-5, 0, 5), (5, 0, 5), (5, 0, -5), (0, 1, 0))
    cx, h, s = 0.3, 1.0, 0.2
    light_v, light_n = _quad((cx - s / 2, h, -s / 2), (cx + s / 2, h, -s / 2), (cx + s / 2, h, s / 2),
                             (cx - s / 2, h, s / 2), (0, -1, 0))
    v = np.concatenate([floor_v, light_v])
    n = np.concatenate([floor_n, light_n])
    mi = np.array([0, 0, 1, 1], np.int32)
    # rows: roughness, alpha, n, diffuse rgb, emit, emission rgb
    mats = np.array([[roughness, 1.0, 1.0, 0.6, 0.5, 0.4, 0, 0, 0, 0],
                     [1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1, 5.0, 4.0, 3.0]], np.float32)
    sc = oracle.Scene(v, n, mi, mats, width=1, height=1, eye=(0.0, 0.5, 0.5), look_at=(0.0, 0.0, 0.0),
                      fov=0.0005, spp=spp, bounces=bounces, seed=seed, estimator=1)
    return sc, (cx, h, s)


def _irradiance(cx, h, s, m=2000):
    u = (np.arange(m) + 0.5) / m * s - s / 2
    U, V = np.meshgrid(u, u, indexing="ij")
    d2 = (cx + U) ** 2 + h * h + V ** 2
    return float(np.sum(h * h / d2 ** 2) * (s / m) ** 2)  # cos_x cos_y / d^2 = h^2 / d^4


@pytest.mark.parametrize("roughness,bounces", [(1.0, 2), (0.5, 2), (1.0, 1)])
def test_direct_lighting_matches_the_integral(oracle, roughness, bounces):
    """Emitter sampling and the traced bounce share the direct light by
    MIS.  With one bounce the floor is the last vertex: the ray leaving it is
    still traced, for the emission it reaches only, so the two weights still
    sum to one."""
    spp = 40000
    sc, (cx, h, s) = _scene(oracle, roughness, spp, bounces=bounces)
    total, sq, rays = sc.render(use_bvh=True)
    mean = total[0] / spp
    var = np.maximum(sq[0] / spp - mean ** 2, 0.0)
    E = _irradiance(cx, h, s)
    expect = roughness * np.array([0.6, 0.5, 0.4]) / np.pi * E * np.array([5.0, 4.0, 3.0])
    sigma = np.sqrt(var / spp)
    assert np.all(np.abs(mean - expect) < 4 * sigma + 1e-6), (mean, expect, sigma)
    assert rays[0] == spp and rays[1] > 0 and rays[2] > 0  # the floor's bounce is traced


def test_independent_streams_agree(oracle):
    """Two independent streams give different draws with the same mean."""
    a, _ = _scene(oracle, 1.0, 20000, seed=3)
    b, _ = _scene(oracle, 1.0, 20000, seed=4)
    ta, qa, _ = a.render()
    tb, qb, _ = b.render()
    ma, mb = ta[0] / 20000, tb[0] / 20000
    sa = np.sqrt(np.maximum(qa[0] / 20000 - ma ** 2, 0) / 20000)
    sb = np.sqrt(np.maximum(qb[0] / 20000 - mb ** 2, 0) / 20000)
    assert np.all(np.abs(ma - mb) < 4 * np.sqrt(sa ** 2 + sb ** 2) + 1e-6)
    assert not np.array_equal(ta, tb)
