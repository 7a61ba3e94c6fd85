"""The physically based estimator (opt-in) on the GPU.

Against the oracle's restatement with the same RNG streams every path
agrees (same IEEE operation order), so per-pixel means match up to the
float accumulation and the ray counts are equal.  Against an analytic
answer, direct lighting of a floor by a small square emitter comes out
right.  Guided sampling leaves the expectation unchanged.
"""
import numpy as np
import pytest

import lisa_gb300 as L
from lisa_gb300 import scenes

pytestmark = pytest.mark.gpu
PHYS = L._native.LISA_ESTIMATOR_PHYSICAL
GUIDED = L._native.LISA_MODE_GUIDED


def _oracle_mean(oracle, sc, **kw):
    s, q, rays = oracle.Scene.from_scene(sc, estimator=1, **kw).render(use_bvh=True)
    spp = kw.get("spp", sc.num_samples)
    mean = s / spp
    var = np.maximum(q / spp - mean * mean, 0.0) * spp / max(spp - 1, 1)
    return mean.reshape(sc.height, sc.width, 3), var.reshape(sc.height, sc.width, 3), rays


def _mismatch(a, b, rtol=1e-5):
    return (np.abs(a - b) > rtol * np.maximum(1.0, np.abs(b))).any(axis=2).mean()


def test_path_by_path_cornell_box(gpu, oracle):
    sc = scenes.cornell_box(width=48, height=32, num_samples=4, num_bounces=7)
    r = L.Renderer(L.params_from_scene(sc), estimator=PHYS)
    st = r.render()
    img = r.image()
    ref, _, rays = _oracle_mean(oracle, sc)
    assert _mismatch(img, ref) <= 0.002
    assert st.rays_primary == rays[0]
    assert abs(int(st.rays_bounce) - int(rays[1])) <= 0.002 * rays[1]
    assert abs(int(st.rays_shadow) - int(rays[2])) <= 0.002 * rays[2]
    assert st.device_status == 0
    assert img.mean() > 0


def test_path_by_path_icosphere(gpu, oracle):
    """Dielectric icosphere: refraction, total internal reflection and the
    Fresnel choice on both sides of the surface."""
    sc = scenes.icosphere_box(level=4, width=40, height=40, num_samples=2, num_bounces=8)
    r = L.Renderer(L.params_from_scene(sc), estimator=PHYS)
    st = r.render()
    ref, _, rays = _oracle_mean(oracle, sc)
    assert _mismatch(r.image(), ref) <= 0.002
    assert st.rays_primary == rays[0]
    assert abs(int(st.rays_shadow) - int(rays[2])) <= 0.002 * rays[2]


def _floor_and_light(roughness, spp, bounces=2):
    """Diffuse floor (albedo 0.6, 0.5, 0.4) and a 0.2 x 0.2 emitter
    (5, 4, 3) one unit above, centred 0.3 to the side; one pixel looking at
    the origin."""
    def quad(p0, p1, p2, p3, n):
        return (np.array([p0, p1, p2, p0, p2, p3], np.float32).reshape(2, 9),
                np.tile(np.asarray(n, np.float32), 6).reshape(2, 9))
    fv, fn = quad((-5, 0, -5), (-5, 0, 5), (5, 0, 5), (5, 0, -5), (0, 1, 0))
    lv, ln = quad((0.2, 1, -0.1), (0.4, 1, -0.1), (0.4, 1, 0.1), (0.2, 1, 0.1), (0, -1, 0))
    mats = np.array([[roughness, 1.0, 1.0, 0.6, 0.5, 0.4, 0, 0, 0, 0],
                     [1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1, 5.0, 4.0, 3.0]], np.float32)
    return L.params_from_arrays(np.concatenate([fv, lv]), np.concatenate([fn, ln]),
                                np.array([0, 0, 1, 1], np.int32), mats, 1, 1, (0.0, 0.5, 0.5), (0.0, 0.0, 0.0),
                                0.0005, spp, bounces)


@pytest.mark.parametrize("roughness,bounces", [(1.0, 2), (0.5, 2), (1.0, 1)])
def test_direct_lighting_matches_the_integral(gpu, roughness, bounces):
    """With one bounce the floor is the last vertex; the ray leaving it is
    traced for emission only, so MIS still splits the direct light."""
    spp = 1 << 20
    r = L.Renderer(_floor_and_light(roughness, spp, bounces), estimator=PHYS)
    st = r.render()
    assert st.rays_bounce > 0
    mean, var = r.image(variance=True)
    u = (np.arange(2000) + 0.5) / 2000 * 0.2 - 0.1
    U, V = np.meshgrid(u, u, indexing="ij")
    E = float(np.sum(1.0 / ((0.3 + U) ** 2 + 1.0 + V ** 2) ** 2) * (0.2 / 2000) ** 2)
    expect = roughness * np.array([0.6, 0.5, 0.4]) / np.pi * E * np.array([5.0, 4.0, 3.0])
    sigma = np.sqrt(var[0, 0] / spp)
    assert np.all(np.abs(mean[0, 0] - expect) < 4 * sigma + 1e-7), (mean[0, 0], expect, sigma)


def test_guided_physical_is_unbiased(gpu):
    sc = scenes.cornell_box(width=24, height=24, num_samples=512, num_bounces=5)
    p = L.params_from_scene(sc)
    plain = L.Renderer(p, seed=1, estimator=PHYS)
    plain.render()
    a, va = plain.image(variance=True)
    guided = L.Renderer(p, seed=2, estimator=PHYS, mode=GUIDED, paths_in_flight=24 * 24 * 32)
    st = guided.render()
    b, vb = guided.image(variance=True)
    assert st.launches_guide > 0 and np.isfinite(st.guide_loss)
    n = sc.num_samples
    s = np.sqrt(va / n + vb / n)
    z = np.abs(a - b) / np.maximum(s, 1e-12)
    z[(s == 0) & (a == b)] = 0
    assert (z > 3).mean() < 0.03, (z > 3).mean()
    d = abs(a.mean() - b.mean())
    agg = np.sqrt((va.mean() + vb.mean()) / (n * a[..., 0].size))
    assert d < 4 * agg + 1e-9, (d, agg)
