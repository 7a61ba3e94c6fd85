"""lisa_trace_soup_noalloc: closest hits without any device allocation.

Callers that cannot call cudaMalloc/cudaFree at query time (a plugin whose
host application's allocator owns the device memory, or a per-frame loop
that cannot take cudaFree's device-wide synchronisation) use this entry
point: the BVH is built in a scratch array compiled into the library.  Its
results must equal those of the renderer-based lisa_trace_closest_device on
the same triangles and rays, bit for bit, on consecutive calls over
different soups (the shared scratch keeps the previous call's contents).

This file is named so that pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

import lisa_gb300 as L
from lisa_gb300 import scenes
from helpers import random_rays

N = L._native


def _dev(a):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _reference_hits(sc, rays_d, n, params=None):
    import torch

    r = L.Renderer(params if params is not None else L.params_from_scene(sc, num_samples=1))
    prim = torch.empty(n, dtype=torch.int32, device="cuda")
    t = torch.empty(n, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    N.check(N.lib().lisa_trace_closest_device(r.handle, C.c_void_p(rays_d.data_ptr()), n,
                                              C.c_void_p(prim.data_ptr()), C.c_void_p(t.data_ptr()), None))
    out = prim.cpu().numpy(), t.cpu().numpy()
    r.close()
    return out


def _noalloc_hits(verts_d, ntri, rays_d, n):
    import torch

    prim = torch.full((n,), -7, dtype=torch.int32, device="cuda")
    t = torch.zeros(n, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    N.check(N.lib().lisa_trace_soup_noalloc(C.c_void_p(verts_d.data_ptr()), ntri, C.c_void_p(rays_d.data_ptr()), n,
                                            C.c_void_p(prim.data_ptr()), C.c_void_p(t.data_ptr()), None))
    return prim.cpu().numpy(), t.cpu().numpy()


@pytest.mark.gpu
def test_noalloc_matches_renderer_trace_on_consecutive_calls(gpu):
    box = scenes.cornell_box()
    ball = scenes.icosphere_box(level=5)  # 20,492 triangles
    for sc, seed in ((box, 21), (ball, 22), (box, 23)):
        v, _, _ = sc.soup()
        rays = random_rays(v, 200_000, seed=seed, eye=sc.eye)
        rays_d = _dev(rays)
        verts_d = _dev(v.reshape(-1))
        got_p, got_t = _noalloc_hits(verts_d, sc.num_triangles, rays_d, rays.shape[0])
        ref_p, ref_t = _reference_hits(sc, rays_d, rays.shape[0])
        assert np.array_equal(got_p, ref_p)
        hit = ref_p >= 0
        assert hit.mean() > 0.3
        assert np.array_equal(got_t[hit].view(np.uint32), ref_t[hit].view(np.uint32))
        assert np.all(np.isinf(got_t[~hit]))


@pytest.mark.gpu
def test_noalloc_at_the_triangle_limit(gpu):
    """A soup of exactly 65,536 triangles (the limit) fits the scratch and
    gives the renderer's hits bit for bit."""
    sc = scenes.icosphere_box(level=6)  # 81,932 triangles, cut to the limit
    v, n, mi = sc.soup()
    T = 65536
    v, n, mi = v[:3 * T], n[:3 * T], mi[:T]
    params = L.params_from_arrays(v, n, mi, sc.material_table(), 64, 64, sc.eye, sc.look_at, sc.fov, 1, 2)
    rays = random_rays(v, 100_000, seed=31, eye=sc.eye)
    rays_d = _dev(rays)
    got_p, got_t = _noalloc_hits(_dev(v.reshape(-1)), T, rays_d, rays.shape[0])
    ref_p, ref_t = _reference_hits(sc, rays_d, rays.shape[0], params=params)
    assert np.array_equal(got_p, ref_p)
    hit = ref_p >= 0
    assert hit.mean() > 0.3
    assert np.array_equal(got_t[hit].view(np.uint32), ref_t[hit].view(np.uint32))


@pytest.mark.gpu
def test_noalloc_empty_soup_and_no_rays(gpu):
    """No triangles: every ray misses (prim -1, t = inf).  No rays: the
    call succeeds and writes nothing."""
    import torch

    rays = random_rays(scenes.cornell_box().soup()[0], 1000, seed=5)
    rays_d = _dev(rays)
    dummy = torch.zeros(9, dtype=torch.float32, device="cuda")
    got_p, got_t = _noalloc_hits(dummy, 0, rays_d, rays.shape[0])
    assert np.all(got_p == -1) and np.all(np.isinf(got_t))
    prim = torch.full((4,), -7, dtype=torch.int32, device="cuda")
    t = torch.zeros(4, dtype=torch.float32, device="cuda")
    p = C.c_void_p
    N.check(N.lib().lisa_trace_soup_noalloc(p(dummy.data_ptr()), 1, p(rays_d.data_ptr()), 0, p(prim.data_ptr()),
                                            p(t.data_ptr()), None))
    torch.cuda.synchronize()
    assert np.all(prim.cpu().numpy() == -7)


@pytest.mark.gpu
def test_noalloc_rejects_oversized_soup(gpu):
    import torch

    dummy = torch.zeros(16, dtype=torch.float32, device="cuda")
    p = C.c_void_p(dummy.data_ptr())
    code = N.lib().lisa_trace_soup_noalloc(p, 65537, p, 1, p, p, None)
    assert code == N.LISA_ERR_INVALID
    assert b"exceeds the no-allocation limit of 65536" in N.lib().lisa_last_error()
