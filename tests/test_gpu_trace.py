"""Closest-hit traversal on the GPU against brute force.

The oracle: the closest hit of every ray by a brute-force scan with the same
watertight triangle test and the lowest-index tie rule.  The BVH result must
match it bit for bit: the triangle index exactly and t as the same float
(stronger than the 4-ulp bound asked of it).
"""
import numpy as np
import pytest

import lisa_gb300 as L
from lisa_gb300 import scenes
from helpers import random_rays


def _check(prim, t, oprim, ot):
    assert np.array_equal(prim, oprim), f"{(prim != oprim).sum()} of {prim.size} triangle ids differ"
    hit = oprim >= 0
    assert np.array_equal(t[hit].view(np.uint32), ot[hit].view(np.uint32))
    assert np.all(np.isinf(t[~hit]))


@pytest.mark.gpu
def test_cornell_box_1m_rays_vs_cpu_brute_force(gpu, oracle):
    sc = scenes.cornell_box()
    v, _, _ = sc.soup()
    r = L.Renderer(L.params_from_scene(sc))
    rays = random_rays(v, 1_000_000, seed=11, eye=sc.eye)
    prim, t = r.trace_closest(rays)
    oprim, ot = oracle.closest(v, rays, use_bvh=False)
    _check(prim, t, oprim, ot)
    assert (oprim >= 0).mean() > 0.5


@pytest.mark.gpu
def test_displaced_icosphere_vs_cpu_bvh_and_gpu_brute_force(gpu, oracle):
    """~1.3M-triangle mesh: 1M rays against the CPU BVH oracle (itself equal
    to brute force on the small scene above), and a subset against the GPU
    brute-force scan."""
    import ctypes as C

    sc = scenes.icosphere_box(level=8)
    v, _, _ = sc.soup()
    r = L.Renderer(L.params_from_scene(sc, num_samples=1))
    rays = random_rays(v, 1_000_000, seed=12, eye=sc.eye)
    prim, t = r.trace_closest(rays)
    oprim, ot = oracle.closest(v, rays, use_bvh=True)
    _check(prim, t, oprim, ot)
    # GPU brute force on a subset
    import torch  # device buffers only

    sub = torch.from_numpy(rays[:4096].copy()).cuda()
    bp = torch.empty(4096, dtype=torch.int32, device="cuda")
    bt = torch.empty(4096, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    L._native.check(L._native.lib().lisa_trace_brute_device(r.handle, C.c_void_p(sub.data_ptr()), 4096,
                                                            C.c_void_p(bp.data_ptr()), C.c_void_p(bt.data_ptr()),
                                                            None))
    _check(prim[:4096], t[:4096], bp.cpu().numpy(), bt.cpu().numpy())


def test_cpu_bvh_oracle_equals_cpu_brute_force(oracle):
    sc = scenes.cornell_box()
    v, _, _ = sc.soup()
    rays = random_rays(v, 200_000, seed=13, eye=sc.eye)
    a = oracle.closest(v, rays, use_bvh=False)
    b = oracle.closest(v, rays, use_bvh=True)
    _check(b[0], b[1], a[0], a[1])


@pytest.mark.gpu
def test_degenerate_and_empty_cases(gpu):
    # a single triangle, zero-direction rays, rays with tmax before the hit
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    n = np.tile(np.array([0, 0, 1], np.float32), (3, 1))
    mats = np.array([[1, 1, 0, 1, 1, 1, 0, 0, 0, 0]], np.float32)
    p = L.params_from_arrays(v, n, [0], mats, 4, 4, (0, 0, 1), (0, 0, 0), 40, 1, 1)
    r = L.Renderer(p)
    rays = np.array([[0.2, 0.2, 1, 1e-4, 0, 0, -1, 1e16],   # hit at t=1
                     [0.2, 0.2, 1, 1e-4, 0, 0, -1, 0.5],    # tmax before the hit
                     [0.2, 0.2, 1, 1e-4, 0, 0, 0, 1e16],    # zero direction: miss
                     [2.0, 2.0, 1, 1e-4, 0, 0, -1, 1e16],   # outside
                     [0.0, 0.0, 1, 1e-4, 0, 0, -1, 1e16]],  # exactly on a vertex: watertight hit
                    np.float32)
    prim, t = r.trace_closest(rays)
    assert prim.tolist() == [0, -1, -1, -1, 0]
    assert t[0] == 1.0


@pytest.mark.gpu
def test_counting_pass(gpu):
    sc = scenes.cornell_box()
    v, _, _ = sc.soup()
    r = L.Renderer(L.params_from_scene(sc))
    rays = random_rays(v, 10_000, seed=14, eye=sc.eye)
    visits, tests = r.trace_count(rays)
    assert visits >= 10_000 and tests > 0
    info = r.bvh_info()
    assert info["tri_slots"] == sc.num_triangles and info["nodes"] >= 1


@pytest.mark.gpu
def test_sah_refinement_keeps_hits_and_cuts_traversal(gpu, oracle):
    """The SAH treelet restructuring of the LBVH (default) against the plain
    LBVH: closest hits stay bit-exact against the CPU BVH oracle, and the
    traversal does less work (node visits + triangle tests per ray)."""
    sc = scenes.icosphere_box(level=6)
    v, _, _ = sc.soup()
    p = L.params_from_scene(sc)
    rays = random_rays(v, 200_000, seed=5, eye=sc.eye)
    refined = L.Renderer(p)
    plain = L.Renderer(p, bvh_lbvh_only=1)
    oprim, ot = oracle.closest(v, rays, use_bvh=True)
    for r in (refined, plain):
        prim, t = r.trace_closest(rays)
        _check(prim, t, oprim, ot)
    nv_r, nt_r = refined.trace_count(rays)
    nv_p, nt_p = plain.trace_count(rays)
    work_r = 1.2 * nv_r + nt_r
    work_p = 1.2 * nv_p + nt_p
    assert work_r < work_p, (nv_r, nt_r, nv_p, nt_p)
