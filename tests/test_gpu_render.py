"""The wavefront estimator on the GPU against the CPU oracle.

Both restate the reference estimator (src/LiSA/src/shader.cu) with the same
RNG streams and the same IEEE operation order, so at small sizes every path
agrees: per-pixel means equal up to the float accumulation (tolerance
1e-5 relative) and the ray counts are identical.  With different streams
the two are independent estimates of the same image: per-pixel means agree
within 3 sigma (sigma from the per-pixel FP64 variances).
"""
import numpy as np
import pytest

import lisa_gb300 as L
from lisa_gb300 import scenes

pytestmark = pytest.mark.gpu


def oracle_mean(oracle, sc, **kw):
    s, q, rays = oracle.Scene.from_scene(sc, **kw).render(use_bvh=True)
    spp = kw.get("spp", sc.num_samples)
    mean = s / spp
    var = np.maximum(q / spp - mean * mean, 0.0) * spp / max(spp - 1, 1)
    return mean.reshape(sc.height, sc.width, 3), var.reshape(sc.height, sc.width, 3), rays


def mismatch_fraction(a, b, rtol=1e-5):
    bad = np.abs(a - b) > rtol * np.maximum(1.0, np.abs(b))
    return bad.any(axis=2).mean()


def test_path_by_path_cornell_box(gpu, oracle):
    sc = scenes.cornell_box(width=48, height=32, num_samples=4, num_bounces=7)
    r = L.Renderer(L.params_from_scene(sc))
    st = r.render()
    img = r.image()
    ref, _, rays = oracle_mean(oracle, sc)
    assert mismatch_fraction(img, ref) <= 0.002
    assert st.rays_primary == rays[0]
    assert abs(int(st.rays_bounce) - int(rays[1])) <= 0.002 * rays[1]
    assert abs(int(st.rays_shadow) - int(rays[2])) <= 0.002 * rays[2]
    assert st.device_status == 0


def test_path_by_path_hard_indirect(gpu, oracle):
    """A 0.02 x 0.02 light behind a baffle: almost every emitter-search ray
    misses the padded bounds of the emissive triangles and stops at its
    first hit, the rest keep the closest-hit traversal; the search's
    outcomes (and so the paths) must equal the oracle's closest-hit scan."""
    sc = scenes.hard_indirect(level=4, width=32, height=32, num_samples=4, num_bounces=8)
    r = L.Renderer(L.params_from_scene(sc))
    st = r.render()
    img = r.image()
    ref, _, rays = oracle_mean(oracle, sc)
    assert mismatch_fraction(img, ref) <= 0.002
    assert st.rays_primary == rays[0]
    assert abs(int(st.rays_bounce) - int(rays[1])) <= 0.002 * rays[1]
    assert abs(int(st.rays_shadow) - int(rays[2])) <= 0.002 * rays[2]
    assert st.device_status == 0
    assert img.max() > 0


@pytest.mark.parametrize("estimator", ["compat", "physical"])
def test_full_size_frame_band_path_by_path(gpu, oracle, estimator):
    """The bench workload at its full size -- the 1,310,720-triangle
    displaced icosphere in the Cornell box, 1024 x 1024, 8 bounces -- at
    2 spp: four rows across the middle of the GPU frame against the
    oracle's paths for those pixels (its CPU BVH over the whole mesh)."""
    est = L._native.LISA_ESTIMATOR_PHYSICAL if estimator == "physical" else L._native.LISA_ESTIMATOR_COMPAT
    sc = scenes.icosphere_box(level=8, width=1024, height=1024, num_samples=2, num_bounces=8)
    r = L.Renderer(L.params_from_scene(sc), estimator=est)
    st = r.render()
    assert st.device_status == 0
    img = r.image().reshape(-1, 3)
    px0, px1 = 508 * 1024, 512 * 1024
    osc = oracle.Scene.from_scene(sc, estimator=1 if estimator == "physical" else 0)
    s, _, _ = osc.render(px0, px1, use_bvh=True)
    ref = (s / sc.num_samples).astype(np.float32)
    band = img[px0:px1]
    bad = (np.abs(band - ref) > 1e-5 * np.maximum(1.0, np.abs(ref))).any(axis=1)
    assert bad.mean() <= 0.002, bad.mean()
    assert band.max() > 0


def test_full_size_soup_band_path_by_path(gpu, oracle):
    """The soup workload at its full size -- 20,000 spheres, 4,480,000
    triangles, 20,000 materials (2,000 of them emitters), 1920 x 1080,
    12 bounces -- at 1 spp: two rows of the GPU frame against the oracle."""
    sc = scenes.sphere_soup()
    p = L.params_from_scene(sc, num_samples=1)
    r = L.Renderer(p)
    st = r.render()
    assert st.device_status == 0
    img = r.image().reshape(-1, 3)
    px0, px1 = 540 * sc.width, 542 * sc.width
    s, _, _ = oracle.Scene.from_scene(sc, spp=1).render(px0, px1, use_bvh=True)
    band = img[px0:px1]
    bad = (np.abs(band - s) > 1e-5 * np.maximum(1.0, np.abs(s))).any(axis=1)
    assert bad.mean() <= 0.002, bad.mean()
    assert band.max() > 0


def test_path_by_path_reference_stream(gpu, oracle):
    """LISA_RNG_PER_PIXEL: one tea<16>(pixel, subframe) stream per pixel
    shared by its samples, exactly the reference raygen (shader.cu:141-155)."""
    sc = scenes.cornell_box(width=32, height=24, num_samples=3, num_bounces=5)
    r = L.Renderer(L.params_from_scene(sc), rng=L._native.LISA_RNG_PER_PIXEL)
    r.render()
    img = r.image()
    ref, _, _ = oracle_mean(oracle, sc, rng_mode=1)
    assert mismatch_fraction(img, ref) <= 0.002


def test_statistical_agreement_independent_streams(gpu, oracle):
    sc = scenes.cornell_box(width=40, height=40, num_samples=256, num_bounces=7)
    r = L.Renderer(L.params_from_scene(sc), seed=7)
    r.render()
    img, var = r.image(variance=True)
    ref, rvar, _ = oracle_mean(oracle, sc, seed=99)
    n = sc.num_samples
    sigma = np.sqrt(var / n + rvar / n)
    z = np.abs(img - ref) / np.maximum(sigma, 1e-12)
    z[(sigma == 0) & (np.abs(img - ref) == 0)] = 0
    frac = (z > 3).mean()
    assert frac < 0.02, frac
    # the two images are not the same draw
    assert mismatch_fraction(img, ref) > 0.5


def test_progressive_equals_batch(gpu):
    """Two progressive launches of 2 spp equal one batch of 4 spp (same
    sample indices, same Kahan order) -- the reference's subframe lerp
    (shader.cu:160-164) is the running mean."""
    sc = scenes.cornell_box(width=32, height=32, num_samples=4, num_bounces=4)
    a = L.Renderer(L.params_from_scene(sc))
    a.render()
    b = L.Renderer(L.params_from_scene(sc))
    b.render_progressive(2)
    st = b.render_progressive(2)
    assert st.samples_total == 4
    assert np.array_equal(a.image(), b.image())
    b.reset()
    b.render_progressive(4)
    assert np.array_equal(a.image(), b.image())


def test_ppm_payload_and_file(gpu, oracle, tmp_path):
    sc = scenes.cornell_box(width=40, height=30, num_samples=8, num_bounces=5)
    r = L.Renderer(L.params_from_scene(sc, output_image=str(tmp_path / "img.ppm")))
    L.render(r)
    img = r.image()
    rgba = r.rgba8()
    ref = oracle.make_color(img.reshape(-1, 3)).reshape(sc.height, sc.width, 4)
    diff = np.abs(rgba.astype(int) - ref.astype(int))
    assert diff.max() <= 1 and (diff > 0).mean() < 0.01  # device powf vs host powf
    payload = r.ppm_rgb8()
    assert np.array_equal(payload, rgba[::-1, :, :3])
    data = (tmp_path / "img.ppm").read_bytes()
    hdr = f"P6\n{sc.width} {sc.height}\n255\n".encode()
    assert data.startswith(hdr) and data[len(hdr):] == payload.tobytes()


@pytest.mark.parametrize("estimator", [0, 1])
def test_batch_of_uneven_scenes_matches_single_renders(gpu, estimator):
    """Scenes with different bounce counts share waves; with the physically
    based estimator each path's emission-only last ray falls at its own
    scene's depth."""
    a = scenes.cornell_box(width=24, height=16, num_samples=2, num_bounces=3)
    b = scenes.icosphere_box(level=3, width=20, height=20, num_samples=3, num_bounces=5)
    batch = L.Renderer([L.params_from_scene(a), L.params_from_scene(b)], paths_in_flight=700, estimator=estimator)
    batch.render()
    for k, sc in enumerate((a, b)):
        single = L.Renderer(L.params_from_scene(sc), estimator=estimator)
        single.render()
        assert np.array_equal(batch.image(k), single.image()), k


def test_batch_render_one_call_writes_every_scene(gpu, tmp_path):
    """lisa_batch_render: one call renders a batch of uneven scenes and
    writes each scene's PPM to its output_image path -- the same bytes as
    a batch renderer's save_image."""
    import ctypes as C

    a = scenes.cornell_box(width=32, height=24, num_samples=4, num_bounces=5)
    b = scenes.icosphere_box(level=3, width=20, height=16, num_samples=8, num_bounces=6)
    pa = L.params_from_scene(a, output_image=str(tmp_path / "a.ppm"))
    pb = L.params_from_scene(b, output_image=str(tmp_path / "b.ppm"))
    arr = (L._native.RendererParams * 2)(pa.raw, pb.raw)
    opts = L.default_options(seed=3)
    st = L._native.RenderStats()
    L._native.check(L._native.lib().lisa_batch_render(C.cast(arr, C.c_void_p), 2, C.cast(C.byref(opts), C.c_void_p),
                                                      C.cast(C.byref(st), C.c_void_p)))
    assert st.rays_primary == 32 * 24 * 4 + 20 * 16 * 8
    r = L.Renderer([pa, pb], opts)
    r.render()
    for k, name in enumerate(("a", "b")):
        want = tmp_path / f"{name}_want.ppm"
        r.save_image(str(want), scene=k)
        assert (tmp_path / f"{name}.ppm").read_bytes() == want.read_bytes()


def test_cli_renders_the_scene_file(gpu, tmp_path):
    """`lisa -s scene.rto` (LiSA's main: parse, render, save_image) writes
    the same PPM bytes as the library rendering the parsed scene."""
    import os
    import subprocess

    sc = scenes.cornell_box(width=40, height=30, num_samples=8, num_bounces=5)
    sc.output_image = str(tmp_path / "cli.ppm")
    rto = scenes.write_rto(sc, str(tmp_path))
    cli = os.path.join(os.path.dirname(L._native.LIB_PATH), "bin", "lisa")
    run = subprocess.run([cli, "-s", rto, "--seed", "5"], capture_output=True, text=True, timeout=300)
    assert run.returncode == 0, run.stderr
    params = L.SceneParser(rto).get_params()
    r = L.Renderer(params, seed=5)
    r.render()
    want = tmp_path / "lib.ppm"
    r.save_image(str(want))
    assert (tmp_path / "cli.ppm").read_bytes() == want.read_bytes()


def test_cuda_graph_replay_matches_stream_launches(gpu):
    """The captured graph (reused across calls with the same wave shape,
    fresh wave table each call) gives the same image as direct launches."""
    sc = scenes.cornell_box(width=32, height=24, num_samples=3, num_bounces=5)
    a = L.Renderer(L.params_from_scene(sc), use_graph=0, stage_timing=1)
    b = L.Renderer(L.params_from_scene(sc), use_graph=1, stage_timing=1)
    for _ in range(3):
        sa = a.render_progressive(3)
        sb = b.render_progressive(3)
        assert sa.rays == sb.rays and sb.launches_total == sa.launches_total
        assert sb.ms_nee > 0 and sb.ms_trace > 0
    assert np.array_equal(a.image(), b.image())


def test_reused_device_memory_gives_the_same_image(gpu):
    """Renderers created after others were destroyed take their buffers from
    the device-memory cache (blocks that still hold the old contents); the
    images are the same, bit for bit, as from a renderer on fresh memory,
    and lisa_device_cache_release hands the cached blocks back."""
    import ctypes as C

    lib = L._native.lib()
    freed = C.c_uint64()
    L._native.check(lib.lisa_device_cache_release(C.byref(freed)))
    icos = scenes.icosphere_box(level=4, width=64, height=48, num_samples=8, num_bounces=6)
    box = scenes.cornell_box(width=64, height=48, num_samples=8, num_bounces=6)
    first = L.Renderer(L.params_from_scene(icos), seed=5)
    first.render()
    want = first.image()
    first.close()
    for other in (box, icos):  # the cached blocks now hold another scene's state
        r = L.Renderer(L.params_from_scene(other), seed=9)
        r.render()
        r.close()
    again = L.Renderer(L.params_from_scene(icos), seed=5)
    again.render()
    assert np.array_equal(again.image(), want)
    again.close()
    L._native.check(lib.lisa_device_cache_release(C.byref(freed)))
    assert freed.value > 0
    L._native.check(lib.lisa_device_cache_release(C.byref(freed)))
    assert freed.value == 0


def test_wave_splitting_small_capacity(gpu):
    """A capacity smaller than one image plane splits planes into pixel
    ranges; the result is unchanged."""
    sc = scenes.cornell_box(width=37, height=23, num_samples=3, num_bounces=4)
    a = L.Renderer(L.params_from_scene(sc))
    a.render()
    b = L.Renderer(L.params_from_scene(sc), paths_in_flight=100)
    b.render()
    assert np.array_equal(a.image(), b.image())


def test_errors_are_status_codes(gpu):
    sc = scenes.cornell_box(width=8, height=8, num_samples=1)
    v, n, mi = sc.soup()
    mi = mi.copy()
    mi[3] = 99  # material index out of range
    p = L.params_from_arrays(v, n, mi, sc.material_table(), 8, 8, sc.eye, sc.look_at, sc.fov, 1, 2)
    with pytest.raises(L.LisaError) as e:
        L.Renderer(p)
    assert e.value.code == L._native.LISA_ERR_INVALID
    # an allocation cap turns into LISA_ERR_OOM, not a crash
    with pytest.raises(L.LisaError) as e:
        L.Renderer(L.params_from_scene(sc), alloc_cap_bytes=1024)
    assert e.value.code == L._native.LISA_ERR_OOM


def test_path_by_path_sphere_soup_many_materials(gpu, oracle):
    """Sphere soup with 1,500 materials (one per sphere, 10 % emissive):
    per-triangle material indices beyond 8 bits, 12 bounces, both
    estimators against the oracle path by path."""
    sc = scenes.sphere_soup(n_spheres=1500, width=40, height=24, num_samples=2, num_bounces=12,
                            extent=100.0 * (1500 / 20000) ** (1 / 3))
    for est in (0, 1):
        r = L.Renderer(L.params_from_scene(sc), estimator=est)
        st = r.render()
        ref, _, rays = oracle_mean(oracle, sc, estimator=est)
        assert mismatch_fraction(r.image(), ref) <= 0.002
        assert st.rays_primary == rays[0]
        assert st.device_status == 0


@pytest.mark.parametrize("name", ["cornell", "hard_indirect", "rough_mix"])
def test_matches_reference_shader_fixture(gpu, tmp_path, name):
    """The GPU estimator against the reference's own shader programs.

    tests/golden/shader/<name>.txt holds per pixel what the reference's
    shader.cu (run on the host over the reference parser's reading of the
    scene, one RNG stream per pixel, closest hits from a scan) wrote.  The
    scene goes through this library's own front end (.rto + OBJ parsed by
    lisa_scene_parse) and renders with the reference's per-pixel stream:
    every pixel's mean must equal the fixture's up to float accumulation
    (1e-5 relative), and the ray totals must be the fixture's (radiance
    rays of zero direction are not traced here: they are misses)."""
    import os
    import sys

    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, os.path.join(here, "golden"))
    import shader_scenes as S

    sc = S.SCENES[name]()
    _, acc, _, cnt = S.read_fixture(os.path.join(here, "golden", "shader", name + ".txt"))
    rto = scenes.write_rto(sc, str(tmp_path))
    params = L.SceneParser(rto).get_params()
    r = L.Renderer(params, rng=L._native.LISA_RNG_PER_PIXEL)
    st = r.render()
    img = r.image().reshape(-1, 3)
    bad = np.abs(img - acc) > 1e-5 * np.maximum(1.0, np.abs(acc))
    assert bad.any(axis=1).sum() == 0, np.where(bad.any(axis=1))[0][:10]
    assert st.rays_primary + st.rays_bounce == int((cnt[:, 0] - cnt[:, 2]).sum())
    assert st.rays_shadow == int(cnt[:, 1].sum())
    assert st.device_status == 0
    # the reference's own OptiX render of the scene with closest-hit
    # occlusion rays (tests/golden/optix): the same paths except where
    # OptiX's triangle intersector rounds a hit distance differently
    optix = np.fromfile(os.path.join(here, "golden", "optix", name + "_closest.f32"), np.float32).reshape(-1, 3)
    same = (np.abs(optix - img) <= 1e-5 * np.maximum(1.0, np.abs(img))).all(axis=1)
    assert same.mean() >= 0.90, same.mean()


@pytest.mark.parametrize("focal", [0.0, 1.2])
def test_thin_lens_path_by_path(gpu, oracle, focal):
    """The thin-lens option (aperture > 0; the reference's camera is a
    pinhole): the lens point is drawn by rejection from the square with the
    path's own stream, so the oracle traces the same paths.  focal 0 puts
    the focal plane at |look_at - eye|."""
    sc = scenes.cornell_box(width=40, height=32, num_samples=4, num_bounces=5)
    r = L.Renderer(L.params_from_scene(sc), aperture=0.05, focal_distance=focal)
    st = r.render()
    img = r.image()
    ref, _, rays = oracle_mean(oracle, sc, lens_radius=0.05, focal_distance=focal)
    assert mismatch_fraction(img, ref) <= 0.002
    assert st.rays_primary == rays[0]
    pin, _, _ = oracle_mean(oracle, sc)
    assert mismatch_fraction(img, pin) > 0.3  # the lens changes the image
