"""Pins the CPU oracle against golden vectors of the reference's own code.

tests/golden/ref_math.txt holds outputs of the reference's device helpers
compiled on the host from its sources (oracle/ref_kernels_dump.cc:
random.h, vec_math.h, maths.cu, bsdfs/lambertian.cu, helpers.h,
Camera.cpp).  The oracle restates those functions; this test shows the
restatement computes the same values: bit for bit where the arithmetic is
the same, within a stated tolerance where the oracle deliberately differs
(pow(x,2)/pow(x,5) as products and pi as a float constant, where the
host-compiled reference rounds through double).
"""
import ctypes as C
import os
import struct

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden", "ref_math.txt")


def f(h: str) -> float:
    return struct.unpack("<f", struct.pack("<I", int(h, 16)))[0]


def fa(hs):
    return np.array([f(h) for h in hs], np.float32)


def records(name):
    with open(GOLD) as fh:
        for line in fh:
            parts = line.split()
            if parts and parts[0] == name:
                yield parts[1:]


def ptr(a):
    return C.c_void_p(a.ctypes.data)


def test_golden_file_complete():
    names = {}
    with open(GOLD) as fh:
        for line in fh:
            names[line.split()[0]] = names.get(line.split()[0], 0) + 1
    for k in ("tea16", "rnd", "normalize", "reflect", "faceforward", "lerp", "fresnel", "refract", "brdf",
              "bounce0", "barynormal", "make_color", "uvw"):
        assert names.get(k, 0) > 0, k


def test_tea16(oracle):
    L = oracle.lib()
    n = 0
    for a, b, v in records("tea16"):
        assert L.oracle_tea16(int(a, 16), int(b, 16)) == int(v, 16)
        n += 1
    assert n >= 40


def test_rnd_stream(oracle):
    L = oracle.lib()
    for rec in records("rnd"):
        s = C.c_uint32(int(rec[0], 16))
        got = [L.oracle_rnd(C.byref(s)) for _ in range(8)]
        assert np.array_equal(np.array(got, np.float32), fa(rec[1:9]))
        assert s.value == int(rec[9], 16)


def test_vector_helpers_bit_exact(oracle):
    L = oracle.lib()
    out = np.empty(3, np.float32)
    for rec in records("normalize"):
        a = fa(rec[0:3])
        L.oracle_normalize(ptr(a), ptr(out))
        assert np.array_equal(out, fa(rec[3:6]))
    for rec in records("reflect"):
        a, b = fa(rec[0:3]), fa(rec[3:6])
        L.oracle_reflect(ptr(a), ptr(b), ptr(out))
        assert np.array_equal(out, fa(rec[6:9]))
    for rec in records("faceforward"):
        a, b = fa(rec[0:3]), fa(rec[3:6])
        L.oracle_faceforward(ptr(a), ptr(b), ptr(a), ptr(out))
        assert np.array_equal(out, fa(rec[6:9]))
    for rec in records("lerp"):
        a, b, t = fa(rec[0:3]), fa(rec[3:6]), f(rec[6])
        L.oracle_lerp(ptr(a), ptr(b), C.c_float(t), ptr(out))
        assert np.array_equal(out, fa(rec[7:10]))


def test_fresnel_within_tolerance(oracle):
    # reference: pow() in double on the host (fast-math __powf on the GPU);
    # oracle: products in float.  Tolerance 4e-7 absolute on values in [0,1].
    L = oracle.lib()
    for rec in records("fresnel"):
        c, eta, ref = f(rec[0]), f(rec[1]), f(rec[2])
        assert abs(L.oracle_fresnel(C.c_float(c), C.c_float(eta)) - ref) <= 4e-7


def test_refract_bit_exact(oracle):
    L = oracle.lib()
    out = np.empty(3, np.float32)
    for rec in records("refract"):
        cosI, d, n, eta = f(rec[0]), fa(rec[1:4]), fa(rec[4:7]), f(rec[7])
        L.oracle_refract(C.c_float(cosI), ptr(d), ptr(n), C.c_float(eta), ptr(out))
        assert np.array_equal(out, fa(rec[8:11]))


def test_brdf_within_tolerance(oracle):
    # reference divides by M_PI in double; oracle by pi rounded to float.
    L = oracle.lib()
    for rec in records("brdf"):
        n, l_, ref = fa(rec[0:3]), fa(rec[3:6]), f(rec[6])
        got = L.oracle_brdf(ptr(n), ptr(l_))
        assert abs(got - ref) <= 2.0 * np.spacing(np.float32(max(abs(ref), 1e-30)))


def test_bounce_roughness0_and_stream(oracle):
    """bounce() with roughness 0 is the mirror direction and still consumes
    the three hemisphere draws (lambertian.cu:7-13)."""
    L = oracle.lib()
    out = np.empty(3, np.float32)
    for i, rec in enumerate(records("bounce0")):
        d, n = fa(rec[0:3]), fa(rec[3:6])
        L.oracle_reflect(ptr(d), ptr(n), ptr(out))
        assert np.array_equal(out, fa(rec[6:9]))
        s = C.c_uint32(1000 + i)
        hemi = np.empty(3, np.float32)
        L.oracle_hemi(ptr(n), C.byref(s), ptr(hemi))
        assert s.value == int(rec[9], 16)


def test_barycentric_normal_bit_exact(oracle):
    L = oracle.lib()
    out = np.empty(3, np.float32)
    for rec in records("barynormal"):
        p, n9, v9 = fa(rec[0:3]), fa(rec[3:12]), fa(rec[12:21])
        L.oracle_barycentric_normal(ptr(p), ptr(n9), ptr(v9), ptr(out))
        assert np.array_equal(out, fa(rec[21:24]))


def test_make_color_bit_exact(oracle):
    rgb = np.stack([fa(rec[0:3]) for rec in records("make_color")])
    ref = np.array([[int(x, 16) for x in rec[3:7]] for rec in records("make_color")], np.uint8)
    assert np.array_equal(oracle.make_color(rgb), ref)


def test_camera_frame_bit_exact(oracle):
    L = oracle.lib()
    out = np.empty(9, np.float32)
    for rec in records("uvw"):
        eye, look, fov = fa(rec[0:3]), fa(rec[3:6]), f(rec[6])
        w, h = int(rec[7]), int(rec[8])
        L.oracle_uvw(ptr(eye), ptr(look), C.c_float(fov), w, h, ptr(out))
        assert np.array_equal(out, fa(rec[9:18]))


# ---- the estimator loop against the reference's own shader programs ---------

SHADER_DIR = os.path.join(HERE, "golden", "shader")


def _shader_scenes():
    import sys

    sys.path.insert(0, os.path.join(HERE, "golden"))
    import shader_scenes

    return shader_scenes


@pytest.mark.parametrize("name", ["cornell", "hard_indirect", "rough_mix"])
def test_estimator_matches_reference_shader(oracle, name):
    """The oracle's estimator against the reference's shader.cu itself.

    tests/golden/shader/<name>.txt holds, per pixel, what the reference's
    raygen / closest-hit / miss programs (src/LiSA/src/shader.cu:102-255,
    with lambertian.cu, maths.cu, random.h) wrote when run on the host over
    the reference SceneParser's reading of the scene (one stream per pixel,
    subframe 0, all spp in one launch as render.cc:133-148 does), with
    closest hits from the oracle's scan.  The oracle in its per-pixel
    stream mode must trace the same paths: the same number of radiance and
    occlusion rays in every pixel (the reference also traces a ray of zero
    direction, which the oracle counts as a miss without tracing it) and
    the same mean.  The means may differ by rounding: the reference
    accumulates samples in float and its BRDF and Schlick terms round
    through double on the host; tolerance 1e-5 relative."""
    S = _shader_scenes()
    sc = S.SCENES[name]()
    h, acc, _, cnt = S.read_fixture(os.path.join(SHADER_DIR, name + ".txt"))
    assert h["soup"] == S.soup_hash(sc), "scene generator changed since the fixture was made"
    assert (h["width"], h["height"], h["spp"], h["bounces"]) == (sc.width, sc.height, sc.num_samples,
                                                                  sc.num_bounces)
    osc = oracle.Scene.from_scene(sc, rng_mode=1, subframe=0)
    npix = sc.width * sc.height
    mean = np.empty((npix, 3), np.float32)
    rays = np.empty((npix, 3), np.int64)
    for p in range(npix):
        s, _, r = osc.render(px0=p, px1=p + 1, threads=1)
        mean[p] = s[0] / sc.num_samples
        rays[p] = r.astype(np.int64)
    assert np.array_equal(rays[:, 0] + rays[:, 1], cnt[:, 0] - cnt[:, 2]), "radiance rays differ"
    assert np.array_equal(rays[:, 2], cnt[:, 1]), "occlusion rays differ"
    assert np.all(np.abs(mean - acc) <= 1e-5 * np.maximum(1.0, np.abs(acc)))
    assert (acc.sum(axis=1) > 0).sum() >= 20  # the scene is lit
    assert cnt[:, 1].sum() > 10 * npix  # and the emitter search ran


# ---- the oracle against the reference's own OptiX render on a GB300 --------

OPTIX_DIR = os.path.join(HERE, "golden", "optix")


def _optix_fixture(name, tag):
    return np.fromfile(os.path.join(OPTIX_DIR, f"{name}_{tag}.f32"), np.float32).reshape(-1, 3)


@pytest.mark.parametrize("name", ["cornell", "hard_indirect", "rough_mix"])
def test_oracle_matches_optix_render(oracle, name):
    """The oracle against the reference's own OptiX pipeline run on a GB300.

    tests/golden/optix/ holds the accumulation buffers that the reference's
    optix_wrapper.cc set-up and shader.cu (compiled with its own nvcc flags)
    produced on the fixture scenes (baseline/make_optix_fixtures.py):

    * ``closest``: shader.cu with its occlusion rays traced for the closest
      hit.  Path by path the same estimator as the oracle: at least 90 % of
      the pixels equal the oracle's to 1e-5 (93-100 % measured; the rest
      diverge where OptiX's closed triangle intersector returns a hit
      distance a few ulps from the watertight test's -- the build without
      fast math agrees no better), and the image means agree to 3 %.  This
      also shows that the device code draws make_float3(rng, rng, rng) left
      to right, as the oracle reads it.
    * ``stock``: shader.cu as shipped, occlusion rays terminating on the
      first hit OptiX finds (shader.cu:69).  That hit may be a surface behind
      the light (the ceiling 1e-3 above the Cornell light quad), which leaves
      the emitter flag unset: the stock render is 29-53 % darker than the
      closest-hit reading, an implementation-defined result of the
      reference that no other traversal reproduces."""
    S = _shader_scenes()
    sc = S.SCENES[name]()
    with open(os.path.join(OPTIX_DIR, "summary.json")) as fh:
        import json

        assert json.load(fh)[name]["soup"] == S.soup_hash(sc)
    osc = oracle.Scene.from_scene(sc, rng_mode=1, subframe=0)
    s, _, _ = osc.render()
    mean = (s / sc.num_samples).astype(np.float32)
    closest = _optix_fixture(name, "closest")
    same = (np.abs(closest - mean) <= 1e-5 * np.maximum(1.0, np.abs(mean))).all(axis=1)
    assert same.mean() >= 0.90, same.mean()
    assert abs(closest.mean() / mean.mean() - 1.0) < 0.03
    stock = _optix_fixture(name, "stock")
    assert stock.mean() < 0.8 * closest.mean()
