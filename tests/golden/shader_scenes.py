"""Scenes of the estimator fixtures (tests/golden/shader/*.txt).

The fixtures hold what the reference's own shader programs
(src/LiSA/src/shader.cu, run on the host by oracle/ref_shader_run.cc over
the reference SceneParser's reading of each scene written as .rto + OBJ)
produce per pixel.  Tests rebuild the same scenes from these seeded
constructors; ``soup_hash`` ties a rebuilt scene to the fixture (the
fixture header carries the hash of the soup the reference parsed).
"""
from __future__ import annotations

import numpy as np

from lisa_gb300 import scenes


def cornell():
    """The small Cornell box: Lambertian walls, a white box, a dielectric
    box (n = 1.5), a UV sphere, a ceiling light."""
    return scenes.cornell_box(width=32, height=24, num_samples=8, num_bounces=7)


def hard_indirect():
    """The hard-indirect scene at icosphere level 3: a 0.02 light behind a
    baffle, so most 30-ray emitter searches fail; a dielectric icosphere."""
    return scenes.hard_indirect(level=3, width=32, height=24, num_samples=8, num_bounces=8)


def rough_mix():
    """Cornell box with glossy materials (roughness 0 and 0.3, the bounce's
    reflect/hemisphere lerp) and a tinted dielectric with n = 1.33 (its
    colour attenuates paths leaving it)."""
    sc = scenes.cornell_box(width=32, height=24, num_samples=8, num_bounces=6)
    sc.materials.append(scenes.Material("mirror", (0.9, 0.9, 0.9), roughness=0.0))
    sc.materials.append(scenes.Material("gloss", (0.8, 0.6, 0.2), roughness=0.3))
    sc.materials.append(scenes.Material("water", (0.7, 0.9, 1.0), alpha=0.5, roughness=None, n=1.33))
    names = {"large_box": "mirror", "sphere": "gloss", "small_box": "water"}
    for m in sc.meshes:
        m.material = names.get(m.name, m.material)
    sc.name = "rough_mix"
    return sc


SCENES = {"cornell": cornell, "hard_indirect": hard_indirect, "rough_mix": rough_mix}


def soup_hash(sc) -> str:
    """FNV-1a (64-bit) of the soup bytes: vertices, normals, material
    indices -- the hash oracle/ref_shader_run.cc prints for the soup the
    reference parser read."""
    v, n, mi = sc.soup()
    h = 0xCBF29CE484222325
    for buf in (v.tobytes(), n.tobytes(), mi.astype(np.int32).tobytes()):
        for b in buf:
            h ^= b
            h = (h * 0x100000001B3) & 0xFFFFFFFFFFFFFFFF
    return f"{h:016x}"


def read_fixture(path):
    """(header dict, accum (P,3) f32, rgba (P,4) u8, radiance/occlusion/zero-direction trace counts (P,3))."""
    with open(path) as fh:
        lines = fh.read().splitlines()
    head = next(ln for ln in lines if ln.startswith("scene ")).split()
    rows = [ln.split() for ln in lines if ln.startswith("px ")]
    h = {"triangles": int(head[1]), "materials": int(head[2]), "width": int(head[3]), "height": int(head[4]),
         "spp": int(head[5]), "bounces": int(head[6]), "soup": head[8]}
    acc = np.array([[int(x, 16) for x in r[2:5]] for r in rows], np.uint32).view(np.float32)
    rgba = np.array([[int(r[5][2 * k:2 * k + 2], 16) for k in range(4)] for r in rows], np.uint8)
    cnt = np.array([[int(x) for x in r[6:9]] for r in rows], np.int64)
    return h, acc, rgba, cnt
