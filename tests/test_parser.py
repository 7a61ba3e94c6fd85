"""The .rto / OBJ front end against the reference SceneParser.

Golden expectations in tests/golden/parser/*.expected were produced by the
reference's own scene_parser.cc + parse_obj.cc (compiled from its sources by
oracle/Makefile, driven by oracle/ref_parse_dump.cc; regenerate with
tests/golden/make_golden.py).  Where that binary is present (built from the
reference tree), the generated Cornell box is also compared live.
"""
import glob
import os
import struct
import subprocess

import numpy as np
import pytest

import lisa_gb300 as L
from lisa_gb300 import scenes

HERE = os.path.dirname(os.path.abspath(__file__))
PARSER_DIR = os.path.join(HERE, "golden", "parser")
CASES = sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(PARSER_DIR, "*.rto")))


def fbits(x: float) -> str:
    return "%08x" % struct.unpack("<I", struct.pack("<f", x))[0]


def fnv1a(data: bytes) -> int:
    h = 1469598103934665603
    a = np.frombuffer(data, np.uint8)
    # vectorised FNV-1a is sequential; do it in chunks of python ints
    for b in a.tolist():
        h ^= b
        h = (h * 1099511628211) & 0xFFFFFFFFFFFFFFFF
    return h


def dump(params: L.Params) -> list:
    p = params.raw
    out = [f"width {p.width}", f"height {p.height}", f"num_samples {p.num_samples}",
           f"num_bounces {p.num_bounces}"]
    oi = p.output_image
    out.append(f"output_image {len(oi)} {oi.hex()}")
    c = p.camera
    out.append("camera " + " ".join(fbits(x) for x in (c.eye.x, c.eye.y, c.eye.z, c.look_at.x, c.look_at.y,
                                                           c.look_at.z, c.fov)))
    out.append(f"num_materials {p.num_materials}")
    for i, m in enumerate(params.materials()):
        if m.emit:
            e = m.emission_color
            out.append(f"material {i} emit {fbits(e.x)} {fbits(e.y)} {fbits(e.z)} alpha {fbits(m.alpha)}")
        elif m.alpha < 1.0:
            d = m.diffuse_color
            out.append(f"material {i} dielectric {fbits(d.x)} {fbits(d.y)} {fbits(d.z)} alpha {fbits(m.alpha)} "
                       f"n {fbits(m.n)}")
        else:
            d = m.diffuse_color
            out.append(f"material {i} diffuse {fbits(d.x)} {fbits(d.y)} {fbits(d.z)} alpha {fbits(m.alpha)} "
                       f"roughness {fbits(m.roughness)}")
    out.append(f"num_vertices {p.num_vertices}")
    blob = params.vertices().tobytes() + params.normals().tobytes() + params.mat_indices().tobytes()
    out.append("soup_fnv1a %016x" % fnv1a(blob))
    return out


def read_expected(name):
    with open(os.path.join(PARSER_DIR, name + ".expected")) as f:
        lines = f.read().splitlines()
    code = int(lines[0].split()[1])
    err = lines[1][len("stderr "):] if len(lines) > 1 else ""
    return code, err, lines[2:]


@pytest.mark.parametrize("case", CASES)
def test_parser_matches_reference(case, monkeypatch):
    monkeypatch.chdir(PARSER_DIR)  # the reference opens OBJ paths relative to the working directory
    code, err, expected = read_expected(case)
    if code != 0:
        with pytest.raises(L.LisaError) as ei:
            L.SceneParser(case + ".rto")
        # same message as the reference prints before exit()
        assert err.split(" | ")[0].strip() in str(ei.value)
        assert ei.value.code in (L._native.LISA_ERR_PARSE, L._native.LISA_ERR_IO)
        return
    got = dump(L.SceneParser(case + ".rto").get_params())
    assert got == expected


def test_parse_string_and_base_dir():
    with open(os.path.join(PARSER_DIR, "basic.rto")) as f:
        text = f.read()
    p = L.SceneParser(text=text, base_dir=PARSER_DIR).get_params()
    _, _, expected = read_expected("basic")
    assert dump(p) == expected


def test_missing_scene_file():
    with pytest.raises(L.LisaError) as ei:
        L.SceneParser("/nonexistent/scene.rto")
    assert ei.value.code == L._native.LISA_ERR_IO


def test_generated_cornell_box_against_reference(tmp_path):
    """The generated workload scene parses identically through both parsers,
    and the parsed soup equals the in-memory soup the bench feeds the C ABI."""
    sc = scenes.cornell_box()
    rto = scenes.write_rto(sc, str(tmp_path))
    params = L.SceneParser(rto).get_params()
    v, n, mi = sc.soup()
    assert np.array_equal(params.vertices(), v)
    assert np.array_equal(params.normals(), n)
    assert np.array_equal(params.mat_indices(), mi)
    import oracle as O

    ref = O.ref_binary("ref_parse_dump")
    if ref is None:
        pytest.skip("reference parser not built here (needs the reference tree)")
    r = subprocess.run([ref, rto], capture_output=True, text=True, check=True)
    expected = [ln for ln in r.stdout.splitlines() if not ln.startswith(("Importing", "Done."))]
    assert dump(params) == expected


def test_obj_append_api(tmp_path):
    import ctypes as C

    N = L._native
    h = C.c_void_p()
    N.check(N.lib().lisa_scene_create_empty(C.byref(h)))
    N.check(N.lib().lisa_scene_append_obj(h, os.path.join(PARSER_DIR, "quirks.obj").encode(), 3))
    raw = N.RendererParams()
    N.check(N.lib().lisa_scene_params(h, C.byref(raw)))
    assert raw.num_vertices == 6  # two faces; the quad keeps its first three corners
    mi = np.ctypeslib.as_array(raw.mat_indices, (2,))
    assert mi.tolist() == [3, 3]
    v = np.ctypeslib.as_array(C.cast(raw.vertices, C.POINTER(C.c_float)), (6, 3))
    assert v[0].tolist() == [-1.5, 2.25, np.float32(0.3)]
    bad = tmp_path / "bad.obj"
    bad.write_text("v 0 0 0\nf 1 1 1\n")
    with pytest.raises(L.LisaError):
        N.check(N.lib().lisa_scene_append_obj(h, str(bad).encode(), 0))
    N.lib().lisa_scene_destroy(h)


def test_parallel_obj_loader_large(tmp_path):
    """A multi-megabyte OBJ goes through the threaded path and de-indexes
    exactly like the single-threaded reader semantics."""
    sc = scenes.icosphere_box(level=5)
    rto = scenes.write_rto(sc, str(tmp_path))
    params = L.SceneParser(rto).get_params()
    v, n, mi = sc.soup()
    assert params.num_triangles == sc.num_triangles
    assert np.array_equal(params.vertices(), v)
    assert np.array_equal(params.normals(), n)
    assert np.array_equal(params.mat_indices(), mi)
