"""The C-ABI library loads without a GPU and exports every symbol
include/lisa_gb.h declares; reference-layout structs keep their layout."""
import ctypes as C
import os
import re

import pytest

import lisa_gb300 as L
from lisa_gb300 import _native as N

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for hdr in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if not hdr.endswith(".h"):
            continue
        text = open(os.path.join(ROOT, "include", hdr)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\**\s*(lisa_[a-z_0-9]+)\s*\(", text, flags=re.M):
            names.append(m.group(1))
    return names


def test_library_exports_every_declared_symbol():
    lib = N.lib()
    names = declared_functions()
    assert len(names) >= 30
    for n in names:
        assert hasattr(lib, n), n
    # and the ctypes table covers them all
    assert set(names) <= set(N.SIGNATURES), set(names) - set(N.SIGNATURES)


def test_reference_struct_layouts():
    # Material: 40 bytes, offsets 0/4/8/12/24/28 (structs.hh:16-23)
    assert C.sizeof(N.Material) == 40
    assert [getattr(N.Material, f).offset for f in ("roughness", "alpha", "n", "diffuse_color", "emit",
                                                     "emission_color")] == [0, 4, 8, 12, 24, 28]
    assert C.sizeof(N.Camera) == 28
    assert C.sizeof(N.Options) == N.default_options().struct_size


def test_errors_without_gpu_are_reported_not_raised():
    lib = N.lib()
    assert lib.lisa_version().startswith(b"lisa_gb300")
    # bad arguments come back as status codes with a message
    assert lib.lisa_scene_parse(None, None) == N.LISA_ERR_INVALID
    assert b"null" in lib.lisa_last_error()
    assert lib.lisa_render(None, None) == N.LISA_ERR_INVALID
    assert lib.lisa_selftest_wait_timeout(0, None) == N.LISA_ERR_INVALID
    assert lib.lisa_guide_train_steps(None, None, None, None, 0, 128, 1, 0.01, None) == N.LISA_ERR_INVALID
    # the device-memory cache empties (without a GPU it never held anything)
    freed = C.c_uint64(123)
    assert lib.lisa_device_cache_release(None) == N.LISA_OK
    assert lib.lisa_device_cache_release(C.byref(freed)) == N.LISA_OK and freed.value == 0


def test_renderer_options_are_checked_before_the_device():
    """Launch and mode options out of range are refused as invalid before
    any device is touched (a block size that is not whole warps, or above
    the persistent kernels' 128 threads, would break their warp-wide
    steps)."""
    import numpy as np
    import pytest

    import lisa_gb300 as L

    v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    n = np.tile(np.array([0, 0, 1], np.float32), (3, 1))
    mats = np.array([[1, 1, 1, 0.5, 0.5, 0.5, 0, 0, 0, 0]], np.float32)
    p = L.params_from_arrays(v, n, np.zeros(1, np.int32), mats, 4, 4, (0, 0, 2), (0, 0, 0), 40.0, 1, 2)
    for kw in (dict(threads_per_block=100), dict(threads_per_block=256), dict(refill_idle=33),
               dict(estimator=9), dict(mode=7)):
        with pytest.raises(N.LisaError) as e:
            L.Renderer(p, **kw)
        assert e.value.code == N.LISA_ERR_INVALID, kw


def test_ppm_writer_matches_save_image_layout(tmp_path):
    import numpy as np

    rgba = np.zeros((3, 4, 4), np.uint8)
    rgba[..., 0] = np.arange(3)[:, None] * 10  # row index in red
    rgba[..., 1] = np.arange(4)[None, :]
    rgba[..., 3] = 255
    p = tmp_path / "a.ppm"
    L.write_ppm(str(p), rgba)
    data = p.read_bytes()
    assert data.startswith(b"P6\n4 3\n255\n")
    pix = np.frombuffer(data[len(b"P6\n4 3\n255\n"):], np.uint8).reshape(3, 4, 3)
    # rows flipped (sutil.cpp:543-553), alpha dropped
    assert pix[0, 0, 0] == 20 and pix[2, 0, 0] == 0
    assert pix[1, 3, 1] == 3
    with pytest.raises(L.LisaError):
        L.write_ppm(str(tmp_path / "a.png"), rgba)


def test_cli_reports_errors_like_the_reference_main(tmp_path):
    """The `lisa` CLI (main.cc's interface): no -s prints the usage and
    fails; a scene that does not exist fails with the parser's message,
    before any device is touched."""
    import os
    import subprocess

    cli = os.path.join(os.path.dirname(N.LIB_PATH), "bin", "lisa")
    r = subprocess.run([cli], capture_output=True, text=True)
    assert r.returncode == 1 and "Missing scene path" in r.stderr
    r = subprocess.run([cli, "-s", str(tmp_path / "none.rto")], capture_output=True, text=True)
    assert r.returncode == 1 and "not found" in r.stderr
