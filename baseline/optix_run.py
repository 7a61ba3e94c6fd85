"""Run the reference's OptiX render (baseline/optix_harness.cc) on a scene.

The harness is built on first use from the sources that
baseline/stage_optix.py staged under baseline/_ref (see its docstring); where
they or the OptiX runtime are missing, ``available()`` says why.

    python baseline/optix_run.py --scene cornell --spp 16
    python baseline/optix_run.py --scene icosphere --spp 16 --reps 5
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
REF = os.path.join(HERE, "_ref")
HARNESS = os.path.join(REF, "lisa_optix_harness")
PTX = os.path.join(REF, "shader.ptx")
PTX_COUNTED = os.path.join(REF, "shader_counted.ptx")
# diagnostic: occlusion rays take the closest hit instead of the first found
PTX_CLOSEST = os.path.join(REF, "shader_closest.ptx")
PTX_CLOSEST_IEEE = os.path.join(REF, "shader_closest_ieee.ptx")  # the same without --use_fast_math
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def _optix_runtime() -> str | None:
    for d in ("/usr/local/nvidia/lib64", "/usr/lib", "/usr/lib64", "/usr/lib/aarch64-linux-gnu",
              "/usr/lib/x86_64-linux-gnu"):
        p = os.path.join(d, "libnvoptix.so.1")
        if os.path.exists(p):
            return d
    return None


def available() -> str | None:
    """None when the OptiX baseline can run here, else the reason."""
    if not (os.path.exists(PTX) and os.path.isdir(os.path.join(REF, "optix_src"))):
        return "reference OptiX sources not staged (baseline/stage_optix.py needs the reference tree)"
    if _optix_runtime() is None:
        return "no libnvoptix.so.1 (OptiX runtime of the NVIDIA driver) on this machine"
    return None


def ensure_built() -> str:
    ok = os.path.exists(HARNESS)
    if ok:
        # a binary built on another host architecture does not run here
        try:
            ok = subprocess.run([HARNESS], capture_output=True).returncode == 2
        except OSError:
            ok = False
    if not ok:
        subprocess.run(["bash", os.path.join(HERE, "build_optix.sh")], check=True)
    return HARNESS


def write_soup(scene, path: str) -> None:
    """The scene's soup in the harness's raw format (optix_harness.cc,
    load_soup): the arrays the reference's SceneParser would produce."""
    v, n, mi = scene.soup()
    table = scene.material_table()  # roughness alpha n diffuse(3) emit emission(3)
    mats = np.zeros(table.shape[0], dtype=[("roughness", "<f4"), ("alpha", "<f4"), ("n", "<f4"),
                                            ("diffuse", "<f4", 3), ("emit", "u1"), ("pad", "u1", 3),
                                            ("emission", "<f4", 3)])
    mats["roughness"], mats["alpha"], mats["n"] = table[:, 0], table[:, 1], table[:, 2]
    mats["diffuse"] = table[:, 3:6]
    mats["emit"] = (table[:, 6] != 0).astype(np.uint8)
    mats["emission"] = table[:, 7:10]
    assert mats.itemsize == 40
    head = np.array([mi.shape[0], table.shape[0], scene.width, scene.height, scene.num_samples, scene.num_bounces],
                    np.uint32)
    cam = np.array([*scene.eye, *scene.look_at, scene.fov], np.float32)
    with open(path, "wb") as f:
        f.write(b"LSOUP1\0\0")
        f.write(head.tobytes())
        f.write(cam.tobytes())
        f.write(np.ascontiguousarray(v, np.float32).tobytes())
        f.write(np.ascontiguousarray(n, np.float32).tobytes())
        f.write(np.ascontiguousarray(mi, np.int32).tobytes())
        f.write(mats.tobytes())


def run(scene, spp: int | None = None, warmup: int = 2, reps: int = 5, count: bool = True,
        accum: bool = False, rto: bool = False, timeout: float = 1200.0, ptx: str | None = None) -> dict:
    """Time the reference's OptiX launch on ``scene`` (spp samples per pixel
    in one launch, subframe 0).  Returns the harness's JSON fields, plus
    ``accum`` (H, W, 3) when asked for.  ``ptx`` replaces the stock shader
    (PTX_CLOSEST: the closest-hit diagnostic)."""
    why = available()
    if why:
        raise RuntimeError(why)
    exe = ensure_built()
    env = dict(os.environ)
    env["LISA_OPTIX_PTX"] = ptx or PTX
    libdir = _optix_runtime()
    env["LD_LIBRARY_PATH"] = libdir + (":" + env["LD_LIBRARY_PATH"] if env.get("LD_LIBRARY_PATH") else "")
    with tempfile.TemporaryDirectory() as d:
        if rto:
            from lisa_gb300 import scenes

            args = ["--rto", scenes.write_rto(scene, d)]
        else:
            p = os.path.join(d, "scene.soup")
            write_soup(scene, p)
            args = ["--soup", p]
        if spp:
            args += ["--spp", str(spp)]
        args += ["--warmup", str(warmup), "--reps", str(reps)]
        if count:
            args += ["--count-ptx", PTX_COUNTED]
        acc_path = os.path.join(d, "accum.f32")
        if accum:
            args += ["--accum", acc_path]
        r = subprocess.run([exe] + args, capture_output=True, text=True, env=env, timeout=timeout, cwd=d)
        if r.returncode != 0:
            raise RuntimeError(f"OptiX harness failed ({r.returncode}): {r.stderr[-2000:]}")
        line = [ln for ln in r.stdout.splitlines() if ln.startswith("{")][-1]
        out = json.loads(line)
        if accum:
            a = np.fromfile(acc_path, np.float32).reshape(scene.height, scene.width, 4)
            out["accum"] = a[:, :, :3].copy()
    out["rays"] = out["rays_radiance"] + out["rays_occlusion"]
    if out["ms_per_launch"] > 0 and count:
        out["mrays_per_s"] = out["rays"] / (out["ms_per_launch"] * 1e3)
    return out


def main() -> None:
    from lisa_gb300 import scenes

    ap = argparse.ArgumentParser()
    ap.add_argument("--scene", default="cornell", choices=["cornell", "icosphere", "soup", "hard_indirect"])
    ap.add_argument("--width", type=int, default=0)
    ap.add_argument("--height", type=int, default=0)
    ap.add_argument("--spp", type=int, default=16)
    ap.add_argument("--bounces", type=int, default=0)
    ap.add_argument("--level", type=int, default=8)
    ap.add_argument("--warmup", type=int, default=2)
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--rto", action="store_true")
    a = ap.parse_args()
    if a.scene == "cornell":
        sc = scenes.cornell_box()
    elif a.scene == "icosphere":
        sc = scenes.icosphere_box(level=a.level)
    elif a.scene == "hard_indirect":
        sc = scenes.hard_indirect(level=a.level)
    else:
        sc = scenes.sphere_soup()
    if a.width:
        sc.width = a.width
    if a.height:
        sc.height = a.height
    if a.bounces:
        sc.num_bounces = a.bounces
    out = run(sc, spp=a.spp, warmup=a.warmup, reps=a.reps, rto=a.rto)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
