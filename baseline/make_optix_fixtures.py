"""Record the reference's OptiX render of the estimator fixture scenes.

Run on a machine with the GPU, after baseline/stage_optix.py staged the
reference sources (they travel in baseline/_ref):

    python baseline/make_optix_fixtures.py gpurun_out/optix_fixtures

For each scene of tests/golden/shader_scenes.py it runs the reference's own
OptiX pipeline (baseline/optix_harness.cc) on the scene written as .rto +
OBJ and read by the reference's SceneParser, and writes the accumulation
buffer (per pixel RGB, float32, row-major) of:

  <scene>_stock.f32         shader.cu as the reference ships it (occlusion
                            rays terminate on the first hit OptiX finds)
  <scene>_closest.f32       occlusion rays take the closest hit
  <scene>_closest_ieee.f32  the same compiled without --use_fast_math

plus summary.json with the traced-ray counts of the stock shader.  The
files are copied to tests/golden/optix/ and compared there with the oracle
(tests/test_oracle_pin.py) and the GPU renderer (tests/test_gpu_render.py).
"""
from __future__ import annotations

import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))

import numpy as np  # noqa: E402

import optix_run as R  # noqa: E402
import shader_scenes as S  # noqa: E402


def main(out_dir: str) -> None:
    why = R.available()
    if why:
        sys.exit(why)
    os.makedirs(out_dir, exist_ok=True)
    summary = {}
    for name, make in S.SCENES.items():
        sc = make()
        rec = {"soup": S.soup_hash(sc)}
        for tag, ptx, count in (("stock", R.PTX, True), ("closest", R.PTX_CLOSEST, False),
                                ("closest_ieee", R.PTX_CLOSEST_IEEE, False)):
            r = R.run(sc, warmup=0, reps=1, count=count, accum=True, rto=True, ptx=ptx)
            np.ascontiguousarray(r.pop("accum"), np.float32).tofile(os.path.join(out_dir, f"{name}_{tag}.f32"))
            if count:
                rec["rays_radiance"] = r["rays_radiance"]
                rec["rays_occlusion"] = r["rays_occlusion"]
        summary[name] = rec
        print(name, rec, flush=True)
    with open(os.path.join(out_dir, "summary.json"), "w") as f:
        json.dump(summary, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "optix_fixtures")
