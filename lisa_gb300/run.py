"""Render one synthetic workload and print its statistics.

  python -m lisa_gb300.run --scene icosphere --res 1024 --spp 16 [--estimator physical] [--guided]
                           [--renders 2] [--level 8] [--width W --height H]

Scenes: cornell (the procedural Cornell box), icosphere (a displaced
icosphere of 20 * 4^level triangles, dielectric, in the box), hard_indirect
(the icosphere scene with a 0.02 x 0.02 light behind a baffle), soup (a
sphere soup of --spheres UV spheres).  Each render is one call of
lisa_render over the given spp; the printed line holds the device time, the
rays traced and the per-stage times.  Used for kernel profiles: every
render launches the same kernel sequence.
"""
from __future__ import annotations

import argparse
import json

from . import scenes as S


def make(args):
    w, h = args.width or args.res, args.height or args.res
    if args.scene == "cornell":
        return S.cornell_box(width=w, height=h, num_samples=args.spp, num_bounces=args.bounces or 7)
    if args.scene == "icosphere":
        return S.icosphere_box(level=args.level, width=w, height=h, num_samples=args.spp,
                               num_bounces=args.bounces or 8)
    if args.scene == "hard_indirect":
        return S.hard_indirect(level=args.level, width=w, height=h, num_samples=args.spp,
                               num_bounces=args.bounces or 8)
    return S.sphere_soup(n_spheres=args.spheres, width=w, height=h, num_samples=args.spp,
                         num_bounces=args.bounces or 12, extent=100.0 * (args.spheres / 20000) ** (1 / 3))


def main(argv=None):
    import lisa_gb300 as L

    ap = argparse.ArgumentParser(prog="python -m lisa_gb300.run")
    ap.add_argument("--scene", default="icosphere", choices=["cornell", "icosphere", "hard_indirect", "soup"])
    ap.add_argument("--res", type=int, default=512)
    ap.add_argument("--width", type=int, default=0)
    ap.add_argument("--height", type=int, default=0)
    ap.add_argument("--spp", type=int, default=16)
    ap.add_argument("--level", type=int, default=8)
    ap.add_argument("--spheres", type=int, default=20000)
    ap.add_argument("--bounces", type=int, default=0)
    ap.add_argument("--estimator", default="compat", choices=["compat", "physical"])
    ap.add_argument("--guided", action="store_true")
    ap.add_argument("--renders", type=int, default=1)
    ap.add_argument("--paths", type=int, default=0, help="paths in flight (0 = default)")
    args = ap.parse_args(argv)
    sc = make(args)
    opts = L.default_options(
        stage_timing=1, paths_in_flight=args.paths,
        estimator=L._native.LISA_ESTIMATOR_PHYSICAL if args.estimator == "physical" else L._native.LISA_ESTIMATOR_COMPAT,
        mode=L._native.LISA_MODE_GUIDED if args.guided else L._native.LISA_MODE_COMPAT)
    r = L.Renderer(L.params_from_scene(sc), opts)
    for k in range(args.renders):
        st = r.render()
        print(json.dumps({"render": k, "scene": sc.name, "triangles": sc.num_triangles, "res": [sc.width, sc.height],
                          "spp": args.spp, "ms": st.ms_device, "rays": st.rays,
                          "mrays_per_s": st.rays / max(st.ms_device, 1e-9) / 1e3,
                          "stages_ms": {"trace": st.ms_trace, "shade": st.ms_shade, "nee": st.ms_nee,
                                        "guide": st.ms_guide, "other": st.ms_other},
                          "guide_infer": {"ms": st.ms_guide_infer, "rows": st.guide_infer_rows},
                          "guide_train": {"ms": st.ms_guide_train, "samples": st.guide_train_samples},
                          "launches": st.launches_total, "status": st.device_status}), flush=True)
    r.close()


if __name__ == "__main__":
    main()
