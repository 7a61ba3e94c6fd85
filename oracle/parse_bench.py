"""Test infrastructure (oracle side), not product code: times the scene front
end -- .rto grammar + OBJ -> triangle soup -- of the product
(lisa_scene_parse, threaded) against the reference's own SceneParser /
parse_obj (src/LiSA/src/scene_parser.cc:35-261, parse_obj.cc:24-69),
compiled from the reference sources into oracle/_ref/ref_parse_dump by
`make -C oracle ref`.  Both read the same files written by
lisa_gb300.scenes; each is run a few times (best of, warm page cache) and
the soups' sizes are checked equal.

  python oracle/parse_bench.py [--scene icosphere|soup|both] [--repeat 3]

Prints one JSON line per scene.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)

REF_BIN = os.path.join(HERE, "_ref", "ref_parse_dump")


def _scene(name):
    from lisa_gb300 import scenes as S

    if name == "icosphere":
        return S.icosphere_box(level=8)  # 1,310,720 + 12 triangles, one large OBJ
    return S.sphere_soup()  # 20,000 UV spheres, one OBJ each


def bench(name: str, repeat: int, workdir: str) -> dict:
    import lisa_gb300 as L
    from lisa_gb300 import scenes as S

    sc = _scene(name)
    d = os.path.join(workdir, name)
    path = S.write_rto(sc, d)
    obj_bytes = sum(os.path.getsize(os.path.join(d, f)) for f in os.listdir(d) if f.endswith(".obj"))
    ref_s, ref_nv = None, None
    if os.path.exists(REF_BIN):
        ts = []
        for _ in range(repeat):
            # the reference logs what it imports; the timing is the last line
            out = subprocess.run([REF_BIN, "--time", path], capture_output=True, text=True,
                                 check=True).stdout.strip().splitlines()[-1].split()
            ts.append(float(out[0]))
            ref_nv = int(out[1])
        ref_s = min(ts)
    ts = []
    nv = None
    for _ in range(repeat):
        t0 = time.perf_counter()
        p = L.SceneParser(path).get_params()
        ts.append(time.perf_counter() - t0)
        nv = p.raw.num_vertices
    ours = min(ts)
    if ref_nv is not None:
        assert ref_nv == nv, (ref_nv, nv)
    return {"scene": sc.name, "triangles": nv // 3, "obj_mb": round(obj_bytes / 1e6, 1), "meshes": len(sc.meshes),
            "reference_s": ref_s, "product_s": round(ours, 4),
            "speedup": round(ref_s / ours, 2) if ref_s else None, "host_threads": os.cpu_count()}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--scene", default="both", choices=["icosphere", "soup", "both"])
    ap.add_argument("--repeat", type=int, default=3)
    args = ap.parse_args(argv)
    names = ["icosphere", "soup"] if args.scene == "both" else [args.scene]
    with tempfile.TemporaryDirectory() as td:
        for n in names:
            print(json.dumps(bench(n, args.repeat, td)), flush=True)


if __name__ == "__main__":
    main()
