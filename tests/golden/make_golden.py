"""Regenerate the golden fixtures from the reference's own code.

Run from the repository root where the reference sources are available:

    make -C oracle ref          # builds oracle/_ref/* from the reference sources
    python tests/golden/make_golden.py

Writes
  tests/golden/parser/*.rto, *.obj   small scenes covering the .rto grammar
                                     and OBJ reader quirks (inputs)
  tests/golden/parser/*.expected     what the reference SceneParser /
                                     parse_obj produce for each (exit status,
                                     stderr message, parsed fields)
  tests/golden/ref_math.txt          reference math / BSDF / camera / tone
                                     map outputs on fixed inputs
  tests/golden/shader/*.txt          per pixel, what the reference's own
                                     shader programs (shader.cu run on the
                                     host by oracle/_ref/ref_shader_run over
                                     the reference parser's reading of the
                                     scene) write: accumulation buffer, frame
                                     buffer, trace counts.  Scenes:
                                     tests/golden/shader_scenes.py
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
PARSER_DIR = os.path.join(HERE, "parser")

OBJS = {
    # plain v/vn/f with v//vn indices
    "tri.obj": "v 0 0 0\nv 1 0 0\nv 0 1 0\nvn 0 0 1\nf 1//1 2//1 3//1\n",
    # v/vt/vn, comments, groups, a quad (only its first three corners count),
    # CRLF line ends, vt lines, exponent and signed numbers
    "quirks.obj": ("# comment\r\no thing\r\nv -1.5 +2.25 3e-1\r\nv 1 0 0\r\nv 0 1 0\r\nv 1 1 0\r\n"
                   "vt 0.5 0.5\r\nvn 0 0 1\r\nvn 0 0 -1\r\ns off\r\ng grp\r\n"
                   "f 1/1/1 2/1/1 3/1/2\r\nf 2/1/1 4/1/2 3/1/1 1/1/1\r\n"),
    # faces that reference vertices of the whole file, trailing spaces,
    # a last line without newline
    "box.obj": "".join([f"v {x} {y} {z}\n" for x in (0, 1) for y in (0, 1) for z in (0, 1)] +
                       ["vn 1 0 0\nvn 0 1 0\n", "f 1//1 2//1 4//1 \n", "f 5//2 6//2 8//2\n",
                        "f 1//1 5//2 6//2"]),
}

BASE = """
material white {{
  color = (1, 1, 1, 1)
  roughness = 1
}}
material glass {{
  color = (1, 1, 1, 0)
  n = 1.5
}}
material light {{
  emit = true
  color = (1, 1, 1, 1)
}}
mesh {{
  obj_file = tri.obj
  material = white
}}
mesh {{
  obj_file = quirks.obj
  material = glass
}}
mesh {{
  obj_file = box.obj
  material = light
}}
camera {{
  position = (0, 0.5, 2)
  look_at = (0, 0.5, 0)
  fov = 45
}}
{extra}
"""

PARAMS = "num_samples = 16\nnum_bounces = 4\nwidth = 32\nheight = 24\noutput_image = out.ppm\n"

CASES = {
    "basic": BASE.format(extra=PARAMS),
    "comments": "/* width = 99 *//* material bad { color = (1,1,1,1) roughness = 1 } */\n" +
                BASE.format(extra="/* multi\nline\ncomment num_samples = 3 */\n" + PARAMS),
    "comment_cr": "/* width = 7 \r */ " + BASE.format(extra=PARAMS),
    "colors_255": BASE.replace("color = (1, 1, 1, 1)\n  roughness = 1",
                               "color = (255, 128, 0.5, 1)\n  roughness = 0.25").format(extra=PARAMS),
    "float_forms": BASE.replace("position = (0, 0.5, 2)", "position = (+.5, -0.25, 3)")
                       .replace("fov = 45", "fov = 37.5").format(extra=PARAMS),
    "duplicate_material": BASE.format(extra=PARAMS) + "material white {\n  color = (0, 1, 0, 1)\n  roughness = 1\n}\n",
    "roughness_and_n": ("material m {\n  color = (0.5, 0.5, 0.5, 1)\n  n = 1.5\n  roughness = 0.3\n}\n"
                        "material q {\n color = (0.5,0.5,0.5,0.5) roughness = 3 n=4}\n"
                        "mesh {\n  obj_file = tri.obj\n  material = q\n}\n"
                        "camera {\n  position = (0,0,1)\n  look_at = (0,0,0)\n  fov = 40\n}\n" + PARAMS),
    "output_trailing": BASE.format(extra=PARAMS.replace("output_image = out.ppm", "output_image =\n   dir/out img.ppm   ")),
    "substring_keys": ("xmaterial m_1 { color=(0.2,0.3,0.4,1) roughness = 0.5 }\n"
                       "mymesh {\n obj_file = tri.obj\n material = m_1\n}\n"
                       "camera{position=(0,0,1) look_at=(0,0,0) fov=40}\n"
                       "image_width = 8\nwidth = 9\nheight=3 num_samples=1 num_bounces=2\noutput_image=a.ppm\n"),
    "obj_path_spaces": BASE.replace("obj_file = tri.obj", "obj_file =    tri.obj   ").format(extra=PARAMS),
    # error cases (the reference exits with a message)
    "err_no_width": BASE.format(extra=PARAMS.replace("width = 32\n", "")),
    "err_roughness_eq": ("material m {\n  color = (1, 1, 1, 1)\n  roughness=1\n}\n"
                         "camera {\n  position = (0,0,1)\n  look_at = (0,0,0)\n  fov = 40\n}\n" + PARAMS),
    "err_no_color": ("material m {\n  colour = (1, 1, 1, 1)\n  roughness = 1\n}\n"
                     "camera {\n  position = (0,0,1)\n  look_at = (0,0,0)\n  fov = 40\n}\n" + PARAMS),
    "err_no_material": "camera {\n  position = (0,0,1)\n  look_at = (0,0,0)\n  fov = 40\n}\n" + PARAMS,
    "err_unknown_mesh_material": BASE.replace("material = white", "material = wood").format(extra=PARAMS),
    "err_two_cameras": BASE.format(extra=PARAMS + "camera {\n position = (0,0,1)\n look_at = (0,0,0)\n fov = 40\n}\n"),
    "err_no_fov": BASE.replace("fov = 45", "fov = wide").format(extra=PARAMS),
    "err_missing_obj": BASE.replace("obj_file = tri.obj", "obj_file = nothing_here.obj").format(extra=PARAMS),
    # the first failing mesh in declaration order decides the error (the
    # product loads the OBJ files side by side)
    "err_obj_before_material": BASE.replace("obj_file = quirks.obj", "obj_file = nothing_here.obj")
                                   .replace("material = light", "material = wood").format(extra=PARAMS),
    "err_material_before_obj": BASE.replace("material = glass", "material = wood")
                                   .replace("obj_file = box.obj", "obj_file = nothing_here.obj").format(extra=PARAMS),
    # many small meshes, materials cycling, appended in declaration order
    "many_meshes": BASE.format(extra=PARAMS) + "".join(
        f"mesh {{\n  obj_file = {('tri.obj', 'quirks.obj', 'box.obj')[k % 3]}\n"
        f"  material = {('white', 'glass', 'light')[(k // 3) % 3]}\n}}\n" for k in range(60)),
}


def main():
    dump = os.path.join(ROOT, "oracle", "_ref", "ref_parse_dump")
    kdump = os.path.join(ROOT, "oracle", "_ref", "ref_kernels_dump")
    if not (os.path.exists(dump) and os.path.exists(kdump)):
        sys.exit("build oracle/_ref first: make -C oracle ref")
    os.makedirs(PARSER_DIR, exist_ok=True)
    for name, text in OBJS.items():
        with open(os.path.join(PARSER_DIR, name), "w", newline="") as f:
            f.write(text)
    for name, text in CASES.items():
        rto = os.path.join(PARSER_DIR, name + ".rto")
        with open(rto, "w", newline="") as f:
            f.write(text)
        r = subprocess.run([dump, name + ".rto"], cwd=PARSER_DIR, capture_output=True, text=True)
        lines = [ln for ln in r.stdout.splitlines() if not ln.startswith(("Importing", "Done."))]
        err = r.stderr.strip().replace("\n", " | ")
        with open(os.path.join(PARSER_DIR, name + ".expected"), "w") as f:
            f.write(f"exit {r.returncode}\n")
            f.write(f"stderr {err}\n")
            f.write("\n".join(lines) + ("\n" if lines else ""))
    r = subprocess.run([kdump], capture_output=True, text=True, check=True)
    with open(os.path.join(HERE, "ref_math.txt"), "w") as f:
        f.write(r.stdout)
    n = write_shader_fixtures()
    print(f"wrote {len(CASES)} parser cases, ref_math.txt and {n} shader fixtures")


def write_shader_fixtures() -> int:
    sys.path.insert(0, ROOT)
    sys.path.insert(0, HERE)
    import shader_scenes
    from lisa_gb300 import scenes

    run = os.path.join(ROOT, "oracle", "_ref", "ref_shader_run")
    out_dir = os.path.join(HERE, "shader")
    os.makedirs(out_dir, exist_ok=True)
    for name, make in shader_scenes.SCENES.items():
        sc = make()
        with tempfile.TemporaryDirectory() as d:
            rto = scenes.write_rto(sc, d)
            r = subprocess.run([run, rto], capture_output=True, text=True, check=True)
        lines = [ln for ln in r.stdout.splitlines() if ln.startswith(("scene ", "px "))]
        head = lines[0].split()
        if head[8] != shader_scenes.soup_hash(sc):
            sys.exit(f"{name}: the reference parser read another soup than the scene's")
        with open(os.path.join(out_dir, name + ".txt"), "w") as f:
            f.write("\n".join(lines) + "\n")
    return len(shader_scenes.SCENES)


if __name__ == "__main__":
    main()
