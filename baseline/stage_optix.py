"""Stage the reference's OptiX render for the headless baseline harness.

Run in a checkout where the reference sources exist:

    LISA_REFERENCE_DIR=/root/reference python baseline/stage_optix.py

Copies the reference files the OptiX path needs into baseline/_ref/optix_src
(git-ignored: nothing of the reference enters the repository's history;
the directory travels with the working tree to the machine that runs the
baseline), writes there a counting copy of shader.cu (one atomicAdd before
each optixTrace, launch parameters extended by a counter pointer) and a
diagnostic copy whose occlusion rays take the closest hit (also compiled
without fast math), and compiles the shaders to PTX with the reference's own nvcc flags
(src/CMakeLists.txt:170-177: --use_fast_math -lineinfo; the lowest virtual
architecture CUDA 13 accepts, compute_75, stands in for sm_50).  The PTX is
handed to OptiX unread.

baseline/build_optix.sh then compiles the harness on the machine with the GPU.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref", "optix_src")

FILES = [
    "src/LiSA/include/optix_wrapper.hh",
    "src/LiSA/include/scene_parser.hh",
    "src/LiSA/include/parse_obj.hh",
    "src/LiSA/include/structs.hh",
    "src/LiSA/src/optix_wrapper.cc",
    "src/LiSA/src/scene_parser.cc",
    "src/LiSA/src/parse_obj.cc",
    "src/LiSA/src/shader.cu",
    "src/LiSA/src/maths.cu",
    "src/LiSA/src/bsdfs/lambertian.cu",
    "src/cuda/random.h",
    "src/cuda/helpers.h",
    "src/sutil/vec_math.h",
    "src/sutil/Preprocessor.h",
    "src/sutil/sutilapi.h",
    "src/sutil/Camera.h",
    "src/sutil/Camera.cpp",
]
DIRS = ["src/optix/include"]

COUNT_STRUCT = """
// counting copy: launch parameters extended by the address of two counters
struct OptixParamsCounted : OptixParams {
  unsigned long long* ray_counts;  // [0] radiance traces, [1] occlusion traces
};
"""


def counted_shader(src: str) -> str:
    """shader.cu with an atomicAdd before each optixTrace (radiance and
    occlusion) and `params` declared with the extended struct."""
    decl = "__constant__ OptixParams params;"
    if src.count(decl) != 1:
        raise RuntimeError("shader.cu: launch parameter declaration not found")
    src = src.replace(decl, "__constant__ OptixParamsCounted params;")
    first_extern = src.index('extern "C" {')
    src = src[:first_extern] + COUNT_STRUCT + src[first_extern:]
    out, n = [], 0
    for line in src.splitlines(keepends=True):
        if line.strip() == "packPointer(inter, u0, u1);":
            # trace_occlusion comes first in the file, trace_radiance second
            idx = 1 if n == 0 else 0
            out.append(line)
            out.append(f"  atomicAdd(&params.ray_counts[{idx}], 1ull);\n")
            n += 1
        else:
            out.append(line)
    if n != 2:
        raise RuntimeError(f"shader.cu: expected 2 trace functions, found {n}")
    return "".join(out)


def closest_occlusion_shader(src: str) -> str:
    """shader.cu with its occlusion rays traced for the closest hit
    (OPTIX_RAY_FLAG_NONE) instead of terminating on the first hit OptiX
    finds (shader.cu:69).  A diagnostic only: it separates the effect of
    first-hit termination from every other difference between the OptiX run
    and this library."""
    flag = "OPTIX_RAY_FLAG_TERMINATE_ON_FIRST_HIT"
    if src.count(flag) != 1:
        raise RuntimeError("shader.cu: occlusion ray flag not found")
    return src.replace(flag, "OPTIX_RAY_FLAG_NONE")


def nvcc_ptx(src: str, out: str, fast_math: bool = True) -> None:
    inc = [os.path.join(OUT, p) for p in ("src/LiSA/src", "src/LiSA/include", "src", "src/cuda",
                                           "src/optix/include")]
    cmd = ["nvcc", "-ptx", "-arch=compute_75"] + (["--use_fast_math"] if fast_math else []) + [
           "-lineinfo", "-std=c++17", "-Wno-deprecated-gpu-targets", "-o", out, src]
    for i in inc:
        cmd[1:1] = ["-I", i]
    subprocess.run(cmd, check=True)


def main() -> None:
    ref = os.environ.get("LISA_REFERENCE_DIR", "")
    if not ref or not os.path.isdir(os.path.join(ref, "src", "LiSA")):
        sys.exit(f"reference tree not found at {ref} (set LISA_REFERENCE_DIR)")
    if os.path.isdir(OUT):
        shutil.rmtree(OUT)
    for rel in FILES:
        dst = os.path.join(OUT, rel)
        os.makedirs(os.path.dirname(dst), exist_ok=True)
        shutil.copy2(os.path.join(ref, rel), dst)
    for rel in DIRS:
        shutil.copytree(os.path.join(ref, rel), os.path.join(OUT, rel))
    shader = os.path.join(OUT, "src/LiSA/src/shader.cu")
    counted = os.path.join(OUT, "src/LiSA/src/shader_counted.cu")
    with open(shader) as f:
        text = f.read()
    with open(counted, "w") as f:
        f.write(counted_shader(text))
    closest = os.path.join(OUT, "src/LiSA/src/shader_closest.cu")
    with open(closest, "w") as f:
        f.write(closest_occlusion_shader(text))
    nvcc_ptx(shader, os.path.join(HERE, "_ref", "shader.ptx"))
    nvcc_ptx(counted, os.path.join(HERE, "_ref", "shader_counted.ptx"))
    nvcc_ptx(closest, os.path.join(HERE, "_ref", "shader_closest.ptx"))
    # the same without --use_fast_math: IEEE-rounded division and square root
    nvcc_ptx(closest, os.path.join(HERE, "_ref", "shader_closest_ieee.ptx"), fast_math=False)
    print(f"staged {len(FILES)} files + {DIRS} into {OUT}; PTX in baseline/_ref/")


if __name__ == "__main__":
    main()
