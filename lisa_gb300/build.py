"""Build the native library in-tree: lisa_gb300/liblisa_gb.so (sm_103a only)
and the `lisa` command-line renderer.

Every CUDA translation unit is compiled by nvcc for sm_103a; host C++ is
compiled by nvcc's host compiler with FP contraction off, so host-side
floating point (camera frame, parsing) is identical on x86 and Arm hosts.
Objects are compiled in parallel and only rebuilt when a source or header
changed.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "liblisa_gb.so")
CLI = os.path.join(HERE, "bin", "lisa")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-I", os.path.join(ROOT, "include"), "-I", CSRC,
          "-Xcompiler", "-fPIC,-ffp-contract=off", "--expt-relaxed-constexpr"]
SOURCES = ["api.cu", "bvh_build.cu", "wavefront.cu", "guide.cu", "noalloc.cu", "autotune.cu", "scene_parser.cc"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def _headers():
    hs = glob.glob(os.path.join(CSRC, "**", "*.cuh"), recursive=True)
    hs += glob.glob(os.path.join(CSRC, "*.h"))
    hs += glob.glob(os.path.join(ROOT, "include", "*.h"))
    return hs


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src: str, extra=()):
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    deps = [src] + _headers() + [__file__]
    if not _stale(obj, deps):
        return obj
    cmd = [nvcc()] + ARCH + COMMON + list(extra) + ["-c", src, "-o", obj]
    if src.endswith(".cu"):
        cmd[1:1] = ["-Xptxas", "-warn-spills"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose: bool = False, extra_flags=()) -> str:
    """Compile and link the library.  extra_flags (e.g. ["-DLISA_BOUNDS"]
    for the bounds-checked build) get their own object directory, so
    switching between builds recompiles what they change; the library and
    the CLI are relinked in place, so the last build wins."""
    global BUILD
    base = BUILD
    if extra_flags:
        import hashlib

        BUILD = base + "_" + hashlib.sha1(" ".join(extra_flags).encode()).hexdigest()[:8]
    try:
        return _build(verbose, extra_flags)
    finally:
        BUILD = base


def _build(verbose: bool, extra_flags) -> str:
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(os.path.dirname(CLI), exist_ok=True)
    srcs = [os.path.join(CSRC, s) for s in SOURCES]
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra_flags), srcs))
    # which flags the library was last linked with: a switch relinks it
    stamp = os.path.join(HERE, "_build", "last_link_flags")
    flags = " ".join(extra_flags)
    try:
        with open(stamp) as f:
            same = f.read() == flags
    except OSError:
        same = not flags
    if not same and os.path.exists(LIB):
        os.remove(LIB)
    if _stale(LIB, objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        os.makedirs(os.path.dirname(stamp), exist_ok=True)
        with open(stamp, "w") as f:
            f.write(flags)
    main = os.path.join(CSRC, "main.cc")
    if os.path.exists(main) and _stale(CLI, [main, LIB]):
        cmd = [nvcc()] + ARCH + COMMON + [main, "-o", CLI, "-L", HERE, "-llisa_gb",
                                          "-Xlinker", "-rpath,$ORIGIN/.."]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"cli build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose:
        print(LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True, extra_flags=sys.argv[1:])
