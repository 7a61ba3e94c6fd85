#!/bin/bash
# Build the headless OptiX baseline harness (baseline/optix_harness.cc) against
# the reference sources staged by baseline/stage_optix.py.  Output:
# baseline/_ref/lisa_optix_harness.  The OptiX runtime itself (libnvoptix) is
# part of the NVIDIA driver and is loaded at run time by optixInit.
set -e
HERE="$(cd "$(dirname "$0")" && pwd)"
S="$HERE/_ref/optix_src"
CUDA="${CUDA_HOME:-/usr/local/cuda}"
if [ ! -d "$S/src/LiSA" ]; then
  echo "baseline/_ref/optix_src missing: run baseline/stage_optix.py where the reference sources are" >&2
  exit 3
fi
g++ -O2 -std=c++20 -include algorithm -include iterator -include iostream -w \
  -DOPTIX_SAMPLE_NAME='"LiSA"' -DOPTIX_SAMPLE_DIR='"LiSA"' \
  -I "$HERE/optix_shim" -I "$S/src/LiSA/include" -I "$S/src/LiSA/src" -I "$S/src" -I "$S/src/cuda" \
  -I "$S/src/optix/include" -I "$CUDA/include" \
  -o "$HERE/_ref/lisa_optix_harness" \
  "$HERE/optix_harness.cc" "$S/src/LiSA/src/optix_wrapper.cc" "$S/src/LiSA/src/scene_parser.cc" \
  "$S/src/LiSA/src/parse_obj.cc" "$S/src/sutil/Camera.cpp" \
  -L "$CUDA/lib64" -lcudart -ldl -lpthread -Wl,-rpath,"$CUDA/lib64"
