// Headless replacement for the one sutil.h declaration the reference's
// OptiX set-up uses (src/LiSA/src/optix_wrapper.cc:166): getInputData, here
// reading PTX that nvcc compiled ahead of time (baseline/stage_optix.py)
// from the file named by the environment variable LISA_OPTIX_PTX.  The
// reference's own sutil.h pulls in CMake-generated configuration and the
// rest of sutil, which the headless harness does not build.
#pragma once

#include <cstddef>

namespace sutil {
const char* getInputData(const char* sample_name, const char* sample_dir, const char* filename, size_t& size);
}
