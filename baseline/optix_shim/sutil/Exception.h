// Headless replacement for the error-check macros the reference's OptiX
// set-up uses (OPTIX_CHECK, OPTIX_CHECK_LOG, CUDA_CHECK, CUDA_SYNC_CHECK in
// src/LiSA/src/optix_wrapper.cc).  Same behaviour -- throw on failure with
// the call text and the OptiX log -- without the display headers the
// reference's sutil/Exception.h includes.
#pragma once

#include <cuda_runtime.h>
#include <optix.h>

#include <sstream>
#include <stdexcept>

#define OPTIX_CHECK(call)                                                                    \
  do {                                                                                       \
    OptixResult res_ = call;                                                                 \
    if (res_ != OPTIX_SUCCESS) {                                                             \
      std::stringstream ss_;                                                                 \
      ss_ << "OptiX call '" << #call << "' failed (" << (int)res_ << ") at " << __FILE__      \
          << ":" << __LINE__;                                                                \
      throw std::runtime_error(ss_.str());                                                   \
    }                                                                                        \
  } while (0)

// expects `log` (char array) and `sizeof_log` (size_t) in scope, as the
// reference's macro does
#define OPTIX_CHECK_LOG(call)                                                                \
  do {                                                                                       \
    OptixResult res_ = call;                                                                 \
    sizeof_log = sizeof(log);                                                                \
    if (res_ != OPTIX_SUCCESS) {                                                             \
      std::stringstream ss_;                                                                 \
      ss_ << "OptiX call '" << #call << "' failed (" << (int)res_ << ") at " << __FILE__      \
          << ":" << __LINE__ << "\nlog: " << log;                                            \
      throw std::runtime_error(ss_.str());                                                   \
    }                                                                                        \
  } while (0)

#define CUDA_CHECK(call)                                                                     \
  do {                                                                                       \
    cudaError_t err_ = call;                                                                 \
    if (err_ != cudaSuccess) {                                                               \
      std::stringstream ss_;                                                                 \
      ss_ << "CUDA call '" << #call << "' failed: " << cudaGetErrorString(err_) << " at "    \
          << __FILE__ << ":" << __LINE__;                                                    \
      throw std::runtime_error(ss_.str());                                                   \
    }                                                                                        \
  } while (0)

#define CUDA_SYNC_CHECK()                                                                    \
  do {                                                                                       \
    cudaDeviceSynchronize();                                                                 \
    cudaError_t err_ = cudaGetLastError();                                                   \
    if (err_ != cudaSuccess) throw std::runtime_error(cudaGetErrorString(err_));             \
  } while (0)
