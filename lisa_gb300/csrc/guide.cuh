// MLP path guide: interfaces shared with the renderer.
#pragma once

#include <cuda_bf16.h>
#include <stdint.h>

#include <memory>

#include "lisa_internal.h"
#include "wavefront.cuh"

namespace lisa {

// One guide network on the device: FP32 master parameters, Adam moments,
// FP32 gradients and the BF16 copies the tensor-core kernels read.
struct GuideNet {
  float* master = nullptr;
  float* adam_m = nullptr;
  float* adam_v = nullptr;
  float* grads = nullptr;
  uint16_t* w_bf16 = nullptr;
  float* loss = nullptr;      // device scalar accumulator
  uint32_t* status = nullptr; // device status word (time-outs, non-finite values)
  uint32_t step = 0;
  ~GuideNet();
};

Status guide_renderer_init(Renderer& r);

}  // namespace lisa
