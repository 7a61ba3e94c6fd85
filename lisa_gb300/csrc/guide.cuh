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
  float* loss = nullptr;      // device scalar accumulator (cleared by each Adam step)
  float* loss_last = nullptr; // loss of the batch of the last Adam step
  uint32_t* status = nullptr; // device status word (time-outs, non-finite values)
  uint32_t* d_step = nullptr; // Adam step count (device)
  // per-CTA partial gradients and losses of the last training launch (one
  // slot per CTA, summed by the Adam step); owned, or shared by a
  // renderer's guides (their training runs one after another on its stream)
  float* grad_part = nullptr;
  float* loss_part = nullptr;
  bool owns_part = false;
  uint32_t nparts = 0;        // slots the last training launch wrote
  ~GuideNet();
};

// Sample sources of the guide kernels.  RAW: n x 64 FP32 features (plus
// directions and weights for training).  GEOM: 4 float4 per sample --
// (p.xyz, N.x) (N.y, N.z, v.x, v.y) (v.z, w.xyz) (weight, emitter flag, -, -) --
// encoded against the scene box.  NEE: the renderer's emitter-search queue
// (hit point, normal, incoming direction).
enum { SRC_RAW = 0, SRC_GEOM = 1, SRC_NEE = 2 };

struct GuideSrc {
  const float* raw;
  const float* dirs;
  const float* weights;
  const float4* geom;
  const float4* nee_a;
  const float4* nee_b;
  const float4* nee_c;
  const float4* ps_att;   // SRC_NEE: path state (emitter flag in .w)
  const uint32_t* count;  // device sample count, clamped to n; null: use n
  uint32_t n;             // samples [first, min(count, n)) are used
  uint32_t first;
  uint32_t no_flag;       // SRC_NEE: the emitter-flag feature is 0 (physically based estimator)
  float bmin[3], bmax[3];
};

// own_partials: allocate the network's own partial-gradient slots (a
// renderer's guides share the renderer's instead)
Status guide_create(uint32_t seed, std::unique_ptr<GuideNet>& out, cudaStream_t s, bool own_partials);
// Fills n training samples from the wave's guided-vertex records (host
// launcher in wavefront.cu).
Status guide_collect(Renderer& r, int wave, uint32_t cap, cudaStream_t s);
// outputs: max_n x 40 floats (entries beyond the live count are not written)
Status guide_launch_infer(GuideNet& g, const GuideSrc& src, int src_kind, float* out, uint32_t max_n,
                          cudaStream_t s);
// one training launch on RAW samples (the guide's own C ABI): each CTA
// writes its partial gradient and loss to its slot; with adam_follows the
// device step count advances for the next Adam step
Status guide_launch_train(GuideNet& g, const GuideSrc& src, float inv_n, uint32_t max_n, cudaStream_t s,
                          bool adam_follows);
// Up to `rounds` Adam steps on slices of `chunk` samples of src (RAW or
// GEOM), in one cooperative launch; grid_bar is one device word of scratch
Status guide_launch_train_rounds(GuideNet& g, const GuideSrc& src, int src_kind, uint32_t chunk, uint32_t rounds,
                                 float lr, uint32_t* grid_bar, cudaStream_t s, unsigned long long* sample_count);
// g.grads / g.loss = sums of the last training launch's partials
Status guide_launch_reduce(GuideNet& g, cudaStream_t s);
// Adam step on the summed partials; also refreshes the BF16 weights and
// moves the loss to loss_last
Status guide_launch_adam(GuideNet& g, float lr, cudaStream_t s);
Status guide_check_status(GuideNet& g, cudaStream_t s);
Status guide_renderer_init(Renderer& r);
// Shared-memory attributes of the renderer's fused inference kernels (wavefront.cu).
Status guided_infer_setup();

}  // namespace lisa

// C-ABI handle of a guide: owns its network, or borrows a renderer's.
struct lisa_guide {
  std::unique_ptr<lisa::GuideNet> net;  // owned network
  lisa::GuideNet* borrowed = nullptr;   // a renderer's network
  cudaStream_t stream = nullptr;
  bool owns_stream = true;
  lisa::GuideNet& get() { return borrowed ? *borrowed : *net; }
};
