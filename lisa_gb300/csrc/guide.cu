// MLP path guide (placeholder until the tensor-core kernels land).
#include "guide.cuh"

namespace lisa {

GuideNet::~GuideNet() {}

Status guide_renderer_init(Renderer&) { return Status(LISA_ERR_UNSUPPORTED, "guided mode not built yet"); }

}  // namespace lisa

using namespace lisa;
extern "C" {
struct lisa_guide {};
int lisa_guide_create(uint32_t, lisa_guide**) { return LISA_ERR_UNSUPPORTED; }
void lisa_guide_destroy(lisa_guide*) {}
int lisa_guide_get_params(lisa_guide*, float*) { return LISA_ERR_UNSUPPORTED; }
int lisa_guide_set_params(lisa_guide*, const float*) { return LISA_ERR_UNSUPPORTED; }
int lisa_guide_forward(lisa_guide*, const float*, uint32_t, float*) { return LISA_ERR_UNSUPPORTED; }
int lisa_guide_train_step(lisa_guide*, const float*, const float*, const float*, uint32_t, float, float*, float*) {
  return LISA_ERR_UNSUPPORTED;
}
int lisa_renderer_guide(lisa_renderer*, int32_t, lisa_guide**) { return LISA_ERR_UNSUPPORTED; }
}
