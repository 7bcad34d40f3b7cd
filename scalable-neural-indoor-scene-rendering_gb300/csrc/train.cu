// Training forward / hand-written adjoint (filled in by the training kernels).
#include "kernels.h"
#include "snisr.h"
#include "snisr_internal.h"

namespace snisr {
int train_ctrl_words(int NT) { return CTRL_HEADER + 4 * NT + 2; }
}  // namespace snisr

using namespace snisr;

extern "C" {
snisr_status snisr_train_forward(snisr_scene*, const float*, const float*, const float*, const float*, const float*,
                                 int64_t, int32_t, float*, void*) {
  return set_error(SNISR_UNSUPPORTED, "train_forward: not built yet");
}
snisr_status snisr_train_backward(snisr_scene*, const float*, const float*, const float*, const float*, const float*,
                                  int64_t, int32_t, const float*, const float*, float*, float*, float*, void*) {
  return set_error(SNISR_UNSUPPORTED, "train_backward: not built yet");
}
}
