// logreg_tc.cu -- tensor-core (tcgen05) BF16 split-precision logistic potential.
#include "common.cuh"
#include "internal.h"

namespace gbn {

bool logreg_tc_supported(const ModelDev&) { return false; }
cudaError_t logreg_tc_prepare(ModelDev&, int) { return cudaErrorNotSupported; }
void logreg_tc_free(ModelDev&) {}
cudaError_t logreg_tc_launch(ModelDev&, const float*, int, double*, float*, const int32_t*, cudaStream_t) {
  return cudaErrorNotSupported;
}

}  // namespace gbn
