// The element kernel with the learned closure as material (mlp_element.cu).
#pragma once

#include "mlp_common.cuh"
#include "nsm_kernels.cuh"

struct nsm_mlp;

namespace nsm {
namespace mlp {

struct MlpElementArgs {
  const uint8_t*      img;             // BF16 operand images
  const float*        P;               // FP32 parameters (biases b2, b3)
  Scales              sc;
  unsigned long long* fallback_count;  // points outside the training envelope
};

cudaError_t setup_element_kernel();
cudaError_t launch_element_mlp(const ElementArgs& a, const MlpElementArgs& m, cudaStream_t stream);

// The closure's device data for the element kernel (defined with nsm_mlp).
bool element_args(nsm_mlp* m, MlpElementArgs* out, double* bulk, double* shear);

}  // namespace mlp
}  // namespace nsm
