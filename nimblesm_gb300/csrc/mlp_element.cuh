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
  const float*        geo;             // [ld_e][8][12] per point: J_X^{-1} (9, row-major), det J_X, 2 unused
};

cudaError_t setup_element_kernel();
cudaError_t launch_element_mlp(const ElementArgs& a, const MlpElementArgs& m, cudaStream_t stream);
// The closure kernel's reference geometry, from the FP32 copy of X: per
// point J_X^{-1} and det J_X as the kernel would form them, into geo
// ([ld_e][8][12] floats).
cudaError_t launch_closure_geometry(const ElementArgs& a, float* geo, cudaStream_t stream);

// The closure's device data for the element kernel (defined with nsm_mlp).
bool element_args(nsm_mlp* m, MlpElementArgs* out, double* bulk, double* shear);

}  // namespace mlp
}  // namespace nsm
