// Launchers of the learned-closure kernels (mlp_kernels.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "mlp_common.cuh"

namespace nsm {
namespace mlp {

cudaError_t setup_kernels();
cudaError_t launch_generate(long n, unsigned long long seed, double sd, double min_det, double K, double G, float* X,
                            float* Y, int* status, cudaStream_t s);
cudaError_t launch_residual_moment(long n, const float* X, const float* Y, float k_over_g, float in_scale,
                                   double* partial, int blocks, cudaStream_t s);
cudaError_t launch_images(const float* P, uint8_t* img, cudaStream_t s);
// One training step over `tiles` tiles of 128 points: point j = first + tile*128 + lane
// is sample (stride_a * j + offset_b) mod n.
cudaError_t launch_train(int tiles, const float* X, const float* Y, long n, long first, long stride_a, long offset_b,
                         const uint8_t* img, const float* P, const Scales& sc, float inv_batch, float* grad_partial,
                         float* loss_partial, int* status, cudaStream_t s);
// Sum of the per-CTA gradients, Adam step, and the updated parameters' BF16
// operand-image entries (img, written in place).
cudaError_t launch_adam(int ncta, const float* grad_partial, float* P, float* m1, float* m2, float lr, float beta1,
                        float beta2, float eps, float bc1, float bc2, uint8_t* img, cudaStream_t s);
cudaError_t launch_sum_gradient(int ncta, const float* grad_partial, float* g, cudaStream_t s);
cudaError_t launch_predict(long n, const float* H, const uint8_t* img, const float* P, const Scales& sc, double K,
                           double G, double* sigma, int* fallback, int* status, cudaStream_t s);

}  // namespace mlp
}  // namespace nsm
