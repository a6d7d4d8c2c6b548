// Diagnostic: the FP64 fused-multiply-add rate of this GPU, the roof that
// binds the FP64 element kernel (GB300's FP64 pipe issues 2 DFMA per SM per
// cycle).  Every thread runs 16 independent FMA chains, 64 warps per SM; the
// chains' sums are stored so that nothing is eliminated.
#include <cuda_runtime.h>

#include "../../include/nimble_gb300.h"
#include "nsm_kernels.cuh"

namespace {

constexpr int kChains = 16;

__global__ void __launch_bounds__(256) k_dfma_probe(int iters, double seed, double* __restrict__ out)
{
  double       a[kChains];
  const double m = 0.9999999, c = 1.0e-7;
#pragma unroll
  for (int j = 0; j < kChains; j++) a[j] = seed + threadIdx.x + j;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int j = 0; j < kChains; j++) a[j] = fma(a[j], m, c);
  }
  double s = 0.0;
#pragma unroll
  for (int j = 0; j < kChains; j++) s += a[j];
  out[blockIdx.x * (size_t)blockDim.x + threadIdx.x] = s;
}

}  // namespace

extern "C" int nsm_fp64_peak_probe(int device, double* tflops)
{
  if (!tflops) return NSM_ERR_INVALID_ARGUMENT;
  if (cudaSetDevice(device) != cudaSuccess) return NSM_ERR_CUDA;
  const int    blocks = nsm::num_sms() * 8, threads = 256, iters = 1024;
  double*      out    = nullptr;
  cudaEvent_t  t0 = nullptr, t1 = nullptr;
  int          rc   = NSM_OK;
  float        best = 0.0f;
  if (cudaMalloc(&out, sizeof(double) * blocks * threads) != cudaSuccess || cudaEventCreate(&t0) != cudaSuccess ||
      cudaEventCreate(&t1) != cudaSuccess)
    rc = NSM_ERR_CUDA;
  for (int rep = 0; rep < 4 && rc == NSM_OK; rep++) {  // the first launch is a warm-up
    cudaEventRecord(t0);
    k_dfma_probe<<<blocks, threads>>>(iters, 1.0 + rep, out);
    cudaEventRecord(t1);
    float ms = 0.0f;
    if (cudaEventSynchronize(t1) != cudaSuccess || cudaEventElapsedTime(&ms, t0, t1) != cudaSuccess) {
      rc = NSM_ERR_CUDA;
      break;
    }
    if (rep > 0 && (best == 0.0f || ms < best)) best = ms;
  }
  if (rc == NSM_OK)
    *tflops = 2.0 * kChains * (double)iters * blocks * threads / (best * 1e-3) / 1e12;
  if (t0) cudaEventDestroy(t0);
  if (t1) cudaEventDestroy(t1);
  cudaFree(out);
  return rc;
}

extern "C" int nsm_device_sm_count(int device, int* count)
{
  if (!count) return NSM_ERR_INVALID_ARGUMENT;
  return cudaDeviceGetAttribute(count, cudaDevAttrMultiProcessorCount, device) == cudaSuccess ? NSM_OK : NSM_ERR_CUDA;
}
