// Diagnostic: one 128 x N x K BF16 GEMM on the 5th-generation tensor cores
// (D = A B^T, FP32 accumulate), through exactly the primitives and operand
// layout the MLP closure uses (tc05.cuh).  It lets a test check the
// descriptors and the tensor-memory read-back against a CPU product.
#include <cuda_runtime.h>

#include "../../include/nimble_gb300.h"
#include "tc05.cuh"

namespace {

using namespace nsm::tc;

__global__ void __launch_bounds__(128) k_tc_selftest(int N, int K, const float* __restrict__ A,
                                                     const float* __restrict__ B, float* __restrict__ D,
                                                     int* __restrict__ status)
{
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ uint64_t mbar;
  __shared__ uint32_t tmem_slot;
  const int           tid = threadIdx.x, warp = tid >> 5;
  uint8_t*            sA  = smem;
  uint8_t*            sB  = smem + 128 * K * 2;
  const uint32_t      ncols = N <= 32 ? 32 : (N <= 64 ? 64 : (N <= 128 ? 128 : 256));

  if (warp == 0) {
    tmem_alloc(&tmem_slot, ncols);
    tmem_relinquish();
  }
  if (tid == 0) mbar_init(&mbar, 1);
  // operands -> BF16, K-major core-matrix tiles
  for (int i = tid; i < 128 * K; i += 128) {
    int r = i / K, k = i % K;
    *reinterpret_cast<__nv_bfloat16*>(sA + kmajor_offset(r, k, K)) = __float2bfloat16_rn(A[i]);
  }
  for (int i = tid; i < N * K; i += 128) {
    int r = i / K, k = i % K;
    *reinterpret_cast<__nv_bfloat16*>(sB + kmajor_offset(r, k, K)) = __float2bfloat16_rn(B[i]);
  }
  fence_proxy_async();
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tbase = tmem_slot;
  if (tid == 0) {
    const uint32_t idesc = idesc_bf16_f32(128, N);
    for (int ks = 0; ks < K / 16; ks++) {
      uint64_t ad = smem_desc(smem_addr(sA) + ks * 2 * kLBO, kLBO, 16 * K);
      uint64_t bd = smem_desc(smem_addr(sB) + ks * 2 * kLBO, kLBO, 16 * K);
      mma_bf16(tbase, ad, bd, idesc, ks > 0);
    }
    mma_commit(&mbar);
  }
  const bool done = mbar_wait(&mbar, 0);
  fence_after_sync();
  if (done) {
    const int row = warp * 32 + (tid & 31);
    for (int c = 0; c < N; c += 16) {
      float v[16];
      tmem_ld16(tbase + ((uint32_t)(warp * 32) << 16) + c, v);
      tmem_wait_ld();
      for (int j = 0; j < 16; j++) D[row * N + c + j] = v[j];
    }
  } else if (tid == 0) {
    atomicOr(status, 1);
  }
  fence_before_sync();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tbase, ncols);
}

// The failure path of every tensor-core wait: tensor memory held, a wait on
// an mbarrier phase that nothing completes, bounded by `limit_us`
// microseconds; the kernel records the timeout, frees its columns and
// returns.
__global__ void __launch_bounds__(128) k_tc_wait_timeout(long limit_us, int* __restrict__ status)
{
  __shared__ uint64_t mbar;
  __shared__ uint32_t tmem_slot;
  const int           tid = threadIdx.x, warp = tid >> 5;
  if (warp == 0) {
    tmem_alloc(&tmem_slot, 32);
    tmem_relinquish();
  }
  if (tid == 0) mbar_init(&mbar, 1);
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const bool done = mbar_wait(&mbar, 0, 1000ull * (uint64_t)limit_us);  // no arrival is ever made
  if (!done && tid == 0) atomicOr(status, 1);
  fence_before_sync();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem_slot, 32);
}

}  // namespace

extern "C" int nsm_tc_wait_timeout_selftest(long limit_us, int* timed_out)
{
  if (!timed_out || limit_us < 1 || limit_us > 100000) return NSM_ERR_INVALID_ARGUMENT;
  int* dS = nullptr;
  int  rc = NSM_OK, status = 0;
  if (cudaMalloc(&dS, sizeof(int)) != cudaSuccess || cudaMemset(dS, 0, sizeof(int)) != cudaSuccess) rc = NSM_ERR_CUDA;
  if (rc == NSM_OK) {
    k_tc_wait_timeout<<<1, 128>>>(limit_us, dS);
    if (cudaDeviceSynchronize() != cudaSuccess ||
        cudaMemcpy(&status, dS, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
      rc = NSM_ERR_CUDA;
  }
  cudaFree(dS);
  *timed_out = status;
  return rc;
}

extern "C" int nsm_tc_selftest(int N, int K, const float* A, const float* B, float* D)
{
  if (!A || !B || !D || N < 16 || N > 256 || (N % 16) || K < 16 || K > 128 || (K % 16))
    return NSM_ERR_INVALID_ARGUMENT;
  float *dA = nullptr, *dB = nullptr, *dD = nullptr;
  int*   dS = nullptr;
  int    status = 0, rc = NSM_OK;
  const size_t smem = (size_t)(128 + N) * K * 2 + 32768;  // operands + slack past the end
  if (cudaMalloc(&dA, sizeof(float) * 128 * K) != cudaSuccess || cudaMalloc(&dB, sizeof(float) * N * K) != cudaSuccess ||
      cudaMalloc(&dD, sizeof(float) * 128 * N) != cudaSuccess || cudaMalloc(&dS, sizeof(int)) != cudaSuccess) {
    rc = NSM_ERR_CUDA;
  }
  if (rc == NSM_OK && (cudaMemcpy(dA, A, sizeof(float) * 128 * K, cudaMemcpyHostToDevice) != cudaSuccess ||
                       cudaMemcpy(dB, B, sizeof(float) * N * K, cudaMemcpyHostToDevice) != cudaSuccess ||
                       cudaMemset(dS, 0, sizeof(int)) != cudaSuccess ||
                       cudaFuncSetAttribute(k_tc_selftest, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
                           cudaSuccess))
    rc = NSM_ERR_CUDA;
  if (rc == NSM_OK) {
    k_tc_selftest<<<1, 128, smem>>>(N, K, dA, dB, dD, dS);
    if (cudaDeviceSynchronize() != cudaSuccess) rc = NSM_ERR_CUDA;
  }
  if (rc == NSM_OK && (cudaMemcpy(D, dD, sizeof(float) * 128 * N, cudaMemcpyDeviceToHost) != cudaSuccess ||
                       cudaMemcpy(&status, dS, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess))
    rc = NSM_ERR_CUDA;
  if (rc == NSM_OK && status) rc = NSM_ERR_STATE;  // the completion wait timed out
  cudaFree(dA);
  cudaFree(dB);
  cudaFree(dD);
  cudaFree(dS);
  return rc;
}
