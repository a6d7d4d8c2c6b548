// Block-material callbacks written with the engine's own arithmetic: the
// neo-Hookean stress from F at step n+1 (src/nimble_material.cc:252-310),
// without state, and the same with one history variable per point,
// state_np1 = state_n + |det F_np1 - det F_n|.  They show the plugin
// contract end to end (views of F and sigma at n and n+1, per-point state at
// n and n+1, work enqueued on the engine's stream) and check it against the
// built-in material.
#include "../../include/nimble_gb300.h"
#include "hex_math.cuh"
#include "nsm_kernels.cuh"

namespace nsm {
namespace {

template <typename T>
__global__ void k_example_stress(int e0, int e1, long ld_e, const T* __restrict__ rec_n, T* __restrict__ rec_np1,
                                 double K, double G, int num_state, const double* __restrict__ state_n,
                                 double* __restrict__ state_np1)
{
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;  // (element, point)
  if (i >= (long)(e1 - e0) * 8) return;
  const long   e   = e0 + i / 8;
  const int    p   = (int)(i % 8);
  const size_t at  = ((size_t)p * ld_e + e) * kIpRecord;
  T*           r   = rec_np1 + at;
  T            F[3][3], H[3][3], C[3][3];
#pragma unroll
  for (int a = 0; a < 3; a++)
#pragma unroll
    for (int b = 0; b < 3; b++) {
      F[a][b] = r[full_slot(a, b)];
      H[a][b] = a == b ? F[a][b] - T(1) : F[a][b];
    }
  const T J = cofactor3<T>(F, C);
  T       sig[6];
  neohookean_stress<T>(H, J, T(K), T(G), sig);
#pragma unroll
  for (int q = 0; q < 6; q++) r[9 + q] = sig[q];
  if (state_np1 != nullptr) {
    const T* rn = rec_n + at;
    T        Fn[3][3], Cn[3][3];
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
      for (int b = 0; b < 3; b++) Fn[a][b] = rn[full_slot(a, b)];
    const T      Jn = cofactor3<T>(Fn, Cn);
    const size_t s  = ((size_t)p * ld_e + e) * num_state;
    state_np1[s]    = state_n[s] + fabs((double)J - (double)Jn);
    for (int k = 1; k < num_state; k++) state_np1[s + k] = state_n[s + k];
  }
}

int launch_example(const nsm_stress_request* r, bool history)
{
  if (!r || r->elem_end < r->elem_begin) return 1;
  if (history && (r->num_state < 1 || !r->state_n || !r->state_np1)) return 1;
  const long count = (long)(r->elem_end - r->elem_begin) * 8;
  if (count == 0) return 0;
  const unsigned     grid = (unsigned)((count + 127) / 128);
  cudaStream_t       s    = static_cast<cudaStream_t>(r->stream);
  const double*      sn   = history ? r->state_n : nullptr;
  double*            snp1 = history ? r->state_np1 : nullptr;
  if (r->precision == NSM_PRECISION_FP64)
    k_example_stress<double><<<grid, 128, 0, s>>>(r->elem_begin, r->elem_end, r->ld_e,
                                                  static_cast<const double*>(r->records_n),
                                                  static_cast<double*>(r->records_np1), r->bulk_modulus,
                                                  r->shear_modulus, r->num_state, sn, snp1);
  else
    k_example_stress<float><<<grid, 128, 0, s>>>(r->elem_begin, r->elem_end, r->ld_e,
                                                 static_cast<const float*>(r->records_n),
                                                 static_cast<float*>(r->records_np1), r->bulk_modulus,
                                                 r->shear_modulus, r->num_state, sn, snp1);
  return cudaGetLastError() == cudaSuccess ? 0 : 1;
}

}  // namespace
}  // namespace nsm

extern "C" int nsm_example_neohookean_callback(void*, const nsm_stress_request* request)
{
  return nsm::launch_example(request, false);
}

extern "C" int nsm_example_history_callback(void*, const nsm_stress_request* request)
{
  return nsm::launch_example(request, true);
}
