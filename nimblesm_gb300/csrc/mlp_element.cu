// Element kernel with the learned closure as the material update: the FP32
// element kernel (element_kernels.cu) with the neo-Hookean stress replaced
// by the MLP of mlp_common.cuh, evaluated on the 5th-generation tensor cores
// inside the element kernel.
//
// One CTA = 128 elements (thread r owns element r) = 8 tiles of 128 points,
// tile p holding integration point p of every element.  Row r of a tile is
// thread r's point, so each layer's accumulator row comes back to the thread
// that owns the element (tensor-memory lane r) with no data exchange.  Points
// outside the training envelope take the plain neo-Hookean stress (FP32) and
// are counted.
#include <cuda_runtime.h>

#include "hex_math.cuh"
#include "mlp_common.cuh"
#include "mlp_element.cuh"
#include "nsm_kernels.cuh"

namespace nsm {
namespace mlp {

using namespace tc;

namespace el {
constexpr int X    = 0;                    // [128][32]
constexpr int A1   = X + 128 * kInX * 2;   // [128][64]
constexpr int A2   = A1 + 128 * kHid * 2;  // [128][64]
constexpr int W    = A2 + 128 * kHid * 2;  // W1x, W2, W3x images
constexpr int B    = W + kOffW2t;          // b2[64], b3[6]
constexpr int END  = B + 512;
constexpr int SMEM = END + 16384;
// Z1 and Z3 share columns (Z1 is consumed before layer 3 writes)
constexpr uint32_t cZ1 = 0, cZ2 = 64, cZ3 = 0, kCols = 128;
}  // namespace el

__device__ __forceinline__ void publish()
{
  fence_proxy_async();
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
}

__device__ __forceinline__ bool wait_commit(uint64_t* mbar, uint32_t& phase, int* err)
{
  const bool ok = mbar_wait(mbar, phase);
  phase ^= 1u;
  if (!ok) atomicOr(err, 1);
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  return *err == 0;
}

__device__ __forceinline__ void ld_cols(uint32_t tb, uint32_t col, int n16, float* v)
{
  const uint32_t lane_base = (uint32_t)((threadIdx.x >> 5) * 32) << 16;
  for (int c = 0; c < n16; c++) tmem_ld16(tb + lane_base + col + 16 * c, v + 16 * c);
  tmem_wait_ld();
}

__device__ __forceinline__ void layer(uint32_t d, const uint8_t* a, int Ka, const uint8_t* b, int N)
{
  const uint32_t idesc = idesc_bf16_f32(128, N);
  for (int ks = 0; ks < Ka / 16; ks++)
    mma_bf16(d, smem_desc(smem_addr(a) + ks * 2 * kLBO, kLBO, 16 * Ka), smem_desc(smem_addr(b) + ks * 2 * kLBO, kLBO, 16 * Ka),
             idesc, ks > 0);
}

__global__ void __launch_bounds__(128) k_element_mlp(ElementArgs a, MlpElementArgs m)
{
  extern __shared__ __align__(1024) uint8_t sm[];
  __shared__ uint64_t mbar;
  __shared__ uint32_t tslot;
  __shared__ int      err;
  const int           r = threadIdx.x, warp = r >> 5;
  const int           e = blockIdx.x * 128 + r;
  const bool          valid = e < a.E;
  const long          ld_e = a.ld_e, ld_n = a.ld_n;

  if (warp == 0) {
    tmem_alloc(&tslot, el::kCols);
    tmem_relinquish();
  }
  if (r == 0) {
    mbar_init(&mbar, 1);
    err = 0;
  }
  {
    const uint4* src = reinterpret_cast<const uint4*>(m.img);
    for (int i = r; i < kOffW2t / 16; i += 128) reinterpret_cast<uint4*>(sm + el::W)[i] = src[i];
    float* bias = reinterpret_cast<float*>(sm + el::B);
    if (r < kHid) bias[r] = m.P[ob2 + r];
    if (r < kOut) bias[64 + r] = m.P[ob3 + r];
  }
  const float* b2 = reinterpret_cast<const float*>(sm + el::B);
  const float* b3 = b2 + 64;

  // gradients of u and X at the points (as the FP32 element kernel)
  float Gu[3][3][2][2], GX[3][3][2][2];
  {
    float xu[8][3], xX[8][3];
    for (int n = 0; n < 8; n++) {
      const int id = valid ? __ldg(&a.conn[n * ld_e + e]) : 0;
      for (int k = 0; k < 3; k++) {
        xu[n][k] = valid ? __ldg(&a.uf[k * ld_n + id]) : 0.0f;
        xX[n][k] = valid ? __ldg(&a.Xf[k * ld_n + id]) : float(sign_bit(n, k));  // a unit cube for idle rows
      }
    }
    nodal_gradient<float>(xu, Gu);
    nodal_gradient<float>(xX, GX);
  }
  float S[3][3][2][2];
  for (int d = 0; d < 3; d++)
    for (int i = 0; i < 3; i++)
      for (int s = 0; s < 2; s++)
        for (int t = 0; t < 2; t++) S[d][i][s][t] = 0.0f;

  const bool     store = a.store_ip || (a.sched != nullptr && a.sched[(long)(*a.step_base + a.k) * a.num_groups].is_output);
  float*         rec   = reinterpret_cast<float*>(a.ip) + (size_t)e * kIpRecord;
  const uint32_t tb    = tslot;
  uint32_t       phase = 0;
  bool           bad = false;
  int            fallbacks = 0;
  const float    K = (float)a.bulk, Gm = (float)a.shear;

  for (int p = 0; p < 8; p++) {
    const int bit[3] = {sx_of(p), sy_of(p), sz_of(p)};
    float     JX[3][3], G0[3][3], det0;
    for (int i = 0; i < 3; i++)
      for (int d = 0; d < 3; d++) JX[i][d] = GX[d][i][bit[other1(d)]][bit[other2(d)]];
    invert3<float>(JX, G0, det0);
    float H[3][3], h[9];
    for (int i = 0; i < 3; i++)
      for (int J = 0; J < 3; J++) {
        float v = 0.0f;
        for (int d = 0; d < 3; d++) v += Gu[d][i][bit[other1(d)]][bit[other2(d)]] * G0[d][J];
        H[i][J]       = v;
        h[3 * i + J] = v;
      }
    // ---- MLP: layer 1 ----
    {
      float xs[9], row[kInX];
      for (int q = 0; q < 9; q++) xs[q] = h[q] * m.sc.in_scale;
      input_row(xs, row);
      for (int k0 = 0; k0 < kInX; k0 += 8) store_chunk(sm + el::X, r, k0, kInX, row + k0);
    }
    publish();
    if (r == 0) {
      layer(tb + el::cZ1, sm + el::X, kInX, sm + el::W + kOffW1, kHid);
      mma_commit(&mbar);
    }
    if (!wait_commit(&mbar, phase, &err)) break;
    {
      float z[64];
      ld_cols(tb, el::cZ1, 4, z);
      for (int q = 0; q < 64; q++) z[q] = gelu(z[q]);
      for (int k0 = 0; k0 < 64; k0 += 8) store_chunk(sm + el::A1, r, k0, kHid, z + k0);
    }
    publish();
    if (r == 0) {
      layer(tb + el::cZ2, sm + el::A1, kHid, sm + el::W + kOffW2, kHid);
      mma_commit(&mbar);
    }
    if (!wait_commit(&mbar, phase, &err)) break;
    {
      float z[64];
      ld_cols(tb, el::cZ2, 4, z);
      for (int q = 0; q < 64; q++) z[q] = gelu(z[q] + b2[q]);
      for (int k0 = 0; k0 < 64; k0 += 8) store_chunk(sm + el::A2, r, k0, kHid, z + k0);
    }
    publish();
    if (r == 0) {
      layer(tb + el::cZ3, sm + el::A2, kHid, sm + el::W + kOffW3, kOutX);
      mma_commit(&mbar);
    }
    if (!wait_commit(&mbar, phase, &err)) break;
    float sig[6];
    {
      float z[16];
      ld_cols(tb, el::cZ3, 1, z);
      if (in_envelope(h, m.sc)) {
        float L[6], xs[9];
        for (int q = 0; q < 9; q++) xs[q] = h[q] * m.sc.in_scale;
        linear_part(h, m.sc.k_over_g, L);
        const float g = gate(xs) * m.sc.res_scale;
        for (int q = 0; q < 6; q++) sig[q] = Gm * (L[q] + g * (z[q] + b3[q]));
      } else {
        float C[3][3], J;
        neohookean<float>(H, K, Gm, sig, C, J);
        fallbacks += valid ? 1 : 0;
      }
    }
    // ---- the rest of the element work, as the FP32 element kernel ----
    float F[3][3], C[3][3];
    for (int i = 0; i < 3; i++)
      for (int k = 0; k < 3; k++) F[i][k] = (i == k ? 1.0f : 0.0f) + H[i][k];
    C[0][0] = F[1][1] * F[2][2] - F[1][2] * F[2][1];
    C[0][1] = F[1][2] * F[2][0] - F[1][0] * F[2][2];
    C[0][2] = F[1][0] * F[2][1] - F[1][1] * F[2][0];
    C[1][0] = F[0][2] * F[2][1] - F[0][1] * F[2][2];
    C[1][1] = F[0][0] * F[2][2] - F[0][2] * F[2][0];
    C[1][2] = F[0][1] * F[2][0] - F[0][0] * F[2][1];
    C[2][0] = F[0][1] * F[1][2] - F[0][2] * F[1][1];
    C[2][1] = F[0][2] * F[1][0] - F[0][0] * F[1][2];
    C[2][2] = F[0][0] * F[1][1] - F[0][1] * F[1][0];
    const float J = F[0][0] * C[0][0] + F[0][1] * C[0][1] + F[0][2] * C[0][2];
    if (valid && (!(J > 0.0f) || !(det0 > 0.0f))) bad = true;
    if (valid && store) {
      float rr[kIpRecord];
      for (int i = 0; i < 3; i++)
        for (int k = 0; k < 3; k++) rr[full_slot(i, k)] = F[i][k];
      for (int q = 0; q < 6; q++) rr[9 + q] = sig[q];
      rr[15] = 0.0f;
      float* dst = rec + (size_t)p * ld_e * kIpRecord;
      for (int k = 0; k < kIpRecord; k += 4) *reinterpret_cast<float4*>(dst + k) = make_float4(rr[k], rr[k + 1], rr[k + 2], rr[k + 3]);
    }
    float P[3][3];
    for (int i = 0; i < 3; i++)
      for (int Jc = 0; Jc < 3; Jc++)
        P[i][Jc] = sig[sym_slot(i, 0)] * C[0][Jc] + sig[sym_slot(i, 1)] * C[1][Jc] + sig[sym_slot(i, 2)] * C[2][Jc];
    for (int d = 0; d < 3; d++)
      for (int i = 0; i < 3; i++) {
        const float q = G0[d][0] * P[i][0] + G0[d][1] * P[i][1] + G0[d][2] * P[i][2];
        S[d][i][bit[other1(d)]][bit[other2(d)]] += det0 * q;
      }
  }
  if (err == 0 && valid) {
    float f[8][3];
    for (int n = 0; n < 8; n++)
      for (int i = 0; i < 3; i++) f[n][i] = 0.0f;
    for (int d = 0; d < 3; d++) {
      const int o1 = other1(d), o2 = other2(d);
      for (int i = 0; i < 3; i++) {
        float R[2][2];
        bwd_transform<float>(S[d][i], R);
        for (int b = 0; b < 2; b++)
          for (int c = 0; c < 2; c++) {
            f[corner_axes(d, 1, o1, b, o2, c)][i] -= R[b][c];
            f[corner_axes(d, 0, o1, b, o2, c)][i] += R[b][c];
          }
      }
    }
    float* fo     = reinterpret_cast<float*>(a.fe) + (size_t)e * 24;
    bool   finite = true;
    for (int n = 0; n < 8; n++)
      for (int i = 0; i < 3; i++) finite = finite && isfinite(f[n][i]);
    for (int k = 0; k < 24; k += 4)
      *reinterpret_cast<float4*>(fo + k) = make_float4(f[k / 3][k % 3], f[(k + 1) / 3][(k + 1) % 3],
                                                       f[(k + 2) / 3][(k + 2) % 3], f[(k + 3) / 3][(k + 3) % 3]);
    if (bad || !finite) atomicOr(a.status, (bad ? NSM_STATUS_BAD_JACOBIAN : 0) | (finite ? 0 : NSM_STATUS_NONFINITE));
  }
  if (fallbacks) atomicAdd(m.fallback_count, (unsigned long long)fallbacks);
  if (r == 0 && err) atomicOr(a.status, NSM_STATUS_TIMEOUT);
  fence_before_sync();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tb, el::kCols);
}

cudaError_t setup_element_kernel()
{
  return cudaFuncSetAttribute(k_element_mlp, cudaFuncAttributeMaxDynamicSharedMemorySize, el::SMEM);
}

cudaError_t launch_element_mlp(const ElementArgs& a, const MlpElementArgs& m, cudaStream_t stream)
{
  if (a.E == 0) return cudaSuccess;
  k_element_mlp<<<(a.E + 127) / 128, 128, el::SMEM, stream>>>(a, m);
  return cudaGetLastError();
}

}  // namespace mlp
}  // namespace nsm
