// The learned constitutive closure: a 9 -> 64 -> 64 -> 6 MLP (GELU) mapping
// the displacement gradient H = F - I to the Cauchy stress over the shear
// modulus, with BF16 weights and FP32 accumulation on the 5th-generation
// tensor cores.
//
// The network is placed on the material's second-order expansion and a cubic
// gate:
//   sigma / G = B(H) + s_r * |x|^3 * MLP(x),   x = H * in_scale,
// where B = L + Q is the neo-Hookean stress to second order in H: L its
// small-strain limit (K/G tr(eps) I + 2 dev(eps), eps = sym H) and Q the
// quadratic terms (base_part below).  The remainder sigma/G - B(H) is
// O(|H|^3), so the network learns the bounded, direction-dependent ratio
// (sigma/G - B) / |x|^3, and its own error is multiplied by |x|^3.  A
// network's error is largest where its training data is thinnest, near
// H = 0; with the gate there it cannot disturb the response of a dynamic
// run (strains ~1e-3, where the quadratic terms are ~1e-3 of the stress and
// the remainder ~1e-6), while it carries the material's higher-order response
// over the training envelope.
//
// Parameters (FP32 master copy, kParams floats): W1[64][9], b1[64], W2[64][64],
// b2[64], W3[6][64], b3[6].  BF16 operand images in the shared-memory tile
// layout of tc05.cuh are derived from them after every update:
//   W1x [64][32]: columns 0-8 W1, 9 b1, 16-24 W1 again.  The input row is
//                 [hi(x) (9), 1, 0 x6, lo(x) (9), 0 x7] with hi = bf16(x) and
//                 lo = bf16(x - hi): a two-term BF16 split of the input, so the
//                 first layer sees the input to ~16 significant bits, and the
//                 bias rides in the constant column.
//   W2  [64][64], W3x [16][64] (rows 0-5 W3), and for the backward pass the
//   transposes W2t [64][64] and W3t [64][16].
#pragma once

#include <cuda_bf16.h>

#include "tc05.cuh"

namespace nsm {
namespace mlp {

constexpr int kIn = 9, kHid = 64, kOut = 6;
constexpr int kInX  = 32;  // extended input width (two-term split + bias column)
constexpr int kOutX = 16;  // padded output width
constexpr int oW1 = 0, ob1 = oW1 + kHid * kIn, oW2 = ob1 + kHid, ob2 = oW2 + kHid * kHid, oW3 = ob2 + kHid,
              ob3 = oW3 + kOut * kHid, kParams = ob3 + kOut;  // 5190

// operand images (bytes), in the order they are laid out
constexpr int kImgW1 = kHid * kInX * 2, kImgW2 = kHid * kHid * 2, kImgW3 = kOutX * kHid * 2,
              kImgW2t = kHid * kHid * 2, kImgW3t = kHid * kOutX * 2;
constexpr int kOffW1 = 0, kOffW2 = kOffW1 + kImgW1, kOffW3 = kOffW2 + kImgW2, kOffW2t = kOffW3 + kImgW3,
              kOffW3t = kOffW2t + kImgW2t, kImgBytes = kOffW3t + kImgW3t;  // 24576

struct Scales {
  float in_scale;   // x = H * in_scale (1 / perturbation)
  float res_scale;  // s_r: rms of (sigma/G - B(H)) / |x|^3 over the training set
  float k_over_g;   // bulk / shear of the trained material
  float envelope;   // |H_ij| bound of the training envelope
  float min_det;    // det F bound of the training envelope
};

// The activation: GELU in its sigmoid form, x sigma(1.702 x) (Hendrycks &
// Gimpel 2016), written as a(u) = u (1 + tanh u) = 2 u sigma(2 u) with
// u = 0.851 x.  The factors 0.851 and 1 / 1.702 sit in the adjacent layers'
// weights, which training learns directly, so a pair of activations costs one
// packed fused multiply-add and two hardware tanh (tanh.approx.f32, relative
// error about 2^-11, below the BF16 rounding of the activations).  Training,
// inference and the CPU oracle all use this form.

__device__ __forceinline__ float tanh_approx(float u)
{
  float t;
  asm("tanh.approx.f32 %0, %1;" : "=f"(t) : "f"(u));
  return t;
}
__device__ __forceinline__ float act(float u)
{
  const float t = tanh_approx(u);
  return fmaf(u, t, u);
}
// a'(u) = 1 + t + u (1 - t^2), t = tanh u
__device__ __forceinline__ float act_grad(float u)
{
  const float t = tanh_approx(u);
  return fmaf(u, fmaf(-t, t, 1.0f), 1.0f + t);
}

// ---- packed FP32x2 arithmetic (fma.rn.f32x2, sm_100 and later) ----
// Each lane is the IEEE round-to-nearest FP32 operation, so a packed
// evaluation is bitwise the scalar one in the same order.
using f32x2 = unsigned long long;
__device__ __forceinline__ f32x2 f2_pack(float x, float y)
{
  f32x2 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(x), "f"(y));
  return r;
}
__device__ __forceinline__ void f2_unpack(f32x2 v, float& x, float& y) { asm("mov.b64 {%0, %1}, %2;" : "=f"(x), "=f"(y) : "l"(v)); }
__device__ __forceinline__ f32x2 f2_fma(f32x2 a, f32x2 b, f32x2 c)
{
  f32x2 d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}

// The activation of two pre-activations, u + u tanh(u), packed to a BF16 pair
// (low half = first value); each lane is bitwise act().
__device__ __forceinline__ uint32_t act_bf16(f32x2 u)
{
  float u0, u1;
  f2_unpack(u, u0, u1);
  float g0, g1;
  f2_unpack(f2_fma(u, f2_pack(tanh_approx(u0), tanh_approx(u1)), u), g0, g1);
  __nv_bfloat162 b = __floats2bfloat162_rn(g0, g1);
  return *reinterpret_cast<uint32_t*>(&b);
}

// The neo-Hookean stress over G to second order in H (x row-major H,
// symmetric order xx, yy, zz, xy, yz, zx).  With J = det(I + H) and the
// reference's sigma = K/2 (J - 1/J) I + G J^{-5/3} dev(F F^T)
// (src/nimble_material.cc:252-310), expanding to second order:
//   K/2 (J - 1/J) = K (tr H - tr(H H) / 2),
//   J^{-5/3} dev(F F^T) = 2 dev(eps) + H H^T - |H|^2 / 3 I - 10/3 tr(H) dev(eps),
// so B = [K/G (tr H - tr(H H)/2) - |H|^2 / 3] I + (2 - 10/3 tr H) dev(eps) + H H^T.
__device__ __forceinline__ void base_part(const float x[9], float k_over_g, float B[6])
{
  const float tr  = x[0] + x[4] + x[8];
  const float d   = tr * (1.0f / 3.0f);
  const float b00 = x[0] * x[0] + x[1] * x[1] + x[2] * x[2];
  const float b11 = x[3] * x[3] + x[4] * x[4] + x[5] * x[5];
  const float b22 = x[6] * x[6] + x[7] * x[7] + x[8] * x[8];
  const float b01 = x[0] * x[3] + x[1] * x[4] + x[2] * x[5];
  const float b12 = x[3] * x[6] + x[4] * x[7] + x[5] * x[8];
  const float b20 = x[6] * x[0] + x[7] * x[1] + x[8] * x[2];
  const float trhh = x[0] * x[0] + x[4] * x[4] + x[8] * x[8] + 2.0f * (x[1] * x[3] + x[5] * x[7] + x[2] * x[6]);
  const float iso  = k_over_g * (tr - 0.5f * trhh) - (b00 + b11 + b22) * (1.0f / 3.0f);
  const float c    = 2.0f - (10.0f / 3.0f) * tr;
  B[0]             = iso + c * (x[0] - d) + b00;
  B[1]             = iso + c * (x[4] - d) + b11;
  B[2]             = iso + c * (x[8] - d) + b22;
  B[3]             = 0.5f * c * (x[1] + x[3]) + b01;
  B[4]             = 0.5f * c * (x[5] + x[7]) + b12;
  B[5]             = 0.5f * c * (x[6] + x[2]) + b20;
}

// The cubic gate |x|^3 (floored so the training target stays finite).
__device__ __forceinline__ float gate(const float xs[9])
{
  float g2 = 0.0f;
#pragma unroll
  for (int j = 0; j < 9; j++) g2 += xs[j] * xs[j];
  return fmaxf(g2 * sqrtf(g2), 1e-30f);
}

// Inside the training envelope: every |H_ij| <= envelope and det F >= min_det.
__device__ __forceinline__ bool in_envelope(const float h[9], const Scales& s)
{
  float m = 0.0f;
#pragma unroll
  for (int j = 0; j < 9; j++) m = fmaxf(m, fabsf(h[j]));
  const float f00 = 1 + h[0], f11 = 1 + h[4], f22 = 1 + h[8];
  const float det = f00 * (f11 * f22 - h[5] * h[7]) - h[1] * (h[3] * f22 - h[5] * h[6]) + h[2] * (h[3] * h[7] - f11 * h[6]);
  return m <= s.envelope && det >= s.min_det;
}

// Write 8 consecutive features (one 16-byte chunk) of row r of a K-major tile.
__device__ __forceinline__ void store_chunk(uint8_t* tile, int r, int k0, int K, const float* v)
{
  __nv_bfloat162 p0 = __floats2bfloat162_rn(v[0], v[1]), p1 = __floats2bfloat162_rn(v[2], v[3]),
                 p2 = __floats2bfloat162_rn(v[4], v[5]), p3 = __floats2bfloat162_rn(v[6], v[7]);
  uint4 w;
  w.x = *reinterpret_cast<uint32_t*>(&p0);
  w.y = *reinterpret_cast<uint32_t*>(&p1);
  w.z = *reinterpret_cast<uint32_t*>(&p2);
  w.w = *reinterpret_cast<uint32_t*>(&p3);
  *reinterpret_cast<uint4*>(tile + tc::kmajor_offset(r, k0, K)) = w;
}

__device__ __forceinline__ void store_bf16(uint8_t* tile, int r, int k, int K, float v)
{
  *reinterpret_cast<__nv_bfloat16*>(tile + tc::kmajor_offset(r, k, K)) = __float2bfloat16_rn(v);
}

// The extended input row [hi(x), 1, 0.., lo(x), 0..] of one point.
__device__ __forceinline__ void input_row(const float x[9], float row[kInX])
{
#pragma unroll
  for (int j = 0; j < kInX; j++) row[j] = 0.0f;
#pragma unroll
  for (int j = 0; j < 9; j++) {
    const float hi = __bfloat162float(__float2bfloat16_rn(x[j]));
    row[j]         = hi;
    row[16 + j]    = x[j] - hi;
  }
  row[9] = 1.0f;
}

}  // namespace mlp
}  // namespace nsm
