// Device math of the hex8 element and the neo-Hookean material, shared by the
// element kernels and the energy kernel.
//
// What is computed is the reference's per-element work
// (src/nimble_block.cc:278-385): F at the 8 Gauss points
// (src/nimble_element.h:430-502), the neo-Hookean stress
// (src/nimble_material.cc:252-310) and the element nodal forces
// f_a = -sum_ip (dN_a/dx . sigma) det(dx/dxi) w (src/nimble_element.h:540-625).
// How it is computed is chosen to spend as few FP64 operations as possible
// (FP64 is this chip's narrow pipe, ~1.2 TFLOP/s):
//   * Tensor-product structure of the trilinear hex: du/dxi at the 8 points
//     takes only 4 distinct values (it does not depend on xi), formed from the
//     4 edge differences along xi by two 2-point transforms; same for eta and
//     zeta.  36 values replace the 72 sums of 8 products per point.  The
//     force assembly (transpose of the gradient) uses the same transform.
//   * H = F - I = (du/dxi) J_X^{-1}, with J_X^{-1} and det J_X precomputed
//     per point at setup; no cancellation in F - I, no per-step inverse.
//   * sigma from b - I = H + H^T + H H^T and J = det F through the cofactor
//     matrix (no polar decomposition: the reference's V V equals F F^T).
//   * J^{-1/3} from an FP32 seed and one third-order correction, so that
//     1/J = r^3 and J^{-5/3} = r^5 need no division.
//   * Forces from the first Piola-Kirchhoff form P = sigma cof(F), since
//     det(J_x) J_x^{-1} sigma = det(J_X) J_X^{-1} P^T.
#pragma once

#include "nsm_common.cuh"

namespace nsm {

template <typename T>
struct Weights {
  // w(+) = 1 + g, w(-) = 1 - g; the 1/8 of the shape functions is folded into c1, c2.
  static constexpr T wp = T(1.0 + kGauss);
  static constexpr T wm = T(1.0 - kGauss);
  static constexpr T c1 = T((1.0 + kGauss) / 8.0);
  static constexpr T c2 = T((1.0 - kGauss) / 8.0);
};

// Edge differences D[b][c] (b, c = sign bits along the two other axes) ->
// derivative values at the Gauss-point sign pairs out[s][t].
template <typename T>
__device__ __forceinline__ void fwd_transform(const T D[2][2], T out[2][2])
{
  using W = Weights<T>;
  T E[2][2];  // E[c][s]
#pragma unroll
  for (int c = 0; c < 2; c++) {
    E[c][1] = W::wp * D[1][c] + W::wm * D[0][c];
    E[c][0] = W::wm * D[1][c] + W::wp * D[0][c];
  }
#pragma unroll
  for (int s = 0; s < 2; s++) {
    out[s][1] = W::c1 * E[1][s] + W::c2 * E[0][s];
    out[s][0] = W::c2 * E[1][s] + W::c1 * E[0][s];
  }
}

// Adjoint of fwd_transform: sums at sign pairs S[s][t] -> edge values R[b][c].
template <typename T>
__device__ __forceinline__ void bwd_transform(const T S[2][2], T R[2][2])
{
  using W = Weights<T>;
  T Z[2][2];  // Z[s][c]
#pragma unroll
  for (int s = 0; s < 2; s++) {
    Z[s][1] = W::c1 * S[s][1] + W::c2 * S[s][0];
    Z[s][0] = W::c2 * S[s][1] + W::c1 * S[s][0];
  }
#pragma unroll
  for (int c = 0; c < 2; c++) {
    R[1][c] = W::wp * Z[1][c] + W::wm * Z[0][c];
    R[0][c] = W::wm * Z[1][c] + W::wp * Z[0][c];
  }
}

// Of the two points that share sign bits along the axes other than d (they
// differ in the bit along d), whether p is the lower-numbered one: the first
// to contribute to their sums.
__host__ __device__ constexpr bool first_of_pair(int d, int p)
{
  return p < corner_of(d == 0 ? 1 - sx_of(p) : sx_of(p), d == 1 ? 1 - sy_of(p) : sy_of(p),
                       d == 2 ? 1 - sz_of(p) : sz_of(p));
}

// Gradient values of a nodal field x[8][3]: G[d][i][s][t] = dx_i/dxi_d at the
// points whose sign bits along the other axes of d are (s, t).
template <typename T>
__device__ __forceinline__ void nodal_gradient(const T x[8][3], T G[3][3][2][2])
{
#pragma unroll
  for (int d = 0; d < 3; d++) {
    const int o1 = other1(d), o2 = other2(d);
#pragma unroll
    for (int i = 0; i < 3; i++) {
      T D[2][2];
#pragma unroll
      for (int b = 0; b < 2; b++)
#pragma unroll
        for (int c = 0; c < 2; c++)
          D[b][c] = x[corner_axes(d, 1, o1, b, o2, c)][i] - x[corner_axes(d, 0, o1, b, o2, c)][i];
      fwd_transform<T>(D, G[d][i]);
    }
  }
}

__device__ __forceinline__ double rcbrt_refined(double J)
{
  // FP32 seed, then y <- y (1 + e/3 + 2e^2/9) with e = 1 - J y^3 (error O(e^3)).
  double y  = (double)rcbrtf((float)J);
  double y3 = y * y * y;
  double e  = fma(-J, y3, 1.0);
  double c  = fma(e, 2.0 / 9.0, 1.0 / 3.0);
  return fma(y * e, c, y);
}
// FP32 form: J^{-1/3} = 2^{-log2(J)/3} with the hardware log2/exp2 (about 2 ulp).
__device__ __forceinline__ float rcbrt_refined(float J) { return exp2f(__log2f(J) * (-1.0f / 3.0f)); }

// Cofactor matrix of M (C[r][c] = cofactor of entry (r, c)) and det M.
template <typename T>
__device__ __forceinline__ T cofactor3(const T M[3][3], T C[3][3])
{
  C[0][0] = M[1][1] * M[2][2] - M[1][2] * M[2][1];
  C[0][1] = M[1][2] * M[2][0] - M[1][0] * M[2][2];
  C[0][2] = M[1][0] * M[2][1] - M[1][1] * M[2][0];
  C[1][0] = M[0][2] * M[2][1] - M[0][1] * M[2][2];
  C[1][1] = M[0][0] * M[2][2] - M[0][2] * M[2][0];
  C[1][2] = M[0][1] * M[2][0] - M[0][0] * M[2][1];
  C[2][0] = M[0][1] * M[1][2] - M[0][2] * M[1][1];
  C[2][1] = M[0][2] * M[1][0] - M[0][0] * M[1][2];
  C[2][2] = M[0][0] * M[1][1] - M[0][1] * M[1][0];
  return M[0][0] * C[0][0] + M[0][1] * C[0][1] + M[0][2] * C[0][2];
}

// Neo-Hookean Cauchy stress (reference src/nimble_material.cc:252-310) from
// H = F - I and J = det F: sigma = K/2 (J - 1/J) I + G J^{-5/3} dev(F F^T).
template <typename T>
__device__ __forceinline__ void neohookean_stress(const T H[3][3], T J, T K, T G, T sig[6])
{
  // b - I = H + H^T + H H^T, one add and three fused multiply-adds per entry
  T B[6];
#pragma unroll
  for (int q = 0; q < 6; q++) {
    const int i = q < 3 ? q : (q == 3 ? 0 : (q == 4 ? 1 : 2));
    const int j = q < 3 ? q : (q == 3 ? 1 : (q == 4 ? 2 : 0));
    B[q]        = fma(H[i][0], H[j][0], fma(H[i][1], H[j][1], fma(H[i][2], H[j][2], H[i][j] + H[j][i])));
  }
  const T r   = rcbrt_refined(J);
  const T r2  = r * r;
  const T r3  = r2 * r;
  const T r5  = r3 * r2;
  const T p   = T(0.5) * K * (J - r3);
  const T m   = (B[0] + B[1] + B[2]) * T(1.0 / 3.0);
  const T Gr5 = G * r5;
  const T q0  = fma(-Gr5, m, p);  // p - G J^{-5/3} tr(b)/3
  sig[0]      = fma(Gr5, B[0], q0);
  sig[1]      = fma(Gr5, B[1], q0);
  sig[2]      = fma(Gr5, B[2], q0);
  sig[3]      = Gr5 * B[3];
  sig[4]      = Gr5 * B[4];
  sig[5]      = Gr5 * B[5];
}

// The neo-Hookean stress from H alone; also returns cof(F) and J = det F.
template <typename T>
__device__ __forceinline__ void neohookean(const T H[3][3], T K, T G, T sig[6], T C[3][3], T& J)
{
  T F[3][3];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int k = 0; k < 3; k++) F[i][k] = (i == k) ? T(1) + H[i][k] : H[i][k];
  J = cofactor3<T>(F, C);
  neohookean_stress<T>(H, J, K, G, sig);
}

// Small-strain elastic stress (ElasticMaterial::GetStress,
// src/nimble_material.cc:98-126): eps = sym(F) - I on the unrotated F,
// sigma = 2 mu eps + lambda tr(eps) I with lambda = K - 2 mu / 3.  From
// H = F - I the strain is sym(H), without the cancellation of F_ii - 1.
template <typename T>
__device__ __forceinline__ void elastic_stress(const T H[3][3], T K, T G, T sig[6])
{
  const T two_mu = T(2) * G, lambda = K - T(2) * G / T(3);
  const T tr     = H[0][0] + H[1][1] + H[2][2];
  sig[0]         = two_mu * H[0][0] + lambda * tr;
  sig[1]         = two_mu * H[1][1] + lambda * tr;
  sig[2]         = two_mu * H[2][2] + lambda * tr;
  sig[3]         = G * (H[0][1] + H[1][0]);
  sig[4]         = G * (H[1][2] + H[2][1]);
  sig[5]         = G * (H[2][0] + H[0][2]);
}

// The elastic stress from H alone; also returns cof(F) and J = det F.
template <typename T>
__device__ __forceinline__ void elastic(const T H[3][3], T K, T G, T sig[6], T C[3][3], T& J)
{
  T F[3][3];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int k = 0; k < 3; k++) F[i][k] = (i == k) ? T(1) + H[i][k] : H[i][k];
  J = cofactor3<T>(F, C);
  elastic_stress<T>(H, K, G, sig);
}

// The stress of the element's material model (also cof(F) and J).
template <typename T>
__device__ __forceinline__ void material_stress(int model, const T H[3][3], T K, T G, T sig[6], T C[3][3], T& J)
{
  if (model == kElastic)
    elastic<T>(H, K, G, sig, C, J);
  else
    neohookean<T>(H, K, G, sig, C, J);
}

// The stress of the element's material model from H and J = det F.
template <typename T>
__device__ __forceinline__ void material_stress_j(int model, const T H[3][3], T J, T K, T G, T sig[6])
{
  if (model == kElastic)
    elastic_stress<T>(H, K, G, sig);
  else
    neohookean_stress<T>(H, J, K, G, sig);
}

template <typename T>
__device__ __forceinline__ T sym(const T s[6], int i, int k)
{
  return s[sym_slot(i, k)];
}

__device__ __forceinline__ double reciprocal(double x) { return 1.0 / x; }
__device__ __forceinline__ float  reciprocal(float x) { return __frcp_rn(x); }

template <typename T>
__device__ __forceinline__ void invert3(const T A[3][3], T inv[3][3], T& det)
{
  T c00 = A[1][1] * A[2][2] - A[1][2] * A[2][1];
  T c01 = A[1][2] * A[2][0] - A[1][0] * A[2][2];
  T c02 = A[1][0] * A[2][1] - A[1][1] * A[2][0];
  det   = A[0][0] * c00 + A[0][1] * c01 + A[0][2] * c02;
  T r   = reciprocal(det);
  inv[0][0] = c00 * r;
  inv[1][0] = c01 * r;
  inv[2][0] = c02 * r;
  inv[0][1] = (A[0][2] * A[2][1] - A[0][1] * A[2][2]) * r;
  inv[1][1] = (A[0][0] * A[2][2] - A[0][2] * A[2][0]) * r;
  inv[2][1] = (A[0][1] * A[2][0] - A[0][0] * A[2][1]) * r;
  inv[0][2] = (A[0][1] * A[1][2] - A[0][2] * A[1][1]) * r;
  inv[1][2] = (A[0][2] * A[1][0] - A[0][0] * A[1][2]) * r;
  inv[2][2] = (A[0][0] * A[1][1] - A[0][1] * A[1][0]) * r;
}

// Strain energy density from H = F - I, without cancellation:
// W = K/4 (J^2 - 1) - K/2 ln J + G/2 (J^{-2/3} tr(F F^T) - 3), whose Cauchy
// stress is the material above (not in the reference; used for the energy
// balance).
__device__ __forceinline__ double energy_density(const double H[3][3], double K, double G)
{
  double trH  = H[0][0] + H[1][1] + H[2][2];
  double trH2 = 0.0, hh = 0.0;
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int k = 0; k < 3; k++) {
      trH2 += H[i][k] * H[k][i];
      hh += H[i][k] * H[i][k];
    }
  double detH = H[0][0] * (H[1][1] * H[2][2] - H[1][2] * H[2][1]) - H[0][1] * (H[1][0] * H[2][2] - H[1][2] * H[2][0]) +
                H[0][2] * (H[1][0] * H[2][1] - H[1][1] * H[2][0]);
  double Jm1   = trH + 0.5 * (trH * trH - trH2) + detH;
  double lnJ   = log1p(Jm1);
  double Jm23  = exp(-2.0 / 3.0 * lnJ);
  double trbm3 = 2.0 * trH + hh;
  double vol   = 0.25 * K * (Jm1 * (Jm1 + 2.0)) - 0.5 * K * lnJ;
  double iso   = 0.5 * G * (3.0 * expm1(-2.0 / 3.0 * lnJ) + Jm23 * trbm3);
  return vol + iso;
}

// Strain energy density of the small-strain elastic material:
// W = mu eps:eps + lambda/2 tr(eps)^2, eps = sym(H), whose stress is elastic().
__device__ __forceinline__ double energy_density_elastic(const double H[3][3], double K, double G)
{
  const double lambda = K - 2.0 * G / 3.0;
  const double tr     = H[0][0] + H[1][1] + H[2][2];
  double       ee     = 0.0;
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int k = 0; k < 3; k++) {
      const double e = 0.5 * (H[i][k] + H[k][i]);
      ee += e * e;
    }
  return G * ee + 0.5 * lambda * tr * tr;
}

}  // namespace nsm
