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
//   * Modal (tensor-product) form of the trilinear hex: du/dxi at the 8
//     points takes only 4 distinct values (it does not depend on xi), formed
//     from the Hadamard transform of the corner values; same for eta and
//     zeta.  36 values replace the 72 sums of 8 products per point.  The
//     force assembly is the transpose: signed point sums to modal
//     coefficients, then the inverse transform to the corners.
//   * H = F - I = (du/dxi) J_X^{-1}, with J_X^{-1}, J_X and 1/det J_X
//     precomputed per point at setup; no cancellation in F - I, no per-step
//     inverse.
//   * sigma from b - I = H + H^T + H H^T and J = det J_x / det J_X through the
//     cofactors of the current Jacobian J_x = J_X + du/dxi (no polar
//     decomposition: the reference's V V equals F F^T).
//   * J^{-1/3} from an FP32 seed and one third-order correction, so that
//     1/J = r^3 and J^{-5/3} = r^5 need no division.
//   * Forces from det(J_x) J_x^{-1} sigma = adj(J_x) sigma, the adjugate
//     being the transposed cofactor matrix already formed for J.
#pragma once

#include "nsm_common.cuh"

namespace nsm {

// Weights of the one-axis form (1 +- g) / 8 of the shape-function
// derivatives at the Gauss points; the fused closure kernel evaluates its
// gradient with them.
template <typename T>
struct Weights {
  static constexpr T wp = T(1.0 + kGauss);
  static constexpr T wm = T(1.0 - kGauss);
  static constexpr T c1 = T((1.0 + kGauss) / 8.0);
  static constexpr T c2 = T((1.0 - kGauss) / 8.0);
};

// Modal form of the trilinear hex.  With corner signs s_c = +-1 per axis,
//   x(xi) = 1/8 sum_m A_m prod_{axes k in m} xi_k,   A_m = sum_c x_c prod_{k in m} s_{c,k},
// over the 8 axis subsets m (bit k of m set = axis k in m); A is the
// Hadamard transform of the corner values.  dx/dxi_d at a Gauss point with
// coordinates sigma_1 g, sigma_2 g along the other two axes is then
//   1/8 (A_d + g (sigma_1 A_{d,o1} + sigma_2 A_{d,o2}) + g^2 sigma_1 sigma_2 A_{d,o1,o2}),
// which takes 4 distinct values per direction.  The functions below work
// with 8 x dx/dxi (the 1/8 is a power of two, folded exactly into the stored
// reference geometry: J_X^{-1} / 8, 8 J_X, 1 / (512 det J_X)).
template <typename T>
__device__ __forceinline__ T& mode(T A[2][2][2], int m)
{
  return A[m & 1][(m >> 1) & 1][(m >> 2) & 1];
}

// A_m of component i of x[8][3] for every m but the constant mode: three
// stages of butterflies (23 additions).
template <typename T>
__device__ __forceinline__ void modal_coefficients(const T x[8][3], int i, T A[2][2][2])
{
  T P[2][2][2];  // after the xi stage: P[mx][by][bz]
#pragma unroll
  for (int by = 0; by < 2; by++)
#pragma unroll
    for (int bz = 0; bz < 2; bz++) {
      const T hi = x[corner_of(1, by, bz)][i], lo = x[corner_of(0, by, bz)][i];
      P[0][by][bz] = hi + lo;
      P[1][by][bz] = hi - lo;
    }
  T Q[2][2][2];  // after the eta stage: Q[mx][my][bz]
#pragma unroll
  for (int mx = 0; mx < 2; mx++)
#pragma unroll
    for (int bz = 0; bz < 2; bz++) {
      Q[mx][0][bz] = P[mx][1][bz] + P[mx][0][bz];
      Q[mx][1][bz] = P[mx][1][bz] - P[mx][0][bz];
    }
#pragma unroll
  for (int mx = 0; mx < 2; mx++)
#pragma unroll
    for (int my = 0; my < 2; my++) {
      A[mx][my][0] = (mx | my) ? Q[mx][my][1] + Q[mx][my][0] : T(0);  // the constant mode is not needed
      A[mx][my][1] = Q[mx][my][1] - Q[mx][my][0];
    }
}

// Gradient values of a nodal field x[8][3]: G[d][i][s][t] = 8 dx_i/dxi_d at
// the points whose sign bits along the other axes of d are (s, t).
template <typename T>
__device__ __forceinline__ void nodal_gradient(const T x[8][3], T G[3][3][2][2])
{
  constexpr T g = T(kGauss), g2 = T(kGauss * kGauss);
#pragma unroll
  for (int i = 0; i < 3; i++) {
    T A[2][2][2];
    modal_coefficients<T>(x, i, A);
#pragma unroll
    for (int d = 0; d < 3; d++) {
      const int o1 = other1(d), o2 = other2(d);
      const T   a  = mode(A, 1 << d);
      const T   b1 = mode(A, (1 << d) | (1 << o1)), b2 = mode(A, (1 << d) | (1 << o2));
      const T   c  = mode(A, 7);
      const T   same = fma(g2, c, a), diff = fma(-g2, c, a);  // sigma_1 sigma_2 = +1 / -1
      const T   P = b1 + b2, M = b1 - b2;
      G[d][i][1][1] = fma(g, P, same);
      G[d][i][0][0] = fma(-g, P, same);
      G[d][i][1][0] = fma(g, M, diff);
      G[d][i][0][1] = fma(-g, M, diff);
    }
  }
}

// Transpose of nodal_gradient, times `scale`: f[c][i] = scale sum_d sum_{s,t}
// (8 dN_c/dxi_d)(s, t) S[d][i][s][t].  The point sums are taken to modal
// coefficients B_m (4 signed sums per direction), which one inverse
// Hadamard transform (butterflies) takes to the corners.
template <typename T>
__device__ __forceinline__ void nodal_adjoint(const T S[3][3][2][2], T scale, T f[8][3])
{
  const T k1 = scale * T(kGauss), k2 = scale * T(kGauss * kGauss);
#pragma unroll
  for (int i = 0; i < 3; i++) {
    T T0[3], T1[3], T2[3], T12[3];  // sum S, sum sigma_1 S, sum sigma_2 S, sum sigma_1 sigma_2 S
#pragma unroll
    for (int d = 0; d < 3; d++) {
      const T(&v)[2][2] = S[d][i];
      const T up = v[1][1] + v[0][0], um = v[1][1] - v[0][0];
      const T wp = v[1][0] + v[0][1], wm = v[1][0] - v[0][1];
      T0[d] = up + wp;
      T12[d] = up - wp;
      T1[d] = um + wm;
      T2[d] = um - wm;
    }
    // B_m: direction d contributes to {d} (T0), {d, o1} (T1), {d, o2} (T2)
    // and {x, y, z} (T12); other1/other2 of x are y, z; of y, x, z; of z, x, y.
    T B[2][2][2];
    mode(B, 1) = scale * T0[0];
    mode(B, 2) = scale * T0[1];
    mode(B, 4) = scale * T0[2];
    mode(B, 3) = k1 * (T1[0] + T1[1]);
    mode(B, 5) = k1 * (T2[0] + T1[2]);
    mode(B, 6) = k1 * (T2[1] + T2[2]);
    mode(B, 7) = k2 * (T12[0] + T12[1] + T12[2]);
    // inverse transform: zeta stage (the constant mode is zero), eta, xi
    T R[2][2][2];  // R[mx][my][bz]
#pragma unroll
    for (int mx = 0; mx < 2; mx++)
#pragma unroll
      for (int my = 0; my < 2; my++) {
        if (mx | my) {
          R[mx][my][1] = B[mx][my][0] + B[mx][my][1];
          R[mx][my][0] = B[mx][my][0] - B[mx][my][1];
        } else {
          R[0][0][1] = B[0][0][1];
          R[0][0][0] = -B[0][0][1];
        }
      }
    T U[2][2][2];  // U[mx][by][bz]
#pragma unroll
    for (int mx = 0; mx < 2; mx++)
#pragma unroll
      for (int bz = 0; bz < 2; bz++) {
        U[mx][1][bz] = R[mx][0][bz] + R[mx][1][bz];
        U[mx][0][bz] = R[mx][0][bz] - R[mx][1][bz];
      }
#pragma unroll
    for (int by = 0; by < 2; by++)
#pragma unroll
      for (int bz = 0; bz < 2; bz++) {
        f[corner_of(1, by, bz)][i] = U[0][by][bz] + U[1][by][bz];
        f[corner_of(0, by, bz)][i] = U[0][by][bz] - U[1][by][bz];
      }
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

__device__ __forceinline__ double rcbrt_refined(double J)
{
  // FP32 seed, then y <- y (1 + e/3 + 2e^2/9) with e = 1 - J y^3 (error O(e^3)).
  // J goes to FP32 and the seed back to FP64 by their bits, with integer
  // operations (conversions would take FP64-pipe slots): the exponent is
  // rebased by 1023 - 127 = 896 and J's mantissa truncated to 23 bits, for J
  // in the FP32 normal range (any other J gives a meaningless seed, as the
  // inverted or degenerate element it comes from is flagged).
  const int      hi = __double2hiint(J);
  const unsigned lo = (unsigned)__double2loint(J);
  const unsigned yb = __float_as_uint(rcbrtf(__uint_as_float(((unsigned)(hi - (896 << 20)) << 3) | (lo >> 29))));
  double         y  = __hiloint2double((int)((yb >> 3) + (896u << 20)), (int)(yb << 29));
  double y3 = y * y * y;
  double e  = fma(-J, y3, 1.0);
  double c  = fma(e, 2.0 / 9.0, 1.0 / 3.0);
  return fma(y * e, c, y);
}
// FP32 form: J^{-1/3} = 2^{-log2(J)/3} with the hardware log2/exp2 (about 2 ulp).
__device__ __forceinline__ float rcbrt_refined(float J) { return exp2f(__log2f(J) * (-1.0f / 3.0f)); }

// 1 + h rounded to nearest even, as the FP64 add gives it, with integer
// operations for |h| < 1/2 (normal h; the rest takes the FP64 add).  With h =
// +-m 2^(e-52), m the 53-bit significand and e <= -2: for h > 0 the sum has
// exponent 0 and significand 2^52 + rne(m 2^e); for h < 0 exponent -1 and
// 2^53 - rne(m 2^(e+1)) (2^53 is even, so rounding the subtrahend to even
// rounds the difference to even).  A significand that reaches 2^53 carries
// into the exponent field, which gives exactly 1.0.
__host__ __device__ __forceinline__ unsigned long long rne_shift(unsigned long long m, int k)
{
  // m / 2^k rounded to nearest even, k >= 1 (m < 2^53)
  if (k >= 54) return 0;
  const unsigned long long q = m >> k, r = m & ((1ull << k) - 1), half = 1ull << (k - 1);
  return q + ((r > half || (r == half && (q & 1))) ? 1 : 0);
}
__host__ __device__ __forceinline__ unsigned long long one_plus_bits(unsigned long long hb)
{
  const int                exp = (int)((hb >> 52) & 0x7ff) - 1023;
  const unsigned long long m   = (hb & ((1ull << 52) - 1)) | (1ull << 52);
  if (hb >> 63)  // 1 - |h|: exponent -1
    return (1022ull << 52) + ((1ull << 53) - rne_shift(m, -(exp + 1))) - (1ull << 52);
  return (1023ull << 52) + rne_shift(m, -exp);  // 1 + h: exponent 0
}
__device__ __forceinline__ double one_plus(double h)
{
  const unsigned long long hb = (unsigned long long)__double_as_longlong(h);
  const int                be = (int)((hb >> 52) & 0x7ff);  // biased exponent: |h| < 1/2 and normal is 1..1021
  if (be == 0 || be > 1021) return 1.0 + h;
  return __longlong_as_double((long long)one_plus_bits(hb));
}
__device__ __forceinline__ float one_plus(float h) { return 1.0f + h; }

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
  if (model == kElastic) {
    elastic_stress<T>(H, K, G, sig);
  } else if (model == kExternal) {  // the block's callback writes it
#pragma unroll
    for (int q = 0; q < 6; q++) sig[q] = T(0);
  } else {
    neohookean_stress<T>(H, J, K, G, sig);
  }
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
