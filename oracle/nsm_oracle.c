/* CPU oracle: plain-C restatement of NimbleSM's explicit hex8 / neo-Hookean
 * step.  TEST INFRASTRUCTURE ONLY (see nsm_oracle.h); never linked into the
 * product.  Compiled with -ffp-contract=off and without fast-math so that each
 * expression rounds exactly as the reference's does.
 *
 * Reference files cited below are paths inside the NimbleSM source tree.
 */
#include "nsm_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Natural coordinate of the Gauss points, the literal of
 * src/nimble_element.cc:58 (not exactly 1/sqrt(3)). */
static const double kGaussCoord = 0.577350269189626;

/* Corner signs in the reference corner order (src/nimble_element.cc:113-120);
 * integration point k sits at kCornerSign[k] * kGaussCoord (:60-91). */
static const int kCornerSign[8][3] = {
    {-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1}, {-1, -1, 1}, {1, -1, 1}, {1, 1, 1}, {-1, 1, 1}};

static double g_N[64];    /* [ip][node] */
static double g_dN[192];  /* [ip][node][3] */
static int    g_tables_ready = 0;

/* src/nimble_element.cc:99-171.  Each factor is formed as the reference writes
 * it: c*(1 -/+ r)*(1 -/+ s)*(1 -/+ t) multiplied left to right, with the sign
 * of c carrying the derivative's sign. */
static void
build_tables(void)
{
  if (g_tables_ready) return;
  const double c = 1.0 / 8.0;
  for (int ip = 0; ip < 8; ip++) {
    double r = kCornerSign[ip][0] * kGaussCoord;
    double s = kCornerSign[ip][1] * kGaussCoord;
    double t = kCornerSign[ip][2] * kGaussCoord;
    for (int n = 0; n < 8; n++) {
      double sx = kCornerSign[n][0], sy = kCornerSign[n][1], sz = kCornerSign[n][2];
      g_N[8 * ip + n]          = c * (1.0 + sx * r) * (1.0 + sy * s) * (1.0 + sz * t);
      g_dN[24 * ip + 3 * n]     = (sx * c) * (1.0 + sy * s) * (1.0 + sz * t);
      g_dN[24 * ip + 3 * n + 1] = (sy * c) * (1.0 + sx * r) * (1.0 + sz * t);
      g_dN[24 * ip + 3 * n + 2] = (sz * c) * (1.0 + sx * r) * (1.0 + sy * s);
    }
  }
  g_tables_ready = 1;
}

void
nsm_oracle_shape_tables(double* values, double* derivatives)
{
  build_tables();
  if (values) memcpy(values, g_N, sizeof(g_N));
  if (derivatives) memcpy(derivatives, g_dN, sizeof(g_dN));
}

/* Invert3x3 (src/nimble_utils.h:1229-1268): cofactor inverse, returns det. */
static double
invert3x3(const double m[3][3], double inv[3][3])
{
  double minor0 = m[1][1] * m[2][2] - m[1][2] * m[2][1];
  double minor1 = m[1][0] * m[2][2] - m[1][2] * m[2][0];
  double minor2 = m[1][0] * m[2][1] - m[1][1] * m[2][0];
  double minor3 = m[0][1] * m[2][2] - m[0][2] * m[2][1];
  double minor4 = m[0][0] * m[2][2] - m[2][0] * m[0][2];
  double minor5 = m[0][0] * m[2][1] - m[0][1] * m[2][0];
  double minor6 = m[0][1] * m[1][2] - m[0][2] * m[1][1];
  double minor7 = m[0][0] * m[1][2] - m[0][2] * m[1][0];
  double minor8 = m[0][0] * m[1][1] - m[0][1] * m[1][0];
  double det    = m[0][0] * minor0 - m[0][1] * minor1 + m[0][2] * minor2;
  inv[0][0]     = minor0 / det;
  inv[0][1]     = -1.0 * minor3 / det;
  inv[0][2]     = minor6 / det;
  inv[1][0]     = -1.0 * minor1 / det;
  inv[1][1]     = minor4 / det;
  inv[1][2]     = -1.0 * minor7 / det;
  inv[2][0]     = minor2 / det;
  inv[2][1]     = -1.0 * minor5 / det;
  inv[2][2]     = minor8 / det;
  return det;
}

/* Jacobian sum_j c_j (x) dN_j/dxi at one point, accumulated over the nodes
 * in order (src/nimble_element.h:458-484, :566-583). */
static void
jacobian(const double* c, int ip, double a[3][3])
{
  for (int i = 0; i < 3; i++)
    for (int k = 0; k < 3; k++) a[i][k] = 0.0;
  for (int j = 0; j < 8; j++) {
    const double* d = &g_dN[24 * ip + 3 * j];
    for (int i = 0; i < 3; i++) {
      a[i][0] += c[3 * j + i] * d[0];
      a[i][1] += c[3 * j + i] * d[1];
      a[i][2] += c[3 * j + i] * d[2];
    }
  }
}

/* Full-tensor slots of row i, column k in the reference storage
 * (K_F_* of src/nimble_utils.h:101-109). */
static const int kFullSlot[3][3] = {{0, 3, 8}, {6, 1, 4}, {5, 7, 2}};

void
nsm_oracle_deformation_gradients(const double* X, const double* x, double* F)
{
  build_tables();
  /* src/nimble_element.cc:333-351 forms disp = x - X, then _impl forms
   * cc = X + disp; both roundings are kept. */
  double cc[24];
  for (int i = 0; i < 24; i++) {
    double disp = x[i] - X[i];
    cc[i]       = X[i] + disp;
  }
  for (int ip = 0; ip < 8; ip++) {
    double a[3][3], b[3][3], b_inv[3][3];
    jacobian(cc, ip, a);
    jacobian(X, ip, b);
    invert3x3(b, b_inv);
    for (int j = 0; j < 3; j++)
      for (int k = 0; k < 3; k++)
        F[9 * ip + kFullSlot[j][k]] = a[j][0] * b_inv[0][k] + a[j][1] * b_inv[1][k] + a[j][2] * b_inv[2][k];
  }
}

/* ---- Left stretch by eigen-decomposition (src/nimble_utils.h:523-551,
 *      :194-206, :650-857, :859-908) ---- */

/* Invert_Full33 (src/nimble_utils.h:523-551) on reference-ordered storage. */
static void
invert_full33(const double* m, double* inv)
{
  enum { XX = 0, YY = 1, ZZ = 2, XY = 3, YZ = 4, ZX = 5, YX = 6, ZY = 7, XZ = 8 };
  double minor0 = m[YY] * m[ZZ] - m[YZ] * m[ZY];
  double minor1 = m[YX] * m[ZZ] - m[YZ] * m[ZX];
  double minor2 = m[YX] * m[ZY] - m[YY] * m[ZX];
  double minor3 = m[XY] * m[ZZ] - m[XZ] * m[ZY];
  double minor4 = m[XX] * m[ZZ] - m[ZX] * m[XZ];
  double minor5 = m[XX] * m[ZY] - m[XY] * m[ZX];
  double minor6 = m[XY] * m[YZ] - m[XZ] * m[YY];
  double minor7 = m[XX] * m[YZ] - m[XZ] * m[YX];
  double minor8 = m[XX] * m[YY] - m[XY] * m[YX];
  double det    = m[XX] * minor0 - m[XY] * minor1 + m[XZ] * minor2;
  inv[XX]       = minor0 / det;
  inv[XY]       = -1.0 * minor3 / det;
  inv[XZ]       = minor6 / det;
  inv[YX]       = -1.0 * minor1 / det;
  inv[YY]       = minor4 / det;
  inv[YZ]       = -1.0 * minor7 / det;
  inv[ZX]       = minor2 / det;
  inv[ZY]       = -1.0 * minor5 / det;
  inv[ZZ]       = minor8 / det;
}

/* Rational minimax approximation of cos(acos(x)/3) on [0,1], degree (6,5)
 * (src/nimble_utils.h:650-665).  The coefficients are the reference's table;
 * they must be identical for bitwise parity. */
static double
cos_of_acos_over_3(double x)
{
  const double x2 = x * x;
  const double x4 = x2 * x2;
  return (0.866025403784438713 + 2.12714890259493060 * x +
          ((1.89202064815951569 + 0.739603278343401613 * x) * x2 +
           (0.121973926953064794 + x * (0.00655637626263929360 + 0.0000390884982780803443 * x)) * x4)) /
         (1.0 + 2.26376989330935617 * x +
          ((1.80461009751278976 + 0.603976798217196003 * x) * x2 +
           (0.0783255761115461708 + 0.00268525944538021629 * x) * x4));
}

static double
sign_of(double x, double y)
{
  return x * (double)(1 - 2 * (y < 0));
}

static double
sel(int b, double v1, double v2)
{
  return b ? v1 : v2;
}

/* Eigenvalues/vectors of a symmetric 3x3 (stored xx,yy,zz,xy,yz,zx):
 * trigonometric largest eigenvalue, column-pivoted QR deflation, Wilkinson
 * shift on the 2x2 remainder, and the near-isotropic fallback
 * (src/nimble_utils.h:667-857).  Vectors are not normalised. */
static void
eigen_sym33(const double* t, double ev[3], double v0[3], double v1[3], double v2[3])
{
  double       cxx = t[0], cyy = t[1], czz = t[2];
  const double cxy = t[3], cyz = t[4], czx = t[5];
  const double c1  = (cxx + cyy + czz) / 3.0;
  cxx -= c1;
  cyy -= c1;
  czz -= c1;
  const double cxy_cxy = cxy * cxy, cyz_cyz = cyz * cyz, czx_czx = czx * czx, cxx_cyy = cxx * cyy;
  const double c2             = cxx_cyy + cyy * czz + czz * cxx - cxy_cxy - cyz_cyz - czx_czx;
  const double ThreeOverA     = -3.0 / c2;
  const double sqrtThreeOverA = sqrt(ThreeOverA);
  const double c3             = cxx * cyz_cyz + cyy * czx_czx - 2.0 * cxy * cyz * czx + czz * (cxy_cxy - cxx_cyy);
  const double rr             = -0.5 * c3 * ThreeOverA * sqrtThreeOverA;
  const double arg            = fabs(rr) < 1.0 ? fabs(rr) : 1.0;
  const double cos_thd3       = cos_of_acos_over_3(arg);
  const double two_cos_thd3   = 2.0 * sign_of(cos_thd3, rr);
  double       e2             = two_cos_thd3 / sqrtThreeOverA;

  double crow0[3] = {cxx - e2, cxy, czx};
  double crow1[3] = {cxy, cyy - e2, cyz};
  double crow2[3] = {czx, cyz, czz - e2};

  const double k0 = crow0[0] * crow0[0] + cxy_cxy + czx_czx;
  const double k1 = cxy_cxy + crow1[1] * crow1[1] + cyz_cyz;
  const double k2 = czx_czx + cyz_cyz + crow2[2] * crow2[2];

  const int k0gk1      = k1 <= k0;
  const int k0gk2      = k2 <= k0;
  const int k1gk2      = k2 <= k1;
  const int k0_largest = k0gk1 && k0gk2;
  const int k1_largest = k1gk2 && !k0gk1;
  const int k2_largest = !(k0_largest || k1_largest);

  double k_row1[3], row2[3], row3[3];
  for (int i = 0; i < 3; i++) {
    k_row1[i] = sel(k0_largest, crow0[i], 0.0) + sel(k1_largest, crow1[i], 0.0) + sel(k2_largest, crow2[i], 0.0);
    row2[i]   = sel(k0_largest, crow1[i], crow0[i]);
    row3[i]   = sel(k2_largest, crow1[i], crow2[i]);
  }
  const double ki_ki = 1.0 / (sel(k0_largest, k0, 0.0) + sel(k1_largest, k1, 0.0) + sel(k2_largest, k2, 0.0));
  const double ki_dpr1 = ki_ki * (k_row1[0] * row2[0] + k_row1[1] * row2[1] + k_row1[2] * row2[2]);
  const double ki_dpr2 = ki_ki * (k_row1[0] * row3[0] + k_row1[1] * row3[1] + k_row1[2] * row3[2]);
  for (int i = 0; i < 3; i++) {
    row2[i] -= ki_dpr1 * k_row1[i];
    row3[i] -= ki_dpr2 * k_row1[i];
  }
  const double a0     = row2[0] * row2[0] + row2[1] * row2[1] + row2[2] * row2[2];
  const double a1     = row3[0] * row3[0] + row3[1] * row3[1] + row3[2] * row3[2];
  const int    a0lea1 = a0 <= a1;
  double       a_row2[3];
  for (int i = 0; i < 3; i++) a_row2[i] = sel(a0lea1, row3[i], row2[i]);
  const double ai_ai = 1.0 / sel(a0lea1, a1, a0);

  v2[0] = k_row1[1] * a_row2[2] - k_row1[2] * a_row2[1];
  v2[1] = k_row1[2] * a_row2[0] - k_row1[0] * a_row2[2];
  v2[2] = k_row1[0] * a_row2[1] - k_row1[1] * a_row2[0];

  const double k_atr11 = cxx * k_row1[0] + cxy * k_row1[1] + czx * k_row1[2];
  const double k_atr21 = cxy * k_row1[0] + cyy * k_row1[1] + cyz * k_row1[2];
  const double k_atr31 = czx * k_row1[0] + cyz * k_row1[1] + czz * k_row1[2];
  const double a_atr12 = cxx * a_row2[0] + cxy * a_row2[1] + czx * a_row2[2];
  const double a_atr22 = cxy * a_row2[0] + cyy * a_row2[1] + cyz * a_row2[2];
  const double a_atr32 = czx * a_row2[0] + cyz * a_row2[1] + czz * a_row2[2];

  double       rm2xx       = (k_row1[0] * k_atr11 + k_row1[1] * k_atr21 + k_row1[2] * k_atr31) * ki_ki;
  const double k_a_rm2xy   = (k_row1[0] * a_atr12 + k_row1[1] * a_atr22 + k_row1[2] * a_atr32);
  double       rm2yy       = (a_row2[0] * a_atr12 + a_row2[1] * a_atr22 + a_row2[2] * a_atr32) * ai_ai;
  const double rm2xy_rm2xy = k_a_rm2xy * k_a_rm2xy * ai_ai * ki_ki;

  const double b        = 0.5 * (rm2xx - rm2yy);
  const double sqrtTerm = sign_of(sqrt(b * b + rm2xy_rm2xy), b);
  double       e0       = rm2yy + b - sqrtTerm;
  double       e1       = rm2xx + rm2yy - e0;
  rm2xx -= e0;
  rm2yy -= e0;
  const double rm2xx2 = rm2xx * rm2xx;
  const double rm2yy2 = rm2yy * rm2yy;
  const double fac1   = sel(rm2xx2 < rm2yy2, k_a_rm2xy * ai_ai, rm2xx);
  const double fac2   = sel(rm2xx2 < rm2yy2, rm2yy, ki_ki * k_a_rm2xy);
  for (int i = 0; i < 3; i++) v0[i] = fac1 * a_row2[i] - fac2 * k_row1[i];
  const int both_zero = (rm2xx2 == 0.0) && (rm2xy_rm2xy == 0.0);
  for (int i = 0; i < 3; i++) v0[i] = sel(both_zero, a_row2[i], v0[i]);

  v1[0] = v2[1] * v0[2] - v2[2] * v0[1];
  v1[1] = v2[2] * v0[0] - v2[0] * v0[2];
  v1[2] = v2[0] * v0[1] - v2[1] * v0[0];

  e0 += c1;
  e1 += c1;
  e2 += c1;
  const double c2tol        = (c1 * c1) * (-1.0e-30);
  const int    c2lsmall_neg = c2 < c2tol;
  ev[0]                     = sel(c2lsmall_neg, e0, c1);
  ev[1]                     = sel(c2lsmall_neg, e1, c1);
  ev[2]                     = sel(c2lsmall_neg, e2, c1);
  const double id[3][3]     = {{1.0, 0.0, 0.0}, {0.0, 1.0, 0.0}, {0.0, 0.0, 1.0}};
  for (int i = 0; i < 3; i++) {
    v0[i] = sel(c2lsmall_neg, v0[i], id[0][i]);
    v1[i] = sel(c2lsmall_neg, v1[i], id[1][i]);
    v2[i] = sel(c2lsmall_neg, v2[i], id[2][i]);
  }
}

/* Left stretch V of F = V R (Polar_Decomp, src/nimble_utils.h:859-908): the
 * eigenpairs of F^{-T} F^{-1} = V^{-2} give V = sum_k lambda_k^{-1/2} n_k n_k^T / |n_k|^2.
 * The rotation, unused by the stress, is not formed. */
static void
left_stretch(const double* F, double* v)
{
  double Finv[9], s[6];
  invert_full33(F, Finv);
  enum { XX = 0, YY = 1, ZZ = 2, XY = 3, YZ = 4, ZX = 5, YX = 6, ZY = 7, XZ = 8 };
  /* Square_Full33T_Full33: s = Finv^T Finv (src/nimble_utils.h:194-206). */
  s[0] = Finv[XX] * Finv[XX] + Finv[YX] * Finv[YX] + Finv[ZX] * Finv[ZX];
  s[1] = Finv[XY] * Finv[XY] + Finv[YY] * Finv[YY] + Finv[ZY] * Finv[ZY];
  s[2] = Finv[XZ] * Finv[XZ] + Finv[YZ] * Finv[YZ] + Finv[ZZ] * Finv[ZZ];
  s[3] = Finv[XX] * Finv[XY] + Finv[YX] * Finv[YY] + Finv[ZX] * Finv[ZY];
  s[4] = Finv[XY] * Finv[XZ] + Finv[YY] * Finv[YZ] + Finv[ZY] * Finv[ZZ];
  s[5] = Finv[XX] * Finv[XZ] + Finv[YX] * Finv[YZ] + Finv[ZX] * Finv[ZZ];
  double ev[3] = {0.0, 0.0, 0.0}, n0[3] = {0.0, 0.0, 0.0}, n1[3] = {0.0, 0.0, 0.0}, n2[3] = {0.0, 0.0, 0.0};
  eigen_sym33(s, ev, n0, n1, n2);
  for (int k = 0; k < 3; k++) ev[k] = ev[k] < 0.0 ? 0.0 : ev[k];
  const double l0 = n0[0] * n0[0] + n0[1] * n0[1] + n0[2] * n0[2];
  const double l1 = n1[0] * n1[0] + n1[1] * n1[1] + n1[2] * n1[2];
  const double l2 = n2[0] * n2[0] + n2[1] * n2[1] + n2[2] * n2[2];
  const double w0 = 1.0 / (sqrt(ev[0]) * l0);
  const double w1 = 1.0 / (sqrt(ev[1]) * l1);
  const double w2 = 1.0 / (sqrt(ev[2]) * l2);
  static const int pr[6][2] = {{0, 0}, {1, 1}, {2, 2}, {0, 1}, {1, 2}, {2, 0}};
  for (int c = 0; c < 6; c++) {
    int i = pr[c][0], j = pr[c][1];
    v[c]  = w0 * n0[i] * n0[j] + w1 * n1[i] * n1[j] + w2 * n2[i] * n2[j];
  }
}

/* NeohookeanMaterial::GetStress (src/nimble_material.cc:252-310). */
static void
neohookean_point(const double* F, double K, double G, double* sig)
{
  double v[6];
  left_stretch(F, v);
  const double xj = v[0] * v[1] * v[2] + 2.0 * v[3] * v[4] * v[5] - v[0] * v[4] * v[4] - v[1] * v[5] * v[5] -
                    v[2] * v[3] * v[3];
  const double cbrt_xj  = cbrt(xj);
  const double fac      = 1.0 / (cbrt_xj * cbrt_xj);
  const double pressure = 0.5 * K * (xj - 1.0 / xj);
  /* b = V V with V symmetric (xx,yy,zz,xy,yz,zx), summed as written. */
  double bxx = v[0] * v[0] + v[3] * v[3] + v[5] * v[5];
  double byy = v[3] * v[3] + v[1] * v[1] + v[4] * v[4];
  double bzz = v[5] * v[5] + v[4] * v[4] + v[2] * v[2];
  double bxy = v[0] * v[3] + v[3] * v[1] + v[5] * v[4];
  double byz = v[3] * v[5] + v[1] * v[4] + v[4] * v[2];
  double bzx = v[5] * v[0] + v[4] * v[3] + v[2] * v[5];
  bxx *= fac;
  byy *= fac;
  bzz *= fac;
  bxy *= fac;
  byz *= fac;
  bzx *= fac;
  const double trace = bxx + byy + bzz;
  bxx                = bxx - trace / 3.0;
  byy                = byy - trace / 3.0;
  bzz                = bzz - trace / 3.0;
  sig[0]             = pressure + G * bxx / xj;
  sig[1]             = pressure + G * byy / xj;
  sig[2]             = pressure + G * bzz / xj;
  sig[3]             = G * bxy / xj;
  sig[4]             = G * byz / xj;
  sig[5]             = G * bzx / xj;
}

void
nsm_oracle_stress(int n, const double* F, double K, double G, double* sigma)
{
  for (int p = 0; p < n; p++) neohookean_point(&F[9 * p], K, G, &sigma[6 * p]);
}

/* ElasticMaterial::GetStress (src/nimble_material.cc:98-126): the strain is
 * the symmetric part of the unrotated F minus I, in the symmetric slots
 * xx, yy, zz, xy, yz, zx (K_S_*); F in the full-tensor slots
 * xx, yy, zz, xy, yz, zx, yx, zy, xz (K_F_*). */
static void
elastic_point(const double* F, double K, double G, double* sig)
{
  double       strain[6];
  const double two_mu = 2.0 * G;
  const double lambda = K - 2.0 * G / 3.0;
  strain[0]           = F[0] - 1.0;
  strain[1]           = F[1] - 1.0;
  strain[2]           = F[2] - 1.0;
  strain[3]           = 0.5 * (F[3] + F[6]);
  strain[4]           = 0.5 * (F[4] + F[7]);
  strain[5]           = 0.5 * (F[5] + F[8]);
  const double trace  = strain[0] + strain[1] + strain[2];
  sig[0]              = two_mu * strain[0] + lambda * trace;
  sig[1]              = two_mu * strain[1] + lambda * trace;
  sig[2]              = two_mu * strain[2] + lambda * trace;
  sig[3]              = two_mu * strain[3];
  sig[4]              = two_mu * strain[4];
  sig[5]              = two_mu * strain[5];
}

void
nsm_oracle_stress_model(int model, int n, const double* F, double K, double G, double* sigma)
{
  for (int p = 0; p < n; p++) {
    if (model == NSM_ORACLE_ELASTIC)
      elastic_point(&F[9 * p], K, G, &sigma[6 * p]);
    else
      neohookean_point(&F[9 * p], K, G, &sigma[6 * p]);
  }
}

/* The material of element e: its block's (ModelData keeps one Block and one
 * Material per element block, src/nimble_model_data.cc:484-493), or the
 * single material. */
static void
material_of(const nsm_oracle_model* m, int e, int* model, double* density, double* K, double* G)
{
  if (m->num_blocks > 1 && m->elem_block) {
    const int b = m->elem_block[e];
    *model      = m->block_model[b];
    *density    = m->block_density[b];
    *K          = m->block_bulk[b];
    *G          = m->block_shear[b];
  } else {
    *model   = m->material_model;
    *density = m->density;
    *K       = m->bulk_modulus;
    *G       = m->shear_modulus;
  }
}

/* ComputeNodalForces_impl with the current coordinates passed as the
 * "reference" and zero displacement (src/nimble_element.cc:457-472,
 * src/nimble_element.h:540-625). */
void
nsm_oracle_nodal_forces(const double* x, const double* s, double* f)
{
  build_tables();
  double cc[24], force[24];
  for (int i = 0; i < 24; i++) {
    cc[i]    = x[i] + 0.0;
    force[i] = 0.0;
  }
  for (int ip = 0; ip < 8; ip++) {
    double a[3][3], ai[3][3];
    jacobian(cc, ip, a);
    const double  jac_det = invert3x3(a, ai);
    const double* sp      = &s[6 * ip];
    for (int n = 0; n < 8; n++) {
      const double* d  = &g_dN[24 * ip + 3 * n];
      double        g1 = d[0] * ai[0][0] + d[1] * ai[1][0] + d[2] * ai[2][0];
      double        g2 = d[0] * ai[0][1] + d[1] * ai[1][1] + d[2] * ai[2][1];
      double        g3 = d[0] * ai[0][2] + d[1] * ai[1][2] + d[2] * ai[2][2];
      double        f1 = g1 * sp[0] + g2 * sp[3] + g3 * sp[5];
      double        f2 = g1 * sp[3] + g2 * sp[1] + g3 * sp[4];
      double        f3 = g1 * sp[5] + g2 * sp[4] + g3 * sp[2];
      f1 *= jac_det * 1.0;
      f2 *= jac_det * 1.0;
      f3 *= jac_det * 1.0;
      force[3 * n] -= f1;
      force[3 * n + 1] -= f2;
      force[3 * n + 2] -= f3;
    }
  }
  memcpy(f, force, sizeof(force));
}

void
nsm_oracle_element(const double* X, const double* u, double K, double G, double* F, double* sigma, double* f)
{
  double x[24];
  for (int i = 0; i < 24; i++) x[i] = X[i] + u[i];
  nsm_oracle_deformation_gradients(X, x, F);
  nsm_oracle_stress(8, F, K, G, sigma);
  nsm_oracle_nodal_forces(x, sigma, f);
}

static void
gather_element(const nsm_oracle_model* m, int e, const double* field, double* out)
{
  for (int n = 0; n < 8; n++) {
    int id = m->conn[8 * e + n];
    for (int k = 0; k < 3; k++) out[3 * n + k] = field[3 * id + k];
  }
}

/* HexElement::ComputeVolumeAverage (src/nimble_element.cc:262-282) ->
 * ComputeVolumeAverageQuantities_impl (src/nimble_element.h:343-392) for nq
 * point quantities (nq <= 32): the element's coordinates enter as
 * "reference" coordinates plus a zero displacement, the current Jacobian and
 * its determinant come from Invert3x3 at each point, volume = sum det, and
 * each average sums q * w * det with w = 1 before one division by the
 * volume. */
void
nsm_oracle_volume_average(const double* x, int nq, const double* q, double* volume, double* avg)
{
  build_tables();
  double cc[24];
  for (int i = 0; i < 24; i++) cc[i] = x[i] + 0.0;
  double vol = 0.0, acc[32];
  for (int k = 0; k < nq; k++) acc[k] = 0.0;
  for (int ip = 0; ip < 8; ip++) {
    double a[3][3], a_inv[3][3];
    jacobian(cc, ip, a);
    double det = invert3x3(a, a_inv);
    vol += det;
    for (int k = 0; k < nq; k++) acc[k] += q[nq * ip + k] * 1.0 * det;
  }
  for (int k = 0; k < nq; k++) avg[k] = acc[k] / vol;
  *volume = vol;
}

/* Block::ComputeDerivedElementData (src/nimble_block.cc:438-497): current
 * coordinates X + u per element (:477-483), then the volume averages of the
 * element's point stresses and deformation gradients. */
void
nsm_oracle_derived_element_data(const nsm_oracle_model* m, const double* u, const double* sigma, const double* F,
                                double* volume, double* avg_sigma, double* avg_F)
{
  for (int e = 0; e < m->num_elem; e++) {
    double x[24], vol_F;
    for (int n = 0; n < 8; n++) {
      int id = m->conn[8 * e + n];
      for (int k = 0; k < 3; k++) x[3 * n + k] = m->coords[3 * id + k] + u[3 * id + k];
    }
    nsm_oracle_volume_average(x, 6, sigma + 48 * (size_t)e, volume + e, avg_sigma + 6 * (size_t)e);
    nsm_oracle_volume_average(x, 9, F + 72 * (size_t)e, &vol_F, avg_F + 9 * (size_t)e);
  }
}

/* Lumped mass of one element: row sums of the consistent mass
 * (src/nimble_element.h:266-309, src/nimble_element.cc:173-193). */
static void
element_lumped_mass(const double* X, double density, double* mass)
{
  double jac_det[8];
  for (int ip = 0; ip < 8; ip++) {
    double a[3][3], ai[3][3];
    jacobian(X, ip, a);
    jac_det[ip] = invert3x3(a, ai);
  }
  for (int i = 0; i < 8; i++) {
    mass[i] = 0.0;
    for (int j = 0; j < 8; j++) {
      double mij = 0.0;
      for (int ip = 0; ip < 8; ip++) mij += 1.0 * density * g_N[ip * 8 + i] * g_N[ip * 8 + j] * jac_det[ip];
      mass[i] += mij;
    }
  }
}

/* Node -> (element, corner) incidence in increasing element order, so that a
 * node-ordered gather adds element contributions in the reference's serial
 * element order. */
typedef struct {
  int* ptr;
  int* idx; /* 8*e + corner */
} incidence;

static int
build_incidence(const nsm_oracle_model* m, incidence* inc)
{
  inc->ptr = (int*)calloc((size_t)m->num_nodes + 1, sizeof(int));
  inc->idx = (int*)malloc(sizeof(int) * 8 * (size_t)(m->num_elem > 0 ? m->num_elem : 1));
  if (!inc->ptr || !inc->idx) return -1;
  for (long k = 0; k < 8L * m->num_elem; k++) inc->ptr[m->conn[k] + 1]++;
  for (int n = 0; n < m->num_nodes; n++) inc->ptr[n + 1] += inc->ptr[n];
  int* fill = (int*)malloc(sizeof(int) * ((size_t)m->num_nodes + 1));
  if (!fill) return -1;
  memcpy(fill, inc->ptr, sizeof(int) * ((size_t)m->num_nodes + 1));
  for (long k = 0; k < 8L * m->num_elem; k++) inc->idx[fill[m->conn[k]]++] = (int)k;
  free(fill);
  return 0;
}

static void
free_incidence(incidence* inc)
{
  free(inc->ptr);
  free(inc->idx);
}

void
nsm_oracle_lumped_mass(const nsm_oracle_model* m, double* mass)
{
  build_tables();
  for (int n = 0; n < m->num_nodes; n++) mass[n] = 0.0;
  double X[24], me[8];
  for (int e = 0; e < m->num_elem; e++) {
    int    model;
    double rho, K, G;
    material_of(m, e, &model, &rho, &K, &G);
    gather_element(m, e, m->coords, X);
    element_lumped_mass(X, rho, me);
    for (int n = 0; n < 8; n++) mass[m->conn[8 * e + n]] += me[n];
  }
}

/* HexElement::ComputeCharacteristicLength (src/nimble_element.cc:221-260):
 * the smaller of the least node-pair distance and the least bounding-box
 * extent; note the box maxima start at 0, as in the reference. */
static double
characteristic_length(const double* c)
{
  double x_max = 0.0, y_max = 0.0, z_max = 0.0;
  double x_min = DBL_MAX, y_min = DBL_MAX, z_min = DBL_MAX, min_d2 = DBL_MAX;
  for (int n = 0; n < 8; n++) {
    double nx = c[3 * n], ny = c[3 * n + 1], nz = c[3 * n + 2];
    if (nx < x_min) x_min = nx;
    if (nx > x_max) x_max = nx;
    if (ny < y_min) y_min = ny;
    if (ny > y_max) y_max = ny;
    if (nz < z_min) z_min = nz;
    if (nz > z_max) z_max = nz;
    for (int k = n + 1; k < 8; k++) {
      double mx = c[3 * k], my = c[3 * k + 1], mz = c[3 * k + 2];
      double d2 = (nx - mx) * (nx - mx) + (ny - my) * (ny - my) + (nz - mz) * (nz - mz);
      if (d2 < min_d2) min_d2 = d2;
    }
  }
  double len = sqrt(min_d2);
  double box = x_max - x_min;
  if (y_max - y_min < box) box = y_max - y_min;
  if (z_max - z_min < box) box = z_max - z_min;
  if (box < len) len = box;
  return len;
}

/* BlockBase::ComputeCriticalTimeStep (src/nimble_block_base.cc:51-84) per
 * block, the least over the blocks. */
double
nsm_oracle_critical_time_step(const nsm_oracle_model* m)
{
  double dt = DBL_MAX;
  double c[24];
  for (int e = 0; e < m->num_elem; e++) {
    int    model;
    double rho, K, G;
    material_of(m, e, &model, &rho, &K, &G);
    const double sound_speed = sqrt(K / rho);
    gather_element(m, e, m->coords, c);
    for (int i = 0; i < 24; i++) c[i] = c[i] + 0.0; /* X + u with u = 0 at setup */
    double dte = characteristic_length(c) / sound_speed;
    if (dte < dt) dt = dte;
  }
  return dt;
}

/* Strain energy density of the elastic material, W = mu eps:eps +
 * lambda/2 tr(eps)^2 with the strain of elastic_point (not in the
 * reference; its stress is elastic_point's). */
static double
elastic_energy_density(const double* F, double K, double G)
{
  const double lambda = K - 2.0 * G / 3.0;
  const double exx = F[0] - 1.0, eyy = F[1] - 1.0, ezz = F[2] - 1.0;
  const double exy = 0.5 * (F[3] + F[6]), eyz = 0.5 * (F[4] + F[7]), ezx = 0.5 * (F[5] + F[8]);
  const double tr = exx + eyy + ezz;
  return G * (exx * exx + eyy * eyy + ezz * ezz + 2.0 * (exy * exy + eyz * eyz + ezx * ezx)) + 0.5 * lambda * tr * tr;
}

/* Strain energy density, evaluated from H = F - I without cancellation:
 * J-1 from the invariants of H, tr(b)-3 = 2 tr H + |H|^2. */
double
nsm_oracle_energy_density(const double* F, double K, double G)
{
  double H[3][3];
  for (int i = 0; i < 3; i++)
    for (int k = 0; k < 3; k++) H[i][k] = F[kFullSlot[i][k]] - (i == k ? 1.0 : 0.0);
  double trH  = H[0][0] + H[1][1] + H[2][2];
  double trH2 = 0.0, hh = 0.0;
  for (int i = 0; i < 3; i++)
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

static double
now_seconds(void)
{
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

typedef struct {
  const nsm_oracle_model* m;
  incidence               inc;
  double*                 mass;
  double*                 fe;    /* [E][24] element nodal forces */
  double*                 F;     /* [E][72] */
  double*                 sigma; /* [E][48] */
  int                     bad_jacobian;
} work;

static int
work_init(work* w, const nsm_oracle_model* m)
{
  memset(w, 0, sizeof(*w));
  w->m     = m;
  size_t E = (size_t)(m->num_elem > 0 ? m->num_elem : 1);
  w->mass  = (double*)malloc(sizeof(double) * (size_t)m->num_nodes);
  w->fe    = (double*)malloc(sizeof(double) * 24 * E);
  w->F     = (double*)malloc(sizeof(double) * 72 * E);
  w->sigma = (double*)malloc(sizeof(double) * 48 * E);
  if (!w->mass || !w->fe || !w->F || !w->sigma) return -1;
  if (build_incidence(m, &w->inc)) return -1;
  return 0;
}

static void
work_free(work* w)
{
  free(w->mass);
  free(w->fe);
  free(w->F);
  free(w->sigma);
  free_incidence(&w->inc);
}

/* ModelData::ComputeInternalForce (src/nimble_model_data.cc:620-667) ->
 * Block::ComputeInternalForce (src/nimble_block.cc:278-436). */
static void
internal_force(work* w, const double* u, double* f_int, int num_threads)
{
  const nsm_oracle_model* m   = w->m;
  int                     bad = 0;
#pragma omp parallel for num_threads(num_threads) schedule(static) reduction(| : bad)
  for (int e = 0; e < m->num_elem; e++) {
    double X[24], ue[24], x[24];
    gather_element(m, e, m->coords, X);
    gather_element(m, e, u, ue);
    for (int i = 0; i < 24; i++) x[i] = X[i] + ue[i];
    double* F = &w->F[72 * (size_t)e];
    double* s = &w->sigma[48 * (size_t)e];
    int    model;
    double rho, K, G;
    material_of(m, e, &model, &rho, &K, &G);
    nsm_oracle_deformation_gradients(X, x, F);
    nsm_oracle_stress_model(model, 8, F, K, G, s);
    nsm_oracle_nodal_forces(x, s, &w->fe[24 * (size_t)e]);
    for (int ip = 0; ip < 8; ip++) {
      double a[3][3], ai[3][3];
      jacobian(x, ip, a);
      if (!(invert3x3(a, ai) > 0.0)) bad = 1;
    }
  }
  w->bad_jacobian |= bad;
#pragma omp parallel for num_threads(num_threads) schedule(static)
  for (int n = 0; n < m->num_nodes; n++) {
    double f0 = 0.0, f1 = 0.0, f2 = 0.0;
    for (int k = w->inc.ptr[n]; k < w->inc.ptr[n + 1]; k++) {
      const double* src = &w->fe[3 * (size_t)w->inc.idx[k]];
      f0 += src[0];
      f1 += src[1];
      f2 += src[2];
    }
    f_int[3 * n]     = f0;
    f_int[3 * n + 1] = f1;
    f_int[3 * n + 2] = f2;
  }
}

/* BoundaryConditionManager::ApplyInitialConditions / ApplyKinematicBC for the
 * explicit scheme, constant magnitudes
 * (src/nimble_boundary_condition_manager.h:93-217). */
static void
apply_initial(const nsm_oracle_model* m, double* v)
{
  for (int b = 0; b < m->num_bcs; b++) {
    if (m->bc_kind[b] != NSM_ORACLE_INITIAL_VELOCITY) continue;
    for (int k = m->bc_ptr[b]; k < m->bc_ptr[b + 1]; k++) v[3 * m->bc_nodes[k] + m->bc_component[b]] = m->bc_value[b];
  }
}

static void
apply_kinematic(const nsm_oracle_model* m, double t_cur, double t_prev, const double* u, double* v)
{
  double delta_t = t_cur - t_prev;
  for (int b = 0; b < m->num_bcs; b++) {
    int c = m->bc_component[b];
    if (m->bc_kind[b] == NSM_ORACLE_PRESCRIBED_VELOCITY) {
      for (int k = m->bc_ptr[b]; k < m->bc_ptr[b + 1]; k++) v[3 * m->bc_nodes[k] + c] = m->bc_value[b];
    } else if (m->bc_kind[b] == NSM_ORACLE_PRESCRIBED_DISPLACEMENT && delta_t > 0.0) {
      for (int k = m->bc_ptr[b]; k < m->bc_ptr[b + 1]; k++) {
        int n            = m->bc_nodes[k];
        v[3 * n + c] = (m->bc_value[b] - u[3 * n + c]) / delta_t;
      }
    }
  }
}

/* One central-difference step, src/integrators/explicit_time_integrator.cc:196-276. */
static void
step(work* w, double* t_cur, double* t_prev, double dt_user, int is_output_step, double* u, double* v, double* a,
     double* f_int, int num_threads)
{
  const nsm_oracle_model* m = w->m;
  long                    n3 = 3L * m->num_nodes;
  *t_prev                    = *t_cur;
  *t_cur += dt_user;
  const double delta = *t_cur - *t_prev;
  const double half  = 0.5 * delta;
  for (long i = 0; i < n3; i++) v[i] += half * a[i];
  apply_kinematic(m, *t_cur, *t_prev, u, v);
  for (long i = 0; i < n3; i++) u[i] += delta * v[i];
  apply_kinematic(m, *t_cur, *t_prev, u, v);
  internal_force(w, u, f_int, num_threads);
  for (int i = 0; i < m->num_nodes; i++) {
    const double oneOverM = 1.0 / w->mass[i];
    for (int k = 0; k < 3; k++) a[3 * i + k] = oneOverM * (f_int[3 * i + k] + 0.0);
  }
  for (long i = 0; i < n3; i++) v[i] += half * a[i];
  if (is_output_step) apply_kinematic(m, *t_cur, *t_prev, u, v);
}

struct nsm_oracle {
  work    w;
  double* u;
  double* v;
  double* a;
  double* f_int;
  double  dt_crit;
  double  t_cur, t_prev, dt_user;
  int     step, num_steps, output_frequency, num_threads;
};

nsm_oracle*
nsm_oracle_create(const nsm_oracle_model* m, int num_threads)
{
  build_tables();
  nsm_oracle* o = (nsm_oracle*)calloc(1, sizeof(nsm_oracle));
  if (!o) return NULL;
  if (work_init(&o->w, m)) {
    free(o);
    return NULL;
  }
  size_t n3      = 3 * (size_t)m->num_nodes;
  o->u           = (double*)calloc(n3, sizeof(double));
  o->v           = (double*)calloc(n3, sizeof(double));
  o->a           = (double*)calloc(n3, sizeof(double));
  o->f_int       = (double*)calloc(n3, sizeof(double));
  o->num_threads = num_threads < 1 ? 1 : num_threads;
  /* src/integrators/explicit_time_integrator.cc:123-125 */
  nsm_oracle_lumped_mass(m, o->w.mass);
  o->dt_crit = nsm_oracle_critical_time_step(m);
  return o;
}

void
nsm_oracle_destroy(nsm_oracle* o)
{
  if (!o) return;
  free(o->u);
  free(o->v);
  free(o->a);
  free(o->f_int);
  work_free(&o->w);
  free(o);
}

double
nsm_oracle_dt_crit(const nsm_oracle* o)
{
  return o->dt_crit;
}

/* src/integrators/explicit_time_integrator.cc:130-147: time schedule, then
 * ApplyInitialConditions and ApplyKinematicConditions(0,0). */
void
nsm_oracle_begin(nsm_oracle* o, double final_time, int num_steps, int output_frequency, const double* v_init)
{
  const nsm_oracle_model* m  = o->w.m;
  size_t                  n3 = 3 * (size_t)m->num_nodes;
  memset(o->u, 0, n3 * sizeof(double));
  memset(o->v, 0, n3 * sizeof(double));
  memset(o->a, 0, n3 * sizeof(double));
  memset(o->f_int, 0, n3 * sizeof(double));
  o->t_cur = o->t_prev = 0.0;
  o->dt_user           = (final_time - 0.0) / num_steps;
  o->step              = 0;
  o->num_steps         = num_steps;
  o->output_frequency  = output_frequency;
  apply_initial(m, o->v);
  if (v_init) memcpy(o->v, v_init, n3 * sizeof(double));
  apply_kinematic(m, 0.0, 0.0, o->u, o->v);
}

int
nsm_oracle_advance(nsm_oracle* o, int k, double* loop_seconds)
{
  double s0 = now_seconds();
  for (int i = 0; i < k && o->step < o->num_steps; i++, o->step++) {
    int is_output = 0;
    if (o->output_frequency != 0 && (o->step % o->output_frequency == 0 || o->step == o->num_steps - 1))
      is_output = 1;
    step(&o->w, &o->t_cur, &o->t_prev, o->dt_user, is_output, o->u, o->v, o->a, o->f_int, o->num_threads);
  }
  if (loop_seconds) *loop_seconds = now_seconds() - s0;
  return o->w.bad_jacobian ? -1 : 0;
}

double
nsm_oracle_time(const nsm_oracle* o)
{
  return o->t_cur;
}

void
nsm_oracle_get_state(const nsm_oracle* o, double* u, double* v, double* a, double* f_int, double* F, double* sigma,
                     double* mass)
{
  const nsm_oracle_model* m  = o->w.m;
  size_t                  n3 = 3 * (size_t)m->num_nodes;
  if (u) memcpy(u, o->u, n3 * sizeof(double));
  if (v) memcpy(v, o->v, n3 * sizeof(double));
  if (a) memcpy(a, o->a, n3 * sizeof(double));
  if (f_int) memcpy(f_int, o->f_int, n3 * sizeof(double));
  if (F) memcpy(F, o->w.F, 72 * (size_t)m->num_elem * sizeof(double));
  if (sigma) memcpy(sigma, o->w.sigma, 48 * (size_t)m->num_elem * sizeof(double));
  if (mass) memcpy(mass, o->w.mass, (size_t)m->num_nodes * sizeof(double));
}

/* ModelData::ComputeInternalForce (src/nimble_model_data.cc:620-667) of the
 * displacement u alone: f_int [N][3] out; F and sigma of every point are kept
 * in the handle (nsm_oracle_get_state).  0, or -1 on a non-positive Jacobian. */
int
nsm_oracle_internal_force(nsm_oracle* o, const double* u, double* f_int)
{
  o->w.bad_jacobian = 0;
  internal_force(&o->w, u, f_int, o->num_threads);
  return o->w.bad_jacobian ? -1 : 0;
}

void
nsm_oracle_set_state(nsm_oracle* o, const double* u, const double* v, const double* a)
{
  size_t n3 = 3 * (size_t)o->w.m->num_nodes;
  if (u) memcpy(o->u, u, n3 * sizeof(double));
  if (v) memcpy(o->v, v, n3 * sizeof(double));
  if (a) memcpy(o->a, a, n3 * sizeof(double));
}

/* Kinetic energy 1/2 sum m |v|^2 and internal energy sum_e sum_ip det J0 W(F)
 * of the current state (the F of the last internal-force evaluation). */
void
nsm_oracle_energies(const nsm_oracle* o, double* ke, double* ie)
{
  const nsm_oracle_model* m = o->w.m;
  double                  k = 0.0, e_int = 0.0;
  for (int i = 0; i < m->num_nodes; i++) {
    const double* v = &o->v[3 * i];
    k += 0.5 * o->w.mass[i] * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
  }
  if (o->step > 0) {
    for (int e = 0; e < m->num_elem; e++) {
      double X[24];
      int    model;
      double rho, K, G;
      material_of(m, e, &model, &rho, &K, &G);
      gather_element(m, e, m->coords, X);
      for (int ip = 0; ip < 8; ip++) {
        double        b[3][3], bi[3][3];
        const double* Fp = &o->w.F[72 * (size_t)e + 9 * ip];
        jacobian(X, ip, b);
        e_int += invert3x3(b, bi) * (model == NSM_ORACLE_ELASTIC ? elastic_energy_density(Fp, K, G)
                                                                 : nsm_oracle_energy_density(Fp, K, G));
      }
    }
  }
  if (ke) *ke = k;
  if (ie) *ie = e_int;
}

int
nsm_oracle_run(
    const nsm_oracle_model* m,
    double                  final_time,
    int                     num_steps,
    int                     output_frequency,
    const double*           v_init,
    int                     num_threads,
    nsm_oracle_result*      out)
{
  nsm_oracle* o = nsm_oracle_create(m, num_threads);
  if (!o) return -2;
  nsm_oracle_begin(o, final_time, num_steps, output_frequency, v_init);
  double secs = 0.0;
  int    rc   = nsm_oracle_advance(o, num_steps, &secs);
  if (out) {
    nsm_oracle_get_state(o, out->u, out->v, out->a, out->f_int, out->F, out->sigma, out->mass);
    out->dt_crit      = o->dt_crit;
    out->loop_seconds = secs;
    nsm_oracle_energies(o, &out->kinetic_energy, &out->internal_energy);
  }
  nsm_oracle_destroy(o);
  return rc;
}

int
nsm_oracle_continue(
    const nsm_oracle_model* m,
    double                  t0,
    double                  dt,
    int                     num_steps,
    int                     num_threads,
    double*                 u,
    double*                 v,
    double*                 a,
    double*                 loop_seconds)
{
  nsm_oracle* o = nsm_oracle_create(m, num_threads);
  if (!o) return -2;
  nsm_oracle_set_state(o, u, v, a);
  o->t_cur = o->t_prev = t0;
  o->dt_user           = dt;
  o->step              = 0;
  o->num_steps         = num_steps;
  o->output_frequency  = 0;
  int rc               = nsm_oracle_advance(o, num_steps, loop_seconds);
  nsm_oracle_get_state(o, u, v, a, NULL, NULL, NULL, NULL);
  nsm_oracle_destroy(o);
  return rc;
}

/* ---- The reference's UQ mode ----
 * nimble_uq::ModelData (src/uq/nimble_uq_model_data.cc:55-248) with UqModel
 * (src/uq/nimble_uq.cc:270-345) on one mesh: the nominal trajectory, num_exact
 * off-nominal trajectories that evaluate the element forces with their own
 * moduli (nimble_uq::Block::ComputeInternalForce with alternative
 * parameters, src/uq/nimble_uq_block.cc:57-164), and num_approx trajectories
 * whose force is the linear closure of the nominal and exact forces
 * (UqModel::ApplyClosure, src/uq/nimble_uq.cc:327-345).  The explicit
 * integrator drives them through the ModelData hooks it calls every step. */

/* Velocity-type conditions act on every trajectory, displacement-type ones
 * on the nominal only (src/nimble_boundary_condition_manager.h:137-206). */
static void
apply_kinematic_uq(const nsm_oracle_model* m, double t_cur, double t_prev, const double* u, double* v, int ns,
                   double** sv)
{
  double delta_t = t_cur - t_prev;
  for (int b = 0; b < m->num_bcs; b++) {
    int c = m->bc_component[b];
    if (m->bc_kind[b] == NSM_ORACLE_PRESCRIBED_VELOCITY) {
      for (int k = m->bc_ptr[b]; k < m->bc_ptr[b + 1]; k++) {
        v[3 * m->bc_nodes[k] + c] = m->bc_value[b];
        for (int s = 0; s < ns; s++) sv[s][3 * m->bc_nodes[k] + c] = m->bc_value[b];
      }
    } else if (m->bc_kind[b] == NSM_ORACLE_PRESCRIBED_DISPLACEMENT && delta_t > 0.0) {
      for (int k = m->bc_ptr[b]; k < m->bc_ptr[b + 1]; k++) {
        int n        = m->bc_nodes[k];
        v[3 * n + c] = (m->bc_value[b] - u[3 * n + c]) / delta_t;
      }
    }
  }
}

/* ModelData::UpdateWithNewVelocity / UpdateWithNewDisplacement of the UQ
 * trajectories (src/uq/nimble_uq_model_data.cc:218-246). */
static void
uq_velocity(const double* mass, long n3, int ns, double** sf, double** sv, double dt)
{
  for (int s = 0; s < ns; s++)
    for (long i = 0; i < n3; i++) {
      const double mi = mass[i / 3];
      const double a  = (1.0 / mi) * (sf[s][i] + 0.0);
      sv[s][i] += dt * a;
    }
}

int
nsm_oracle_run_uq(
    const nsm_oracle_model* m,
    int                     num_exact,
    const double*           exact_bulk,
    const double*           exact_shear,
    int                     num_approx,
    const double*           coef,
    double                  final_time,
    int                     num_steps,
    int                     output_frequency,
    const double*           v_init,
    int                     num_threads,
    int                     max_outputs,
    double*                 out_u,
    double*                 out_v,
    double*                 out_f,
    double*                 out_su,
    double*                 out_sv,
    double*                 out_sf,
    int*                    out_num_outputs)
{
  build_tables();
  const int  ns = num_exact + num_approx, B = m->num_blocks > 1 ? m->num_blocks : 1;
  const long n3 = 3L * m->num_nodes;
  nsm_oracle* o = nsm_oracle_create(m, num_threads);
  if (!o) return -2;
  nsm_oracle_begin(o, final_time, num_steps, output_frequency, NULL);
  nsm_oracle_model* mk = (nsm_oracle_model*)calloc((size_t)(num_exact > 0 ? num_exact : 1), sizeof(nsm_oracle_model));
  work*             wk = (work*)calloc((size_t)(num_exact > 0 ? num_exact : 1), sizeof(work));
  double**          su = (double**)calloc((size_t)(ns > 0 ? ns : 1), sizeof(double*));
  double**          sv = (double**)calloc((size_t)(ns > 0 ? ns : 1), sizeof(double*));
  double**          sf = (double**)calloc((size_t)(ns > 0 ? ns : 1), sizeof(double*));
  int               rc = 0;
  for (int s = 0; s < ns; s++) {
    su[s] = (double*)calloc((size_t)n3, sizeof(double));
    sv[s] = (double*)calloc((size_t)n3, sizeof(double));
    sf[s] = (double*)calloc((size_t)n3, sizeof(double));
  }
  for (int k = 0; k < num_exact; k++) {
    mk[k] = *m;
    if (m->num_blocks > 1) {
      mk[k].block_bulk  = exact_bulk + (size_t)k * B;
      mk[k].block_shear = exact_shear + (size_t)k * B;
    } else {
      mk[k].bulk_modulus  = exact_bulk[k];
      mk[k].shear_modulus = exact_shear[k];
    }
    if (work_init(&wk[k], &mk[k])) rc = -2;
  }
  if (rc == 0) {
    /* initial conditions of every trajectory */
    for (int s = 0; s < ns; s++) apply_initial(m, sv[s]);
    if (v_init)
      for (int s = 0; s < ns; s++) memcpy(sv[s], v_init, (size_t)n3 * sizeof(double));
    if (v_init) memcpy(o->v, v_init, (size_t)n3 * sizeof(double));
    apply_kinematic_uq(m, 0.0, 0.0, o->u, o->v, ns, sv);
  }
  const double* mass     = o->w.mass;
  int           recorded = 0;
  for (int step_i = 0; rc == 0 && step_i < num_steps; step_i++) {
    int is_output = 0;
    if (output_frequency != 0 && (step_i % output_frequency == 0 || step_i == num_steps - 1)) is_output = 1;
    o->t_prev = o->t_cur;
    o->t_cur += o->dt_user;
    const double delta = o->t_cur - o->t_prev, half = 0.5 * delta;
    for (long i = 0; i < n3; i++) o->v[i] += half * o->a[i];
    uq_velocity(mass, n3, ns, sf, sv, half);
    apply_kinematic_uq(m, o->t_cur, o->t_prev, o->u, o->v, ns, sv);
    for (long i = 0; i < n3; i++) o->u[i] += delta * o->v[i];
    for (int s = 0; s < ns; s++)
      for (long i = 0; i < n3; i++) su[s][i] += delta * sv[s][i];
    apply_kinematic_uq(m, o->t_cur, o->t_prev, o->u, o->v, ns, sv);
    internal_force(&o->w, o->u, o->f_int, o->num_threads);
    for (int k = 0; k < num_exact; k++) internal_force(&wk[k], su[k], sf[k], o->num_threads);
    for (int s = 0; s < num_approx; s++) {
      double*       f = sf[num_exact + s];
      const double* c = coef + (size_t)s * (num_exact + 1);
      for (long i = 0; i < n3; i++) {
        f[i] = o->f_int[i] * c[0];
        for (int k = 0; k < num_exact; k++) f[i] += sf[k][i] * c[k + 1];
      }
    }
    for (int i = 0; i < m->num_nodes; i++) {
      const double oneOverM = 1.0 / mass[i];
      for (int k = 0; k < 3; k++) o->a[3 * i + k] = oneOverM * (o->f_int[3 * i + k] + 0.0);
    }
    for (long i = 0; i < n3; i++) o->v[i] += half * o->a[i];
    uq_velocity(mass, n3, ns, sf, sv, half);
    if (is_output) apply_kinematic_uq(m, o->t_cur, o->t_prev, o->u, o->v, ns, sv);
    if ((is_output || (output_frequency == 0 && step_i == num_steps - 1)) && recorded < max_outputs) {
      const size_t t = (size_t)recorded;
      if (out_u) memcpy(out_u + t * n3, o->u, (size_t)n3 * sizeof(double));
      if (out_v) memcpy(out_v + t * n3, o->v, (size_t)n3 * sizeof(double));
      if (out_f) memcpy(out_f + t * n3, o->f_int, (size_t)n3 * sizeof(double));
      for (int s = 0; s < ns; s++) {
        const size_t base = (t * ns + s) * (size_t)n3;
        if (out_su) memcpy(out_su + base, su[s], (size_t)n3 * sizeof(double));
        if (out_sv) memcpy(out_sv + base, sv[s], (size_t)n3 * sizeof(double));
        if (out_sf) memcpy(out_sf + base, sf[s], (size_t)n3 * sizeof(double));
      }
      recorded++;
    }
  }
  if (o->w.bad_jacobian) rc = -1;
  for (int k = 0; k < num_exact; k++)
    if (wk[k].bad_jacobian) rc = -1;
  if (out_num_outputs) *out_num_outputs = recorded;
  for (int k = 0; k < num_exact; k++) work_free(&wk[k]);
  for (int s = 0; s < ns; s++) {
    free(su[s]);
    free(sv[s]);
    free(sf[s]);
  }
  free(su);
  free(sv);
  free(sf);
  free(wk);
  free(mk);
  nsm_oracle_destroy(o);
  return rc;
}

/* Extended-precision Cauchy stress of the displacement field u at the
 * integration points of the listed elements (long double: at least a 64-bit
 * significand).  The same constitutive law as the reference
 * (src/nimble_material.cc:252-310), evaluated as
 * sigma = K/2 (J - 1/J) I + G J^{-5/3} dev(b) with b - I = H + H^T + H H^T and
 * H = (du/dxi)(dX/dxi)^{-1}, which has no cancellation.  Not a restatement of
 * the reference's arithmetic: it is the accuracy yardstick the reference's and
 * the engine's FP64 stresses are both measured against. */
void
nsm_oracle_stress_exact(const nsm_oracle_model* m, const double* u, int num, const int* elems, double* sigma)
{
  build_tables();
  for (int q = 0; q < num; q++) {
    int         e = elems[q];
    long double X[8][3], U[8][3];
    for (int n = 0; n < 8; n++)
      for (int k = 0; k < 3; k++) {
        X[n][k] = m->coords[3 * m->conn[8 * e + n] + k];
        U[n][k] = u[3 * m->conn[8 * e + n] + k];
      }
    for (int ip = 0; ip < 8; ip++) {
      long double JX[3][3] = {{0}}, Ju[3][3] = {{0}};
      for (int j = 0; j < 8; j++)
        for (int i = 0; i < 3; i++)
          for (int k = 0; k < 3; k++) {
            JX[i][k] += X[j][i] * (long double)g_dN[24 * ip + 3 * j + k];
            Ju[i][k] += U[j][i] * (long double)g_dN[24 * ip + 3 * j + k];
          }
      long double c[3][3];
      c[0][0] = JX[1][1] * JX[2][2] - JX[1][2] * JX[2][1];
      c[0][1] = JX[0][2] * JX[2][1] - JX[0][1] * JX[2][2];
      c[0][2] = JX[0][1] * JX[1][2] - JX[0][2] * JX[1][1];
      c[1][0] = JX[1][2] * JX[2][0] - JX[1][0] * JX[2][2];
      c[1][1] = JX[0][0] * JX[2][2] - JX[0][2] * JX[2][0];
      c[1][2] = JX[0][2] * JX[1][0] - JX[0][0] * JX[1][2];
      c[2][0] = JX[1][0] * JX[2][1] - JX[1][1] * JX[2][0];
      c[2][1] = JX[0][1] * JX[2][0] - JX[0][0] * JX[2][1];
      c[2][2] = JX[0][0] * JX[1][1] - JX[0][1] * JX[1][0];
      long double det = JX[0][0] * c[0][0] + JX[0][1] * c[1][0] + JX[0][2] * c[2][0];
      long double H[3][3];
      for (int i = 0; i < 3; i++)
        for (int J = 0; J < 3; J++) {
          long double h = 0;
          for (int k = 0; k < 3; k++) h += Ju[i][k] * c[k][J] / det;
          H[i][J] = h;
        }
      long double F[3][3];
      for (int i = 0; i < 3; i++)
        for (int k = 0; k < 3; k++) F[i][k] = (i == k ? 1.0L : 0.0L) + H[i][k];
      long double Jd = F[0][0] * (F[1][1] * F[2][2] - F[1][2] * F[2][1]) -
                       F[0][1] * (F[1][0] * F[2][2] - F[1][2] * F[2][0]) +
                       F[0][2] * (F[1][0] * F[2][1] - F[1][1] * F[2][0]);
      long double B[3][3];
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
          long double t = H[i][0] * H[j][0] + H[i][1] * H[j][1] + H[i][2] * H[j][2];
          B[i][j]       = H[i][j] + H[j][i] + t;
        }
      long double r   = 1.0L / cbrtl(Jd);
      long double pr  = 0.5L * (long double)m->bulk_modulus * (Jd - 1.0L / Jd);
      long double mm  = (B[0][0] + B[1][1] + B[2][2]) / 3.0L;
      long double Gr5 = (long double)m->shear_modulus * r * r * r * r * r;
      double*     s   = &sigma[48 * (size_t)q + 6 * ip];
      s[0]            = (double)(pr + Gr5 * (B[0][0] - mm));
      s[1]            = (double)(pr + Gr5 * (B[1][1] - mm));
      s[2]            = (double)(pr + Gr5 * (B[2][2] - mm));
      s[3]            = (double)(Gr5 * B[0][1]);
      s[4]            = (double)(Gr5 * B[1][2]);
      s[5]            = (double)(Gr5 * B[2][0]);
    }
  }
}

