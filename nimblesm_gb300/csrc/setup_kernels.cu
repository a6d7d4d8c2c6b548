// One-time setup kernels: per-integration-point reference geometry, lumped
// mass and critical time step.  This translation unit is compiled with
// --fmad=false so that each product and sum rounds exactly as the reference's
// host code does; the lumped mass and the time step then equal the
// reference's bit for bit.
#include "nsm_kernels.cuh"

namespace nsm {

__constant__ double c_dN[8 * 8 * 3];  // [ip][node][xi] shape-function derivatives
__constant__ double c_N[8 * 8];       // [ip][node] shape-function values

// Shape tables at the Gauss points, formed as src/nimble_element.cc:99-171
// writes them: c*(1 -/+ r)*(1 -/+ s)*(1 -/+ t) multiplied left to right.
void shape_tables(double* N, double* dN)
{
  const double c = 1.0 / 8.0;
  for (int ip = 0; ip < 8; ip++) {
    double r = (sx_of(ip) ? 1.0 : -1.0) * kGauss, s = (sy_of(ip) ? 1.0 : -1.0) * kGauss,
           t = (sz_of(ip) ? 1.0 : -1.0) * kGauss;
    for (int n = 0; n < 8; n++) {
      double sx = sx_of(n) ? 1.0 : -1.0, sy = sy_of(n) ? 1.0 : -1.0, sz = sz_of(n) ? 1.0 : -1.0;
      N[8 * ip + n]          = c * (1.0 + sx * r) * (1.0 + sy * s) * (1.0 + sz * t);
      dN[24 * ip + 3 * n]     = (sx * c) * (1.0 + sy * s) * (1.0 + sz * t);
      dN[24 * ip + 3 * n + 1] = (sy * c) * (1.0 + sx * r) * (1.0 + sz * t);
      dN[24 * ip + 3 * n + 2] = (sz * c) * (1.0 + sx * r) * (1.0 + sy * s);
    }
  }
}

cudaError_t upload_shape_tables(cudaStream_t stream)
{
  double N[64], dN[192];
  shape_tables(N, dN);
  cudaError_t e = cudaMemcpyToSymbolAsync(c_N, N, sizeof(N), 0, cudaMemcpyHostToDevice, stream);
  if (e != cudaSuccess) return e;
  return cudaMemcpyToSymbolAsync(c_dN, dN, sizeof(dN), 0, cudaMemcpyHostToDevice, stream);
}

// Invert3x3 (src/nimble_utils.h:1229-1268).
__device__ __forceinline__ double invert3x3(const double m[3][3], double inv[3][3])
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

// Per element: the reference Jacobian J_X = sum_j X_j (x) dN_j/dxi at each
// integration point, accumulated as src/nimble_element.h:458-491 does, its
// inverse, determinant and the determinant's reciprocal (planes
// geo[ip * kGeoPerPoint + q][E], scaled for the modal gradient: q = 0..8
// J_X^{-1} / 8, q = 9 det J_X, q = 10..18 8 J_X, q = 19 1 / (512 det J_X));
// the element's lumped mass
// (src/nimble_element.h:266-309, src/nimble_element.cc:173-193) as planes
// me[c][E]; and the element's stable time step L_e / sqrt(K/rho)
// (src/nimble_block_base.cc:51-84, src/nimble_element.cc:221-260).
__global__ void k_setup_elements(int E, long ld_e, const int* __restrict__ conn, const double* __restrict__ X,
                                 long ld_n, const int* __restrict__ elem_group, const GroupMaterial* __restrict__ mats,
                                 double* __restrict__ geo, double* __restrict__ me, double* __restrict__ dt_elem,
                                 int* __restrict__ status)
{
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= E) return;
  const GroupMaterial mat = mats[elem_group ? elem_group[e] : 0];
  const double density = mat.density, sound_speed = mat.sound_speed;
  double x[8][3];
#pragma unroll
  for (int n = 0; n < 8; n++) {
    int id = conn[n * ld_e + e];
#pragma unroll
    for (int k = 0; k < 3; k++) x[n][k] = X[k * ld_n + id];
  }
  double jdet[8];
  bool   bad = false;
#pragma unroll 1
  for (int ip = 0; ip < 8; ip++) {
    double b[3][3] = {{0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}};
    for (int j = 0; j < 8; j++) {
      const double* d = &c_dN[24 * ip + 3 * j];
      for (int i = 0; i < 3; i++) {
        b[i][0] += x[j][i] * d[0];
        b[i][1] += x[j][i] * d[1];
        b[i][2] += x[j][i] * d[2];
      }
    }
    double bi[3][3];
    double det = invert3x3(b, bi);
    jdet[ip]   = det;
    if (!(det > 0.0)) bad = true;
    // scaled for the modal gradient (8 du/dxi), by powers of two (exact):
    // J_X^{-1} / 8, 8 J_X and 1 / (512 det J_X); det J_X itself unscaled
    for (int k = 0; k < 3; k++)
      for (int J = 0; J < 3; J++) {
        geo[(ip * kGeoPerPoint + k * 3 + J) * ld_e + e]      = bi[k][J] * 0.125;
        geo[(ip * kGeoPerPoint + 10 + k * 3 + J) * ld_e + e] = b[k][J] * 8.0;
      }
    geo[(ip * kGeoPerPoint + 9) * ld_e + e]  = det;
    geo[(ip * kGeoPerPoint + 19) * ld_e + e] = (1.0 / det) * (1.0 / 512.0);
  }
  for (int i = 0; i < 8; i++) {
    double m = 0.0;
    for (int j = 0; j < 8; j++) {
      double mij = 0.0;
      for (int ip = 0; ip < 8; ip++) mij += 1.0 * density * c_N[ip * 8 + i] * c_N[ip * 8 + j] * jdet[ip];
      m += mij;
    }
    me[i * ld_e + e] = m;
  }
  // characteristic length with X + u, u = 0 at setup
  double x_max = 0.0, y_max = 0.0, z_max = 0.0;
  double x_min = 1.7976931348623157e308, y_min = x_min, z_min = x_min, min_d2 = x_min;
  for (int n = 0; n < 8; n++) {
    double nx = x[n][0] + 0.0, ny = x[n][1] + 0.0, nz = x[n][2] + 0.0;
    if (nx < x_min) x_min = nx;
    if (nx > x_max) x_max = nx;
    if (ny < y_min) y_min = ny;
    if (ny > y_max) y_max = ny;
    if (nz < z_min) z_min = nz;
    if (nz > z_max) z_max = nz;
    for (int m = n + 1; m < 8; m++) {
      double mx = x[m][0] + 0.0, my = x[m][1] + 0.0, mz = x[m][2] + 0.0;
      double d2 = (nx - mx) * (nx - mx) + (ny - my) * (ny - my) + (nz - mz) * (nz - mz);
      if (d2 < min_d2) min_d2 = d2;
    }
  }
  double len = sqrt(min_d2);
  double box = x_max - x_min;
  if (y_max - y_min < box) box = y_max - y_min;
  if (z_max - z_min < box) box = z_max - z_min;
  if (box < len) len = box;
  dt_elem[e] = len / sound_speed;
  if (bad) atomicOr(status, NSM_STATUS_BAD_JACOBIAN);
}

// Nodal lumped mass: element contributions summed in increasing element
// order (the reference's serial scatter order, src/nimble_block.cc:139-144),
// and its reciprocal as the reference forms it each step
// (src/integrators/explicit_time_integrator.cc:250-251).
__global__ void k_gather_mass(int N, const int* __restrict__ node_ptr, const int* __restrict__ node_inc,
                              const double* __restrict__ me, long ld_e, double* __restrict__ mass,
                              double* __restrict__ inv_mass)
{
  int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  double m = 0.0;
  for (int k = node_ptr[n]; k < node_ptr[n + 1]; k++) {
    int ec = node_inc[k];  // 8*e + corner
    m += me[(ec & 7) * ld_e + (ec >> 3)];
  }
  mass[n]     = m;
  inv_mass[n] = 1.0 / m;
}

// Minimum over each sample's contiguous element range: one block per sample.
__global__ void k_group_min(const int* __restrict__ elem_off, const double* __restrict__ in, double* __restrict__ out)
{
  __shared__ double s[256];
  const int         g = blockIdx.x;
  double            v = 1.7976931348623157e308;
  for (int i = elem_off[g] + threadIdx.x; i < elem_off[g + 1]; i += blockDim.x) v = fmin(v, in[i]);
  s[threadIdx.x] = v;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) s[threadIdx.x] = fmin(s[threadIdx.x], s[threadIdx.x + w]);
    __syncthreads();
  }
  if (threadIdx.x == 0) out[g] = s[0];
}

// Deterministic minimum of n doubles: per-block minima, then one block.
__global__ void k_min_reduce(long n, const double* __restrict__ in, double* __restrict__ out)
{
  __shared__ double s[256];
  double            v = 1.7976931348623157e308;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    v = fmin(v, in[i]);
  s[threadIdx.x] = v;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) s[threadIdx.x] = fmin(s[threadIdx.x], s[threadIdx.x + w]);
    __syncthreads();
  }
  if (threadIdx.x == 0) out[blockIdx.x] = s[0];
}

// Derived element output (Block::ComputeDerivedElementData,
// src/nimble_block.cc:438-497 -> HexElement::ComputeVolumeAverage,
// src/nimble_element.cc:262-282 and src/nimble_element.h:343-392): the
// current coordinates x = X + u, at each point the current Jacobian
// sum_n (x_n + 0) (x) dN_n/dxi and its determinant (Invert3x3), the element
// volume sum_p det_p and the volume averages sum_p (q_p w_p) det_p / volume,
// w_p = 1, of the stress and the deformation gradient (each component on its
// own, as the reference averages every requested element field).  The operations and their order are the reference's and
// this file is compiled without FMA contraction, so for the same u and
// point stresses the result is the reference's bit for bit.
template <typename TR>
__global__ void k_derived_element(int E, long ld_e, const int* __restrict__ conn, const double* __restrict__ X,
                                  const double* __restrict__ u, long ld_n, const TR* __restrict__ ip,
                                  double* __restrict__ volume, double* __restrict__ avg_sigma,
                                  double* __restrict__ avg_F, int* __restrict__ status)
{
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= E) return;
  double x[8][3];
#pragma unroll
  for (int n = 0; n < 8; n++) {
    int id = conn[n * ld_e + e];
#pragma unroll
    for (int k = 0; k < 3; k++) x[n][k] = X[k * ld_n + id] + u[k * ld_n + id];
  }
  double vol = 0.0, acc[15];  // F slots 0-8, sigma 9-14 (the record's order)
#pragma unroll
  for (int q = 0; q < 15; q++) acc[q] = 0.0;
  bool   bad = false;
#pragma unroll 1
  for (int p = 0; p < 8; p++) {
    double a[3][3] = {{0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}};
    for (int j = 0; j < 8; j++) {
      const double* d  = &c_dN[24 * p + 3 * j];
      const double  c0 = x[j][0] + 0.0, c1 = x[j][1] + 0.0, c2 = x[j][2] + 0.0;
      a[0][0] += c0 * d[0];
      a[0][1] += c0 * d[1];
      a[0][2] += c0 * d[2];
      a[1][0] += c1 * d[0];
      a[1][1] += c1 * d[1];
      a[1][2] += c1 * d[2];
      a[2][0] += c2 * d[0];
      a[2][1] += c2 * d[1];
      a[2][2] += c2 * d[2];
    }
    double    ai[3][3];
    const double det = invert3x3(a, ai);
    if (!(det > 0.0)) bad = true;
    vol += det;
    const TR* rec = ip + ((size_t)p * ld_e + e) * kIpRecord;
#pragma unroll
    for (int q = 0; q < 15; q++) acc[q] += (double)rec[q] * 1.0 * det;
  }
#pragma unroll
  for (int q = 0; q < 6; q++) avg_sigma[6 * (size_t)e + q] = acc[9 + q] / vol;
#pragma unroll
  for (int q = 0; q < 9; q++) avg_F[9 * (size_t)e + q] = acc[q] / vol;
  volume[e] = vol;
  if (bad) atomicOr(status, NSM_STATUS_BAD_JACOBIAN);
}

cudaError_t launch_derived_element(int E, long ld_e, const int* conn, const double* X, const double* u, long ld_n,
                                   const void* ip, int ip_is_float, double* volume, double* avg_sigma, double* avg_F,
                                   int* status, cudaStream_t stream)
{
  if (E == 0) return cudaSuccess;
  if (ip_is_float)
    k_derived_element<float><<<grid_for(E, 128), 128, 0, stream>>>(E, ld_e, conn, X, u, ld_n, (const float*)ip, volume,
                                                                   avg_sigma, avg_F, status);
  else
    k_derived_element<double><<<grid_for(E, 128), 128, 0, stream>>>(E, ld_e, conn, X, u, ld_n, (const double*)ip,
                                                                     volume, avg_sigma, avg_F, status);
  return cudaGetLastError();
}

cudaError_t launch_setup(const SetupArgs& a, cudaStream_t stream)
{
  // (an empty mesh launches only the reductions, whose minimum over no
  // element is the largest double)
  if (a.E > 0)
    k_setup_elements<<<grid_for(a.E, 128), 128, 0, stream>>>(a.E, a.ld_e, a.conn, a.X, a.ld_n, a.elem_group, a.mats,
                                                             a.geo, a.me, a.dt_elem, a.status);
  if (a.N > 0)
    k_gather_mass<<<grid_for(a.N, 256), 256, 0, stream>>>(a.N, a.node_ptr, a.node_inc, a.me, a.ld_e, a.mass,
                                                          a.inv_mass);
  if (a.num_groups == 1) {
    int blocks = grid_for(a.E, 256);
    if (blocks > 1024) blocks = 1024;
    if (blocks < 1) blocks = 1;
    k_min_reduce<<<blocks, 256, 0, stream>>>(a.E, a.dt_elem, a.dt_partial);
    k_min_reduce<<<1, 256, 0, stream>>>(blocks, a.dt_partial, a.dt_out);
  } else {
    k_group_min<<<a.num_groups, 256, 0, stream>>>(a.elem_off, a.dt_elem, a.dt_out);
  }
  return cudaGetLastError();
}

}  // namespace nsm
