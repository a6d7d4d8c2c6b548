// Fused hex8 element kernel: gather -> deformation gradient -> neo-Hookean
// Cauchy stress -> B^T sigma, one thread per element, for the FP64 plain form
// and the FP32 mixed form (same code, T = double / float).  The element math
// and the reasons for its form are in hex_math.cuh.
#include "hex_math.cuh"
#include "nsm_kernels.cuh"

namespace nsm {

// Vector stores of a thread's contiguous values (16-byte aligned).
__device__ __forceinline__ void store_vec(float* dst, const float* v, int n)
{
#pragma unroll
  for (int k = 0; k < n; k += 4)
    *reinterpret_cast<float4*>(dst + k) = make_float4(v[k], v[k + 1], v[k + 2], v[k + 3]);
}
__device__ __forceinline__ void store_vec(double* dst, const double* v, int n)
{
#pragma unroll
  for (int k = 0; k < n; k += 2) *reinterpret_cast<double2*>(dst + k) = make_double2(v[k], v[k + 1]);
}

// Warp-cooperative stores.  A thread's point record (64 or 128 B) is
// contiguous, and so are those of the 32 consecutive elements of a warp;
// stored lane by lane, each store instruction would scatter 16-byte pieces a
// record apart, which HBM takes at half the rate of contiguous writes.
// Instead the warp passes its 32 records through a shared-memory tile and
// each instruction writes 512 contiguous bytes.  The tile slots are swizzled
// (4 and 8 chunks per record) so that neither the per-lane writes nor the
// transposed reads conflict on banks.
template <int kChunks>
__device__ __forceinline__ int tile_slot(int row, int c)
{
  if constexpr (kChunks == 4) return row * 4 + (c ^ ((row >> 1) & 3));
  else if constexpr (kChunks == 8) return row * 8 + (c ^ (row & 7));
  else return row * (kChunks + 1) + c;
}
template <int kChunks>
__host__ __device__ constexpr int tile_chunks() { return 32 * (kChunks == 4 || kChunks == 8 ? kChunks : kChunks + 1); }

__device__ __forceinline__ uint4 pack16(const float* v, int c)
{
  return make_uint4(__float_as_uint(v[4 * c]), __float_as_uint(v[4 * c + 1]), __float_as_uint(v[4 * c + 2]),
                    __float_as_uint(v[4 * c + 3]));
}
__device__ __forceinline__ uint4 pack16(const double* v, int c)
{
  const unsigned long long a = __double_as_longlong(v[2 * c]), b = __double_as_longlong(v[2 * c + 1]);
  return make_uint4((unsigned)a, (unsigned)(a >> 32), (unsigned)b, (unsigned)(b >> 32));
}

// dst: the first lane's block; all 32 lanes of the warp take part.
template <int kChunks, typename T>
__device__ __forceinline__ void warp_store(uint4* __restrict__ dst, const T* v, uint4* tile, int lane)
{
  __syncwarp();  // the tile's previous contents have been read
#pragma unroll
  for (int c = 0; c < kChunks; c++) tile[tile_slot<kChunks>(lane, c)] = pack16(v, c);
  __syncwarp();
#pragma unroll
  for (int k = 0; k < kChunks; k++) {
    const int j = k * 32 + lane;
    dst[j]      = tile[tile_slot<kChunks>(j / kChunks, j % kChunks)];
  }
}

// Finiteness without the FP64 pipe: an exponent field of all ones is an
// infinity or a NaN.
__device__ __forceinline__ bool finite_bits(double x) { return (__double2hiint(x) & 0x7ff00000) != 0x7ff00000; }
__device__ __forceinline__ bool finite_bits(float x) { return isfinite(x); }

// J > 0 without the FP64 pipe: the sign and magnitude bits of an IEEE number
// order like a signed integer (a NaN J passes here and is caught as a
// non-finite force).
__device__ __forceinline__ bool positive(double x) { return __double_as_longlong(x) > 0; }
__device__ __forceinline__ bool positive(float x) { return x > 0.0f; }

// Nodal values of the element: FP64 form from the FP64 field, FP32 form from
// the FP32 copy (no FP64 conversions, which would run on the FP64 pipe).
template <typename T>
__device__ __forceinline__ T load_node(const double* f64, const float* f32, long i);
template <>
__device__ __forceinline__ double load_node<double>(const double* f64, const float*, long i) { return __ldg(&f64[i]); }
template <>
__device__ __forceinline__ float load_node<float>(const double*, const float* f32, long i) { return __ldg(&f32[i]); }

// Where an element's nodal values come from.  GlobalNodes: gathered from the
// node planes through the connectivity.  StagedNodes: this thread's slots of a
// shared-memory stage that cp.async filled one element ahead (FP32 form).
template <typename T>
struct GlobalNodes {
  const ElementArgs& a;
  int                id[8];
  __device__ __forceinline__ GlobalNodes(const ElementArgs& args, int e) : a(args)
  {
#pragma unroll
    for (int n = 0; n < 8; n++) id[n] = __ldg(&a.conn[n * a.ld_e + e]);
  }
  __device__ __forceinline__ T u(int n, int k) const { return load_node<T>(a.u, a.uf, k * a.ld_n + id[n]); }
  __device__ __forceinline__ T X(int n, int k) const { return __ldg(&a.Xf[k * a.ld_n + id[n]]); }
};

// Stage layout: [48][blockDim] floats per element slot, values 0..23 u
// (node-major, 3 components), 24..47 X; thread t owns column t, so the lanes of
// a warp read consecutive words.
constexpr int kStageValues = 48;
struct StagedNodes {
  const float* s;  // this thread's column of the stage
  int          B;  // column stride (threads per block)
  __device__ __forceinline__ float u(int n, int k) const { return s[(n * 3 + k) * B]; }
  __device__ __forceinline__ float X(int n, int k) const { return s[(24 + n * 3 + k) * B]; }
};

// FP64 form: reference geometry precomputed (geo planes).  FP32 form: the
// reference Jacobian is rebuilt from X each step with the same transform.
// kPass: 0 the fused step (F, sigma, records, forces); with a block-material
// callback the step is split as the reference's plugin path splits it,
// 1 kinematics (F and the built-in materials' sigma into the records; zero
// sigma where the callback computes it), 2 forces from the recorded sigma.
template <typename T, bool kPrecomputedGeo, class Nodes, int kPass = 0>
__device__ __forceinline__ void element_work(const ElementArgs& a, const int e, const Nodes& nodes);

// One thread per element, or (persistent form) a fixed grid of blocks walking
// the elements of all samples in tiles of blockDim.x.
template <typename T, bool kPrecomputedGeo, bool kPersistent, int kMinBlocks = 1, int kPass = 0>
__global__ void __launch_bounds__(128, kMinBlocks) k_element(ElementArgs a)
{
  if constexpr (!kPersistent) {
    const int e = a.e_begin + blockIdx.x * blockDim.x + threadIdx.x;
    if (e < a.E) element_work<T, kPrecomputedGeo, GlobalNodes<T>, kPass>(a, e, GlobalNodes<T>(a, e));
  } else {
    for (long e = a.e_begin + blockIdx.x * (long)blockDim.x + threadIdx.x; e < a.E;
         e += (long)gridDim.x * blockDim.x)
      element_work<T, kPrecomputedGeo>(a, (int)e, GlobalNodes<T>(a, (int)e));
  }
}

// Staged FP32 form: a persistent grid in which each thread walks the elements
// e, e + stride, ... with the next element's 48 nodal values (u and X) and the
// connectivity of the one after in flight as cp.async copies into its own
// shared-memory columns while it computes the current element.  Neither the
// connectivity load nor the gather it addresses stalls the element math, and
// nothing staged is held in registers.  Copy groups are per thread and each
// thread reads only its own columns: no block barrier is needed.

// Per thread and slot: kStageValues floats (values 0..23 u, 24..47 X), then
// 8 connectivity entries; column stride B.  Two slots, for the element being
// computed and the next one.
constexpr int kStageWords = kStageValues + 8;

__device__ __forceinline__ void stage_conn(const ElementArgs& a, long e, int* col, int B)
{
#pragma unroll
  for (int n = 0; n < 8; n++) cp_async4(col + n * B, a.conn + n * a.ld_e + e);
}

__device__ __forceinline__ void stage_nodes(const ElementArgs& a, const int* conn_col, float* col, int B)
{
#pragma unroll
  for (int n = 0; n < 8; n++) {
    const int id = conn_col[n * B];
#pragma unroll
    for (int k = 0; k < 3; k++) {
      cp_async4(col + (n * 3 + k) * B, a.uf + k * a.ld_n + id);
      cp_async4(col + (24 + n * 3 + k) * B, a.Xf + k * a.ld_n + id);
    }
  }
}

__global__ void __launch_bounds__(128, 3) k_element_staged(ElementArgs a)
{
  extern __shared__ float stage_mem[];  // [2][kStageWords][blockDim.x]
  const int  B      = blockDim.x;
  const long stride = (long)gridDim.x * B;
  const int  slot   = kStageWords * B;
  float*     cur    = stage_mem + threadIdx.x;  // slot of the element being computed
  float*     nxt    = cur + slot;               // slot of the next one
  long       e      = a.e_begin + blockIdx.x * (long)B + threadIdx.x;
  // prologue: connectivity of e (waited for), its nodal values and the
  // connectivity of e + stride in flight
  if (e < a.E) stage_conn(a, e, reinterpret_cast<int*>(cur + kStageValues * B), B);
  cp_async_commit();
  cp_async_wait_all();
  if (e < a.E) stage_nodes(a, reinterpret_cast<const int*>(cur + kStageValues * B), cur, B);
  if (e + stride < a.E) stage_conn(a, e + stride, reinterpret_cast<int*>(nxt + kStageValues * B), B);
  cp_async_commit();
  for (; e < a.E; e += stride) {
    cp_async_wait_all();  // this element's values and the next one's connectivity
    if (e + stride < a.E) stage_nodes(a, reinterpret_cast<const int*>(nxt + kStageValues * B), nxt, B);
    if (e + 2 * stride < a.E) stage_conn(a, e + 2 * stride, reinterpret_cast<int*>(cur + kStageValues * B), B);
    cp_async_commit();
    element_work<float, false>(a, (int)e, StagedNodes{cur, B});
    float* t = cur;
    cur      = nxt;
    nxt      = t;
  }
  cp_async_wait_all();
}

template <typename T, bool kPrecomputedGeo, class Nodes, int kPass>
__device__ __forceinline__ void element_work(const ElementArgs& a, const int e, const Nodes& nodes)
{
  const long ld_e = a.ld_e;

  // displacement gradient at the points (36 distinct values)
  T Gu[3][3][2][2];
  {
    T x[8][3];
#pragma unroll
    for (int n = 0; n < 8; n++)
#pragma unroll
      for (int k = 0; k < 3; k++) x[n][k] = nodes.u(n, k);
    nodal_gradient<T>(x, Gu);
  }
  T GX[3][3][2][2];
  if constexpr (!kPrecomputedGeo) {
    T x[8][3];
#pragma unroll
    for (int n = 0; n < 8; n++)
#pragma unroll
      for (int k = 0; k < 3; k++) x[n][k] = nodes.X(n, k);
    nodal_gradient<T>(x, GX);
  }

  T S[3][3][2][2];  // point sums of Q[d][i] grouped by the other-axis sign pairs
#pragma unroll
  for (int d = 0; d < 3; d++)
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int s = 0; s < 2; s++)
#pragma unroll
        for (int t = 0; t < 2; t++) S[d][i][s][t] = T(0);

  T   K = T(a.bulk), Gm = T(a.shear);
  int model = a.model;
  if (a.elem_group) {
    const GroupMaterial& m = a.mats[__ldg(&a.elem_group[e])];
    K                      = T(m.bulk);
    Gm                     = T(m.shear);
    model                  = m.model;
  }
  bool    bad = false;
  T*      rec = reinterpret_cast<T*>(a.ip) + (size_t)e * kIpRecord;
  const bool store =
      kPass == 1 ||
      (kPass == 0 && (a.store_ip || (a.sched != nullptr && a.sched[(long)(*a.step_base + a.k) * a.num_groups].is_output)));
  // a warp of 32 consecutive elements stores through its tile; a partial warp lane by lane
  constexpr int kRecChunks = kIpRecord * (int)sizeof(T) / 16;
  constexpr int kTile      = tile_chunks<kRecChunks>();
  __shared__ uint4 tiles[4][kTile];  // blocks of at most 128 threads
  const int        lane   = threadIdx.x & 31;
  const long       e0     = (long)e - lane;  // the warp's elements are e0 .. e0 + 31
  const bool       whole  = e0 + 32 <= a.E;
  uint4*           tile   = tiles[(threadIdx.x >> 5) & 3];

#pragma unroll
  for (int p = 0; p < 8; p++) {
    const int bit[3] = {sx_of(p), sy_of(p), sz_of(p)};
    T         G0[3][3], JX[3][3], idet0;  // J_X^{-1} / 8, 8 J_X, 1 / (512 det J_X)
    if (kPrecomputedGeo) {
#pragma unroll
      for (int q = 0; q < 9; q++) {
        G0[q / 3][q % 3] = T(__ldg(&a.geo[(p * kGeoPerPoint + q) * ld_e + e]));
        JX[q / 3][q % 3] = T(__ldg(&a.geo[(p * kGeoPerPoint + 10 + q) * ld_e + e]));
      }
      idet0 = T(__ldg(&a.geo[(p * kGeoPerPoint + 19) * ld_e + e]));
    } else {
      T det0;
#pragma unroll
      for (int i = 0; i < 3; i++)
#pragma unroll
        for (int d = 0; d < 3; d++) JX[i][d] = GX[d][i][bit[other1(d)]][bit[other2(d)]];
      invert3<T>(JX, G0, det0);
      if (!(det0 > T(0))) bad = true;  // (checked once at setup in the FP64 form)
      idet0 = reciprocal(det0);
    }
    // Du[i][d] = 8 du_i/dxi_d;  H = Du G0;  8 J_x = 8 J_X + Du, J_x the current Jacobian
    T Du[3][3], H[3][3], Jx[3][3];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int d = 0; d < 3; d++) {
        Du[i][d] = Gu[d][i][bit[other1(d)]][bit[other2(d)]];
        Jx[i][d] = JX[i][d] + Du[i][d];
      }
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int J = 0; J < 3; J++) H[i][J] = fma(Du[i][0], G0[0][J], fma(Du[i][1], G0[1][J], Du[i][2] * G0[2][J]));
    // det J_x = J det J_X, and the force term det(J_x) J_x^{-1} sigma = adj(J_x) sigma
    T       Cx[3][3];
    const T J = cofactor3<T>(Jx, Cx) * idet0;
    T sig[6];
    if constexpr (kPass == 2) {  // the stress the kinematics pass and the callback recorded
#pragma unroll
      for (int q = 0; q < 6; q++) sig[q] = rec[(size_t)p * ld_e * kIpRecord + 9 + q];
    } else {
      material_stress_j<T>(model, H, J, K, Gm, sig);
    }
    if (!positive(J)) bad = true;  // inverted element
    if (store) {
      T r[kIpRecord];
#pragma unroll
      for (int i = 0; i < 3; i++)
#pragma unroll
        for (int k = 0; k < 3; k++) r[full_slot(i, k)] = (i == k) ? one_plus(H[i][k]) : H[i][k];
#pragma unroll
      for (int q = 0; q < 6; q++) r[9 + q] = sig[q];
      r[15] = T(0);
      if (whole)
        warp_store<kRecChunks>(reinterpret_cast<uint4*>(reinterpret_cast<T*>(a.ip) + ((size_t)p * ld_e + e0) * kIpRecord),
                               r, tile, lane);
      else
        store_vec(rec + (size_t)p * ld_e * kIpRecord, r, kIpRecord);
    }
    // Q[d][i] = sum_k adj(J_x)[d][k] sigma[k][i] = sum_k cof(J_x)[k][d] sigma[k][i],
    // summed over the two points of each sign pair (the first assigns)
    if constexpr (kPass != 1) {
#pragma unroll
      for (int d = 0; d < 3; d++)
#pragma unroll
        for (int i = 0; i < 3; i++) {
          T&      acc  = S[d][i][bit[other1(d)]][bit[other2(d)]];
          const T tail = first_of_pair(d, p) ? Cx[2][d] * sym(sig, 2, i) : fma(Cx[2][d], sym(sig, 2, i), acc);
          acc          = fma(Cx[0][d], sym(sig, 0, i), fma(Cx[1][d], sym(sig, 1, i), tail));
        }
    }
  }
  if constexpr (kPass == 1) {  // kinematics only: the records are written
    if (bad) atomicOr(a.status, NSM_STATUS_BAD_JACOBIAN);
    return;
  }

  // f_a,i = - sum_p sum_d dN_a/dxi_d(p) Q_p[d][i].  J_x and hence Q carry
  // the factor 8^2 of the modal gradient, dN/dxi another 8: scale -1/512.
  T f[8][3];
  nodal_adjoint<T>(S, T(-1.0 / 512.0), f);
  T    fv[24];
  bool finite = true;
#pragma unroll
  for (int n = 0; n < 8; n++)
#pragma unroll
    for (int i = 0; i < 3; i++) {
      fv[n * 3 + i] = f[n][i];
      finite        = finite & finite_bits(f[n][i]);
    }
  // corner-major planes fe[(3 c + i) ld_e + e]: each store instruction writes
  // 32 consecutive elements of one plane, and the node kernel's gather of a
  // row of nodes reads 32 consecutive elements of one plane
  T* fe = reinterpret_cast<T*>(a.fe) + e;
#pragma unroll
  for (int q = 0; q < 24; q++) fe[(size_t)q * ld_e] = fv[q];
  if (bad || !finite) atomicOr(a.status, (bad ? NSM_STATUS_BAD_JACOBIAN : 0) | (finite ? 0 : NSM_STATUS_NONFINITE));
}

// Point records before the first evaluation: F = I, sigma = 0, as the
// reference initialises its element data.
template <typename T>
__global__ void k_ip_identity(int E, long ld_e, T* __restrict__ ip)
{
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= E) return;
  for (int p = 0; p < 8; p++) {
    T* rec = ip + ((size_t)p * ld_e + e) * kIpRecord;
#pragma unroll
    for (int i = 0; i < 3; i++) rec[full_slot(i, i)] = T(1);
  }
}

cudaError_t launch_ip_identity(int E, long ld_e, void* ip, int ip_is_float, cudaStream_t stream)
{
  if (E == 0) return cudaSuccess;
  if (ip_is_float)
    k_ip_identity<float><<<grid_for(E, 128), 128, 0, stream>>>(E, ld_e, (float*)ip);
  else
    k_ip_identity<double><<<grid_for(E, 128), 128, 0, stream>>>(E, ld_e, (double*)ip);
  return cudaGetLastError();
}

int num_sms()
{
  static int n = 0;
  if (n == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (n <= 0) n = 1;
  }
  return n;
}

template <typename T, bool kGeo>
static cudaError_t launch_element(ElementArgs a, const ElementLaunch& l, cudaStream_t stream)
{
  if (a.E <= a.e_begin) return cudaSuccess;
  const int block = (l.block == 64 || l.block == 128) ? l.block : 128;
  a.persistent    = l.persistent;
  int grid        = grid_for(a.E - a.e_begin, block);
  if (l.persistent) {
    int g = l.blocks_per_sm * num_sms();
    if (g < grid) grid = g;
  }
  // register bound: FP32 for 3 blocks of 128 per SM (measured fastest); FP64
  // none, or 3 blocks
  constexpr int kMin = sizeof(T) == 4 ? 3 : 1;
  if (l.persistent)
    k_element<T, kGeo, true, kMin><<<grid, block, 0, stream>>>(a);
  else if (l.blocks_per_sm == 3 && block == 128)
    k_element<T, kGeo, false, 3><<<grid, block, 0, stream>>>(a);
  else
    k_element<T, kGeo, false, kMin><<<grid, block, 0, stream>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_element_fp64(const ElementArgs& a, const ElementLaunch& l, cudaStream_t stream)
{
  return launch_element<double, true>(a, l, stream);
}

cudaError_t launch_element_pass(const ElementArgs& a, int is_float, int pass, cudaStream_t stream)
{
  if (a.E <= a.e_begin) return cudaSuccess;
  const int grid = grid_for(a.E - a.e_begin, 128);
  if (pass != 1 && pass != 2) return cudaErrorInvalidValue;
  if (is_float) {
    if (pass == 1)
      k_element<float, false, false, 3, 1><<<grid, 128, 0, stream>>>(a);
    else
      k_element<float, false, false, 3, 2><<<grid, 128, 0, stream>>>(a);
  } else {
    if (pass == 1)
      k_element<double, true, false, 1, 1><<<grid, 128, 0, stream>>>(a);
    else
      k_element<double, true, false, 1, 2><<<grid, 128, 0, stream>>>(a);
  }
  return cudaGetLastError();
}

cudaError_t launch_element_fp32(const ElementArgs& a, const ElementLaunch& l, cudaStream_t stream)
{
  if (!l.staged) return launch_element<float, false>(a, l, stream);
  if (a.E <= a.e_begin) return cudaSuccess;
  const int    block = (l.block == 64 || l.block == 128) ? l.block : 128;
  const size_t smem  = 2 * kStageWords * block * sizeof(float);
  static bool  configured = false;
  if (!configured) {  // 56 KB at 128 threads: above the default 48 KB of dynamic shared memory
    const int   most = 2 * kStageWords * 128 * (int)sizeof(float);
    cudaError_t err  = cudaSuccess;
    err = cudaFuncSetAttribute(k_element_staged, cudaFuncAttributeMaxDynamicSharedMemorySize, most);
    if (err == cudaSuccess)
      err = cudaFuncSetAttribute(k_element_staged, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    if (err != cudaSuccess) return err;
    configured = true;
  }
  ElementArgs  b     = a;
  b.persistent       = 1;
  int grid           = grid_for(a.E - a.e_begin, block);
  const int g        = (l.blocks_per_sm > 0 ? l.blocks_per_sm : 1) * num_sms();
  if (g < grid) grid = g;
  k_element_staged<<<grid, block, smem, stream>>>(b);
  return cudaGetLastError();
}

// Energies of the current state, FP64 whatever the element precision:
// kinetic 1/2 m v.v per node and internal det J_X W(F) per point, with H
// rebuilt from u (so an FP32 F store does not limit the energy's accuracy).
// Per-block partial sums in a fixed order, then one block: deterministic.
__global__ void __launch_bounds__(128) k_energy_partials(int N, long ld_n, const double* __restrict__ mass,
                                                         const double* __restrict__ v, int E, long ld_e,
                                                         const int* __restrict__ conn, const double* __restrict__ u,
                                                         const double* __restrict__ geo,
                                                         const int* __restrict__ elem_group,
                                                         const GroupMaterial* __restrict__ mats,
                                                         double* __restrict__ partial)
{
  __shared__ double s_ke[128], s_ie[128];
  double            ke = 0.0, ie = 0.0;
  for (long n = blockIdx.x * (long)blockDim.x + threadIdx.x; n < N; n += (long)gridDim.x * blockDim.x) {
    double vx = v[n], vy = v[ld_n + n], vz = v[2 * ld_n + n];
    ke += 0.5 * mass[n] * (vx * vx + vy * vy + vz * vz);
  }
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < E; e += (long)gridDim.x * blockDim.x) {
    double x[8][3];
#pragma unroll
    for (int c = 0; c < 8; c++) {
      int id = conn[c * ld_e + e];
#pragma unroll
      for (int k = 0; k < 3; k++) x[c][k] = u[k * ld_n + id];
    }
    double Gu[3][3][2][2];
    nodal_gradient<double>(x, Gu);
    const GroupMaterial& mat = mats[elem_group ? elem_group[e] : 0];
    const double         K = mat.bulk, Gm = mat.shear;
    const bool           elastic_model = mat.model == kElastic;
#pragma unroll 1
    for (int p = 0; p < 8; p++) {
      const int bit[3] = {sx_of(p), sy_of(p), sz_of(p)};
      double    G0[3][3];
      for (int q = 0; q < 9; q++) G0[q / 3][q % 3] = geo[(p * kGeoPerPoint + q) * ld_e + e];
      double H[3][3];
      for (int i = 0; i < 3; i++)
        for (int J = 0; J < 3; J++) {
          double h = 0.0;
          for (int d = 0; d < 3; d++) {
            const int o1 = other1(d), o2 = other2(d);
            h += Gu[d][i][bit[o1]][bit[o2]] * G0[d][J];
          }
          H[i][J] = h;
        }
      // (a block whose stress a callback computes has no energy density here)
      if (mat.model != kExternal)
        ie += geo[(p * kGeoPerPoint + 9) * ld_e + e] *
              (elastic_model ? energy_density_elastic(H, K, Gm) : energy_density(H, K, Gm));
    }
  }
  s_ke[threadIdx.x] = ke;
  s_ie[threadIdx.x] = ie;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      s_ke[threadIdx.x] += s_ke[threadIdx.x + w];
      s_ie[threadIdx.x] += s_ie[threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    partial[2 * blockIdx.x]     = s_ke[0];
    partial[2 * blockIdx.x + 1] = s_ie[0];
  }
}

__global__ void k_energy_final(int nblocks, const double* __restrict__ partial, double* __restrict__ out)
{
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double ke = 0.0, ie = 0.0;
  for (int b = 0; b < nblocks; b++) {
    ke += partial[2 * b];
    ie += partial[2 * b + 1];
  }
  out[0] = ke;
  out[1] = ie;
}

cudaError_t launch_energies(int N, long ld_n, const double* mass, const double* v, int E, long ld_e,
                            const int* conn, const double* u, const double* geo, const int* elem_group,
                            const GroupMaterial* mats, double* partial, double* out, cudaStream_t stream)
{
  const int blocks = kEnergyBlocks;
  k_energy_partials<<<blocks, 128, 0, stream>>>(N, ld_n, mass, v, E, ld_e, conn, u, geo, elem_group, mats, partial);
  k_energy_final<<<1, 32, 0, stream>>>(blocks, partial, out);
  return cudaGetLastError();
}

// Per-point records ip[(p*ld_e + e)*16 + slot] -> reference layout
// dst[(e*8 + p)*comps + c] in doubles (F: slots 0..8, sigma: slots 9..14).
template <typename T>
__global__ void k_ip_to_aos(int E, long ld_e, const T* __restrict__ ip, int which, double* __restrict__ dst)
{
  const int comps = which == 0 ? 9 : 6, first = which == 0 ? 0 : 9;
  long      i     = blockIdx.x * (long)blockDim.x + threadIdx.x;
  long      total = (long)E * 8 * comps;
  if (i >= total) return;
  int  c = (int)(i % comps);
  long r = i / comps;
  int  p = (int)(r % 8);
  long e = r / 8;
  dst[i] = (double)ip[((size_t)p * ld_e + e) * kIpRecord + first + c];
}

cudaError_t launch_ip_to_aos(int E, long ld_e, const void* ip, int src_is_float, int which, double* dst,
                             cudaStream_t stream)
{
  long total = (long)E * 8 * (which == 0 ? 9 : 6);
  if (total == 0) return cudaSuccess;
  if (src_is_float)
    k_ip_to_aos<float><<<grid_for(total, 256), 256, 0, stream>>>(E, ld_e, (const float*)ip, which, dst);
  else
    k_ip_to_aos<double><<<grid_for(total, 256), 256, 0, stream>>>(E, ld_e, (const double*)ip, which, dst);
  return cudaGetLastError();
}

// Per-sample max |x| over listed nodes; values are non-negative doubles, so
// their bit patterns order like 64-bit integers and atomicMax on the bits is
// an exact, order-independent maximum.
__global__ void k_group_max_abs(int count, const int* __restrict__ nodes, const double* __restrict__ field, long ld_n,
                                int component, const int* __restrict__ node_group, unsigned long long* out)
{
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  int    n = nodes[i];
  double v = fabs(field[component * ld_n + n]);
  int    g = node_group ? node_group[n] : 0;
  atomicMax(&out[g], (unsigned long long)__double_as_longlong(v));
}

cudaError_t launch_group_max_abs(int count, const int* nodes, const double* field, long ld_n, int component,
                                 const int* node_group, int num_groups, double* out, cudaStream_t stream)
{
  cudaError_t e = cudaMemsetAsync(out, 0, sizeof(double) * num_groups, stream);
  if (e != cudaSuccess || count == 0) return e;
  k_group_max_abs<<<grid_for(count, 256), 256, 0, stream>>>(count, nodes, field, ld_n, component, node_group,
                                                            reinterpret_cast<unsigned long long*>(out));
  return cudaGetLastError();
}

__global__ void k_to_float(long n, const double* __restrict__ src, float* __restrict__ dst)
{
  long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i < n) dst[i] = (float)src[i];
}

cudaError_t launch_to_float(long n, const double* src, float* dst, cudaStream_t stream)
{
  if (n == 0) return cudaSuccess;
  k_to_float<<<grid_for(n, 256), 256, 0, stream>>>(n, src, dst);
  return cudaGetLastError();
}

__global__ void k_node_soa_to_aos(int N, long ld_n, const double* __restrict__ src, double* __restrict__ dst)
{
  long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= 3L * N) return;
  dst[i] = src[(i % 3) * ld_n + i / 3];
}

__global__ void k_node_aos_to_soa(int N, long ld_n, const double* __restrict__ src, double* __restrict__ dst,
                                  float* __restrict__ dstf)
{
  long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= 3L * N) return;
  const double x = src[i];
  dst[(i % 3) * ld_n + i / 3] = x;
  if (dstf) dstf[(i % 3) * ld_n + i / 3] = (float)x;
}

cudaError_t launch_node_soa_to_aos(int N, long ld_n, const double* src, double* dst, cudaStream_t stream)
{
  if (N == 0) return cudaSuccess;
  k_node_soa_to_aos<<<grid_for(3L * N, 256), 256, 0, stream>>>(N, ld_n, src, dst);
  return cudaGetLastError();
}

cudaError_t launch_node_aos_to_soa(int N, long ld_n, const double* src, double* dst, float* dstf,
                                   cudaStream_t stream)
{
  if (N == 0) return cudaSuccess;
  k_node_aos_to_soa<<<grid_for(3L * N, 256), 256, 0, stream>>>(N, ld_n, src, dst, dstf);
  return cudaGetLastError();
}

}  // namespace nsm
