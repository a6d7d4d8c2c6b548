// Element kernel with the learned closure as the material update: the FP32
// element work (element_kernels.cu) with the neo-Hookean stress replaced by
// the MLP of mlp_common.cuh, evaluated on the 5th-generation tensor cores
// inside the element kernel.
//
// One thread per integration point.  A CTA of 128 threads holds 16 elements
// x 8 points (thread r = 8 * element + point), so one 128-row tile of points
// per network layer, and accumulator row r (tensor-memory lane r) comes back
// to the thread that owns point r.  A warp holds 4 whole elements, so all
// element-level exchange stays inside the warp:
//   * gather: thread (element, p) loads node p of its element and stages it
//     in shared memory; each thread then reads the element's 8 nodes;
//   * B^T sigma: each thread forms its point's contribution to the 24 nodal
//     forces, and a 3-level butterfly over the element's 8 lanes leaves lane
//     p with the sum for node p (21 shuffles, no shared memory).
// The CTAs are persistent: each loads the operand images once and walks
// chunks of 16 elements.  The three layers use the same 64 tensor-memory
// columns in turn, so up to 8 CTAs fit the 512 columns of an SM.  The biases
// of layers 2 and 3 are written into the accumulator by one extra K = 16 MMA
// before the layer's own (bias_mma), so no thread adds a bias.
// Points outside the training envelope take the plain neo-Hookean stress
// (FP32) and are counted.
#include <cuda_runtime.h>

#include "hex_math.cuh"
#include "mlp_common.cuh"
#include "mlp_element.cuh"
#include "nsm_kernels.cuh"

namespace nsm {
namespace mlp {

using namespace tc;

namespace el {
// A: [128][64] activations; the layer-1 input X [128][32] uses its first
// 8 KB, and the per-warp node staging (4 elements x 8 nodes x 32 B) sits in
// the warp's own X rows (bytes [2048 w, 2048 w + 1024)).
constexpr int A    = 0;
constexpr int W    = A + 128 * kHid * 2;  // W1x, W2, W3x images
constexpr int ONE  = W + kOffW2t;         // [8][16] ones in columns 0-2, read by every 8-row group (SBO 0)
constexpr int B2b  = ONE + 256;           // [64][16]: three-term BF16 split of b2 in columns 0-2
constexpr int B3b  = B2b + 2048;          // [16][16]: of b3 (rows 0-5)
constexpr int SMEM = B3b + 512;
constexpr int kStageWarp = 2048;          // bytes between the warps' staging areas
constexpr uint32_t kCols = 64;
constexpr int kElems = 16;                // elements per chunk
}  // namespace el

// Make this CTA's operand writes visible to the tensor core and order them
// before the MMAs thread 0 is about to issue; false if any thread has
// recorded a timed-out wait (the whole CTA then leaves its loop together).
__device__ __forceinline__ bool publish(const int* err)
{
  fence_proxy_async();
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  return *err == 0;
}

// Each thread waits for the commit itself (no block barrier): a timeout is
// recorded and acted on at the next publish().
__device__ __forceinline__ void wait_commit(uint64_t* mbar, uint32_t& phase, int* err)
{
  if (!mbar_wait(mbar, phase)) atomicOr(err, 1);
  phase ^= 1u;
  fence_after_sync();
}

// acc0: the first K-step accumulates onto what the columns hold (the bias
// written there by bias_mma) instead of overwriting it.
__device__ __forceinline__ void layer(uint32_t d, const uint8_t* a, int Ka, const uint8_t* b, int N, bool acc0 = false)
{
  const uint32_t idesc = idesc_bf16_f32(128, N);
  for (int ks = 0; ks < Ka / 16; ks++)
    mma_bf16(d, smem_desc(smem_addr(a) + ks * 2 * kLBO, kLBO, 16 * Ka), smem_desc(smem_addr(b) + ks * 2 * kLBO, kLBO, 16 * Ka),
             idesc, acc0 || ks > 0);
}

// Term t of the three-term BF16 split of an FP32 value: hi + mid + lo equals
// v to 2^-27 relative, so the tensor core's FP32 sum 1 hi + 1 mid + 1 lo is v.
__device__ __forceinline__ float bias_term(float v, int t)
{
  const float hi = __bfloat162float(__float2bfloat16_rn(v));
  if (t == 0) return hi;
  const float r1  = v - hi;
  const float mid = __bfloat162float(__float2bfloat16_rn(r1));
  return t == 1 ? mid : r1 - mid;
}
// D = ones * bias^T (one K = 16 step, overwriting D): every accumulator row
// starts at the layer's FP32 bias, and the layer's MMAs accumulate onto it.
// The A operand is one [8][16] core-matrix pair with ones in columns 0-2;
// its stride between 8-row groups is 0, so all 128 rows read the same 256
// bytes.  The B operand holds the bias's three-term split in columns 0-2.
__device__ __forceinline__ void bias_mma(uint32_t d, const uint8_t* ones, const uint8_t* bias, int N)
{
  mma_bf16(d, smem_desc(smem_addr(ones), kLBO, 0), smem_desc(smem_addr(bias), kLBO, 256), idesc_bf16_f32(128, N), false);
}
// Hidden-layer epilogue: 64 accumulator columns of this thread's row, read as
// two 32-column halves (two tensor-memory loads per wait) -> act(z) -> BF16
// row r of the [128][64] activation tile, two columns per packed FP32x2
// operation.  (No bias is added here: the next layer's first MMA writes it,
// see bias_mma.)
__device__ __forceinline__ void hidden_epilogue(uint32_t taddr, uint8_t* tile, int r)
{
#pragma unroll
  for (int h = 0; h < 4; h += 2) {
    float z[32];
    tmem_ld16(taddr + 16 * h, z);
    tmem_ld16(taddr + 16 * h + 16, z + 16);
    tmem_wait_ld();
#pragma unroll
    for (int k0 = 0; k0 < 32; k0 += 8) {
      uint32_t w[4];
#pragma unroll
      for (int j = 0; j < 4; j++) w[j] = act_bf16(f2_pack(z[k0 + 2 * j], z[k0 + 2 * j + 1]));
      *reinterpret_cast<uint4*>(tile + kmajor_offset(r, 16 * h + k0, kHid)) = make_uint4(w[0], w[1], w[2], w[3]);
    }
  }
}

// Derivative weights of this thread's point: dN_n/dxi_d at point p is
// sgn_d(n) * w[d][b][c] with (b, c) the corner's sign bits along the two
// other axes: w = (b == s ? 1+g : 1-g) * (c == t ? (1+g)/8 : (1-g)/8),
// (s, t) the point's sign bits along those axes (the 2-point transforms of
// hex_math.cuh, evaluated at one point).
__device__ __forceinline__ void point_weights(int p, float w[3][2][2])
{
  using Wt         = Weights<float>;
  const int bit[3] = {sx_of(p), sy_of(p), sz_of(p)};
#pragma unroll
  for (int d = 0; d < 3; d++) {
    const int s = bit[other1(d)], t = bit[other2(d)];
#pragma unroll
    for (int b = 0; b < 2; b++)
#pragma unroll
      for (int c = 0; c < 2; c++) w[d][b][c] = (b == s ? Wt::wp : Wt::wm) * (c == t ? Wt::c1 : Wt::c2);
  }
}

// dx_i/dxi_d at the point: D[i][d].
__device__ __forceinline__ void point_gradient(const float x[8][3], const float w[3][2][2], float D[3][3])
{
#pragma unroll
  for (int d = 0; d < 3; d++) {
    const int o1 = other1(d), o2 = other2(d);
#pragma unroll
    for (int i = 0; i < 3; i++) {
      float v = 0.0f;
#pragma unroll
      for (int b = 0; b < 2; b++)
#pragma unroll
        for (int c = 0; c < 2; c++)
          v = fmaf(w[d][b][c], x[corner_axes(d, 1, o1, b, o2, c)][i] - x[corner_axes(d, 0, o1, b, o2, c)][i], v);
      D[i][d] = v;
    }
  }
}

// A warp holds 4 consecutive elements x 8 points.  Its 32 point records
// (plane p, elements e..e+3: 256 contiguous bytes per plane) go out through
// the warp's 2 KB slice of the input tile, two planes per store instruction
// (512 bytes in two 256-byte runs), instead of 16-byte pieces a record apart.
// Slot swizzle: conflict-free for the per-lane writes (8 consecutive lanes,
// one chunk) and for the reads (two lanes 8 apart, four chunks each).
__device__ __forceinline__ int rec_slot(int row, int c)
{
  return ((row ^ ((row >> 3) & 1)) << 2) + (c ^ ((row >> 1) & 3));
}

__global__ void __launch_bounds__(128, 6) k_element_mlp(ElementArgs a, MlpElementArgs m)
{
  extern __shared__ __align__(1024) uint8_t sm[];
  __shared__ uint64_t mbar;
  __shared__ uint32_t tslot;
  __shared__ int      err;
  const int           r = threadIdx.x, warp = r >> 5, lane = r & 31;
  const int           p = r & 7, el = r >> 3;
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
    // the layers' BF16 weight images
    const uint4* src = reinterpret_cast<const uint4*>(m.img);
    for (int i = r; i < kOffW2t / 16; i += 128) reinterpret_cast<uint4*>(sm + el::W)[i] = src[i];
    for (int i = r; i < 64 * 16; i += 128) {
      const int n = i / 16, k = i % 16;
      store_bf16(sm + el::B2b, n, k, 16, k < 3 ? bias_term(m.P[ob2 + n], k) : 0.0f);
      if (n < 16) store_bf16(sm + el::B3b, n, k, 16, (k < 3 && n < kOut) ? bias_term(m.P[ob3 + n], k) : 0.0f);
      if (n < 8) store_bf16(sm + el::ONE, n, k, 16, k < 3 ? 1.0f : 0.0f);
    }
  }
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tb    = tslot;
  const uint32_t taddr = tb + ((uint32_t)(warp * 32) << 16);
  uint8_t* const stage = sm + el::A + warp * el::kStageWarp;
  const bool     store = a.store_ip || (a.sched != nullptr && a.sched[(long)(*a.step_base + a.k) * a.num_groups].is_output);
  const float    K = (float)a.bulk, Gm = (float)a.shear;
  float          w[3][2][2];
  point_weights(p, w);
  uint32_t phase     = 0;
  int      fallbacks = 0;
  int      status    = 0;

  // The gather is software-pipelined one chunk ahead: the next chunk's node
  // id is loaded while layer 1 runs and its coordinates while layer 2 runs.
  const long nchunks = (a.E + el::kElems - 1) / el::kElems;
  auto node_of = [&](long c) -> int {
    const long e = c * el::kElems + el;
    return (c < nchunks && e < a.E) ? __ldg(&a.conn[p * ld_e + e]) : -1;
  };
  auto values_of = [&](int id, float4& v) {
    v = id >= 0 ? make_float4(__ldg(&a.uf[id]), __ldg(&a.uf[ld_n + id]), __ldg(&a.uf[2 * ld_n + id]), 0.0f)
                : make_float4(0.0f, 0.0f, 0.0f, 0.0f);  // idle rows: zero displacement
  };
  int    id_next = node_of(blockIdx.x);
  float4 nv;
  values_of(id_next, nv);
  for (long chunk = blockIdx.x; chunk < nchunks; chunk += gridDim.x) {
    const long e     = chunk * el::kElems + el;
    const bool valid = e < a.E;

    // ---- the point's reference geometry (computed when the closure was attached) ----
    float G0[3][3], det0, h[9];
    if (valid) {
      const float4* gp = reinterpret_cast<const float4*>(m.geo + ((size_t)e * 8 + p) * 12);
      const float4  g0 = __ldg(gp), g1 = __ldg(gp + 1), g2 = __ldg(gp + 2);
      G0[0][0] = g0.x, G0[0][1] = g0.y, G0[0][2] = g0.z, G0[1][0] = g0.w;
      G0[1][1] = g1.x, G0[1][2] = g1.y, G0[2][0] = g1.z, G0[2][1] = g1.w;
      G0[2][2] = g2.x, det0 = g2.y;
    } else {  // idle rows: a unit element
#pragma unroll
      for (int q = 0; q < 9; q++) G0[q / 3][q % 3] = q % 4 == 0 ? 1.0f : 0.0f;
      det0 = 1.0f;
    }

    // ---- gather: node p's displacement, staged for the element's 8 lanes ----
    reinterpret_cast<float4*>(stage + (lane >> 3) * 128)[p] = nv;
    __syncwarp();
    float Du[3][3];
    {
      float         xu[8][3];
      const float4* st = reinterpret_cast<const float4*>(stage + (lane >> 3) * 128);
#pragma unroll
      for (int n = 0; n < 8; n++) {
        const float4 v = st[n];
        xu[n][0] = v.x, xu[n][1] = v.y, xu[n][2] = v.z;
      }
      point_gradient(xu, w, Du);
    }
    __syncwarp();  // the staging area is overwritten by this warp's input rows below

#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int J = 0; J < 3; J++) h[3 * i + J] = Du[i][0] * G0[0][J] + Du[i][1] * G0[1][J] + Du[i][2] * G0[2][J];

    // ---- layer 1: input row -> Z1 ----
    {
      float xs[9], row[kInX];
#pragma unroll
      for (int q = 0; q < 9; q++) xs[q] = h[q] * m.sc.in_scale;
      input_row(xs, row);
#pragma unroll
      for (int k0 = 0; k0 < kInX; k0 += 8) store_chunk(sm + el::A, r, k0, kInX, row + k0);
    }
    if (!publish(&err)) break;
    if (r == 0) {
      layer(tb, sm + el::A, kInX, sm + el::W + kOffW1, kHid);
      mma_commit(&mbar);
    }
    id_next = node_of(chunk + gridDim.x);
    wait_commit(&mbar, phase, &err);
    hidden_epilogue(taddr, sm + el::A, r);
    // ---- layer 2 ----
    if (!publish(&err)) break;
    if (r == 0) {
      bias_mma(tb, sm + el::ONE, sm + el::B2b, kHid);
      layer(tb, sm + el::A, kHid, sm + el::W + kOffW2, kHid, true);
      mma_commit(&mbar);
    }
    values_of(id_next, nv);
    wait_commit(&mbar, phase, &err);
    hidden_epilogue(taddr, sm + el::A, r);
    // ---- layer 3 ----
    if (!publish(&err)) break;
    if (r == 0) {
      bias_mma(tb, sm + el::ONE, sm + el::B3b, kOutX);
      layer(tb, sm + el::A, kHid, sm + el::W + kOffW3, kOutX, true);
      mma_commit(&mbar);
    }
    wait_commit(&mbar, phase, &err);
    float sig[6];
    {
      float z[16];
      tmem_ld16(taddr, z);
      tmem_wait_ld();
      if (in_envelope(h, m.sc)) {
        float L[6], xs[9];
#pragma unroll
        for (int q = 0; q < 9; q++) xs[q] = h[q] * m.sc.in_scale;
        base_part(h, m.sc.k_over_g, L);
        const float g = gate(xs) * m.sc.res_scale;
#pragma unroll
        for (int q = 0; q < 6; q++) sig[q] = Gm * fmaf(g, z[q], L[q]);
      } else {
        float H[3][3], C[3][3], J;
#pragma unroll
        for (int q = 0; q < 9; q++) H[q / 3][q % 3] = h[q];
        neohookean<float>(H, K, Gm, sig, C, J);
        fallbacks += valid ? 1 : 0;
      }
    }

    // ---- the point's share of B^T sigma (first Piola-Kirchhoff form) ----
    float F[3][3], C[3][3];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int k = 0; k < 3; k++) F[i][k] = (i == k ? 1.0f : 0.0f) + h[3 * i + k];
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
    if (valid && (!(J > 0.0f) || !(det0 > 0.0f))) status |= NSM_STATUS_BAD_JACOBIAN;
    if (store) {
      const long e_first = chunk * el::kElems + 4 * warp;  // the warp's elements e_first .. e_first + 3
      float      rr[kIpRecord];
#pragma unroll
      for (int i = 0; i < 3; i++)
#pragma unroll
        for (int k = 0; k < 3; k++) rr[full_slot(i, k)] = F[i][k];
#pragma unroll
      for (int q = 0; q < 6; q++) rr[9 + q] = sig[q];
      rr[15] = 0.0f;
      if (e_first + 4 <= a.E) {
        float4* tile = reinterpret_cast<float4*>(stage);  // free until the next chunk's staging
#pragma unroll
        for (int c = 0; c < 4; c++)
          tile[rec_slot(lane, c)] = make_float4(rr[4 * c], rr[4 * c + 1], rr[4 * c + 2], rr[4 * c + 3]);
        __syncwarp();
        float4* ip4 = reinterpret_cast<float4*>(a.ip);
#pragma unroll
        for (int k = 0; k < 4; k++) {
          const int plane = 2 * k + (lane >> 4), j = lane & 15;  // chunk j of the plane's 4 records
          ip4[((size_t)plane * ld_e + e_first) * 4 + j] = tile[rec_slot((j >> 2) * 8 + plane, j & 3)];
        }
        __syncwarp();  // the slice is read before the next chunk's staging
      } else if (valid) {
        float* dst = reinterpret_cast<float*>(a.ip) + ((size_t)p * ld_e + e) * kIpRecord;
#pragma unroll
        for (int k = 0; k < kIpRecord; k += 4)
          *reinterpret_cast<float4*>(dst + k) = make_float4(rr[k], rr[k + 1], rr[k + 2], rr[k + 3]);
      }
    }
    float S[3][3];  // S[d][i] = det0 sum_J G0[d][J] P[i][J],  P = sigma cof(F)
    {
      float P[3][3];
#pragma unroll
      for (int i = 0; i < 3; i++)
#pragma unroll
        for (int Jc = 0; Jc < 3; Jc++)
          P[i][Jc] = sig[sym_slot(i, 0)] * C[0][Jc] + sig[sym_slot(i, 1)] * C[1][Jc] + sig[sym_slot(i, 2)] * C[2][Jc];
#pragma unroll
      for (int d = 0; d < 3; d++)
#pragma unroll
        for (int i = 0; i < 3; i++) S[d][i] = det0 * (G0[d][0] * P[i][0] + G0[d][1] * P[i][1] + G0[d][2] * P[i][2]);
    }
    // Nodal forces in modal form.  dN_n/dxi_d(p) = sgn_d(n) prod_{k != d} (1 + g s_{n,k} t_{p,k}) / 8
    // (s, t the corner's and the point's signs), so f_n = -sum_p sum_d dN_n/dxi_d(p) S_p[d] is the
    // inverse Walsh-Hadamard transform, over the element's 8 lanes, of the modes
    // B_M = -g^(|M|-1)/8 sum_{d in M} A_{d, M\d},  A_{d,M'} = sum_p t_p^M' S_p[d]
    // (S[d] transformed along the two other axes and summed along d).  Lane p holds mode
    // M = {axes where p's sign is +}; lane masks 1, 3, 4 flip the x, y, z sign.
    // (the lane's constants are rebuilt from %laneid here rather than held across the loop)
    uint32_t lid;
    asm volatile("mov.u32 %0, %%laneid;" : "=r"(lid));
    const int   q            = (int)(lid & 7u);
    const int   pb[3]        = {sx_of(q), sy_of(q), sz_of(q)};
    const int   msize        = pb[0] + pb[1] + pb[2];
    const float gk           = msize == 3 ? float(-kGauss * kGauss / 8.0) : (msize == 2 ? float(-kGauss / 8.0) : -0.125f);
    const float mode_sign[3] = {pb[0] ? -1.0f : 1.0f, pb[1] ? -1.0f : 1.0f, pb[2] ? -1.0f : 1.0f};
    const float mode_k[3]    = {pb[0] ? gk : 0.0f, pb[1] ? gk : 0.0f, pb[2] ? gk : 0.0f};
#pragma unroll
    for (int ax = 0; ax < 3; ax++) {
      const int flip = ax == 0 ? 1 : (ax == 1 ? 3 : 4);
#pragma unroll
      for (int d = 0; d < 3; d++)
#pragma unroll
        for (int i = 0; i < 3; i++) {
          const float pv = __shfl_xor_sync(0xffffffffu, S[d][i], flip);
          S[d][i]        = ax == d ? S[d][i] + pv : fmaf(mode_sign[ax], pv, S[d][i]);
        }
    }
    float g1[3];
#pragma unroll
    for (int i = 0; i < 3; i++) g1[i] = fmaf(mode_k[2], S[2][i], fmaf(mode_k[1], S[1][i], mode_k[0] * S[0][i]));
#pragma unroll
    for (int ax = 0; ax < 3; ax++) {
      const int flip = ax == 0 ? 1 : (ax == 1 ? 3 : 4);
#pragma unroll
      for (int i = 0; i < 3; i++) g1[i] = fmaf(-mode_sign[ax], __shfl_xor_sync(0xffffffffu, g1[i], flip), g1[i]);
    }
    if (valid) {
      float* fo = reinterpret_cast<float*>(a.fe) + (size_t)(3 * p) * ld_e + e;  // corner-major planes
      fo[0]      = g1[0];
      fo[ld_e]   = g1[1];
      fo[2 * ld_e] = g1[2];
      if (!isfinite(g1[0]) || !isfinite(g1[1]) || !isfinite(g1[2])) status |= NSM_STATUS_NONFINITE;
    }
  }
  if (status) atomicOr(a.status, status);
  if (fallbacks) atomicAdd(m.fallback_count, (unsigned long long)fallbacks);
  fence_before_sync();
  __syncthreads();  // every thread's timeout record is in `err`
  if (r == 0 && err) {
    mbar_wait(&mbar, phase ^ 1u);  // bounded: let the timed-out MMA drain before the columns are freed
    atomicOr(a.status, NSM_STATUS_TIMEOUT);
  }
  __syncthreads();
  if (warp == 0) tmem_dealloc(tb, el::kCols);
}

// Reference geometry of every point for the closure kernel: the same
// gather, point gradient and inverse the kernel formed per step before.
__global__ void k_closure_geometry(ElementArgs a, float* __restrict__ geo)
{
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= 8L * a.E) return;
  const long e = i >> 3;
  const int  p = (int)(i & 7);
  float      w[3][2][2];
  point_weights(p, w);
  float x[8][3];
#pragma unroll
  for (int n = 0; n < 8; n++) {
    const int id = __ldg(&a.conn[n * a.ld_e + e]);
#pragma unroll
    for (int k = 0; k < 3; k++) x[n][k] = __ldg(&a.Xf[k * a.ld_n + id]);
  }
  float DX[3][3], G0[3][3], det0;
  point_gradient(x, w, DX);
  invert3<float>(DX, G0, det0);
  float4* out = reinterpret_cast<float4*>(geo + i * 12);
  out[0]      = make_float4(G0[0][0], G0[0][1], G0[0][2], G0[1][0]);
  out[1]      = make_float4(G0[1][1], G0[1][2], G0[2][0], G0[2][1]);
  out[2]      = make_float4(G0[2][2], det0, 0.0f, 0.0f);
}

cudaError_t launch_closure_geometry(const ElementArgs& a, float* geo, cudaStream_t stream)
{
  if (a.E == 0) return cudaSuccess;
  k_closure_geometry<<<(unsigned)((8L * a.E + 127) / 128), 128, 0, stream>>>(a, geo);
  return cudaGetLastError();
}

static int g_blocks_per_sm = 0;

// Co-resident CTAs per SM from the kernel's registers and shared memory and
// the device's limits, capped by the SM's 512 tensor-memory columns.  (The
// runtime's occupancy query answers 1 for this kernel, which would leave a
// single 4-warp CTA per SM.)  The CTAs never wait on one another, so a
// count above what the hardware co-schedules only adds a wave.
cudaError_t setup_element_kernel()
{
  cudaError_t e = cudaFuncSetAttribute(k_element_mlp, cudaFuncAttributeMaxDynamicSharedMemorySize, el::SMEM);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(k_element_mlp, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
  if (e != cudaSuccess) return e;
  cudaFuncAttributes fa;
  if ((e = cudaFuncGetAttributes(&fa, k_element_mlp)) != cudaSuccess) return e;
  int dev = 0, regs_sm = 0, smem_sm = 0, smem_rsv = 0, threads_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev);
  cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
  cudaDeviceGetAttribute(&smem_rsv, cudaDevAttrReservedSharedMemoryPerBlock, dev);
  cudaDeviceGetAttribute(&threads_sm, cudaDevAttrMaxThreadsPerMultiProcessor, dev);
  const int warp_regs = ((fa.numRegs * 32 + 255) / 256) * 256;  // allocated per warp in units of 256
  const int by_regs   = regs_sm / (warp_regs * 4);
  const int by_smem   = smem_sm / ((int)fa.sharedSizeBytes + el::SMEM + smem_rsv);
  const int by_thr    = threads_sm / 128;
  int       n         = 512 / (int)el::kCols;
  n                   = by_regs < n ? by_regs : n;
  n                   = by_smem < n ? by_smem : n;
  n                   = by_thr < n ? by_thr : n;
  g_blocks_per_sm     = n < 1 ? 1 : n;
  return cudaSuccess;
}

cudaError_t launch_element_mlp(const ElementArgs& a, const MlpElementArgs& m, cudaStream_t stream)
{
  if (a.E == 0) return cudaSuccess;
  if (a.e_begin != 0) return cudaErrorInvalidValue;  // the closure kernel runs over all elements
  const long chunks = (a.E + el::kElems - 1) / el::kElems;
  const long cap    = (long)num_sms() * (g_blocks_per_sm > 0 ? g_blocks_per_sm : 1);
  const int  grid   = (int)(chunks < cap ? chunks : cap);
  k_element_mlp<<<grid, 128, el::SMEM, stream>>>(a, m);
  return cudaGetLastError();
}

}  // namespace mlp
}  // namespace nsm
