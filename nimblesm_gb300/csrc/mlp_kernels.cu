// Kernels of the learned constitutive closure (network and layouts in
// mlp_common.cuh): training-set generation from the neo-Hookean material,
// the training step (forward + backward, all GEMMs on the 5th-generation
// tensor cores), a deterministic gradient reduction with Adam, the BF16
// operand images, and batched inference.
#include <cuda_runtime.h>

#include "hex_math.cuh"
#include "mlp_common.cuh"
#include "mlp_kernels.cuh"
#include "nsm_kernels.cuh"

namespace nsm {
namespace mlp {

using namespace tc;

// ---------------------------------------------------------------------------
// Training set: F = I + N(0, s^2) per entry, rejected while det F < min_det,
// sigma from the engine's FP64 neo-Hookean (the same function the FP64 element
// kernel uses, parity-checked against the reference); stored as H = F - I
// (row-major) and sigma / G (symmetric order), FP32.

__device__ __forceinline__ uint64_t splitmix64(uint64_t& s)
{
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z          = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z          = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

__device__ __forceinline__ double uniform01(uint64_t& s) { return ((splitmix64(s) >> 11) + 0.5) * (1.0 / 9007199254740992.0); }

__global__ void k_generate(long n, unsigned long long seed, double sd, double min_det, double K, double G,
                           float* __restrict__ X, float* __restrict__ Y, int* __restrict__ status)
{
  long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint64_t s = seed ^ (0x632BE59BD9B4E019ull * (uint64_t)(i + 1));
  double   H[3][3];
  bool     ok = false;
  for (int attempt = 0; attempt < 64 && !ok; attempt++) {
    for (int q = 0; q < 9; q += 2) {  // Box-Muller pairs
      double u1 = uniform01(s), u2 = uniform01(s);
      double r = sqrt(-2.0 * log(u1)), t = 6.283185307179586 * u2;
      H[q / 3][q % 3] = sd * r * cos(t);
      if (q + 1 < 9) H[(q + 1) / 3][(q + 1) % 3] = sd * r * sin(t);
    }
    double F00 = 1 + H[0][0], F11 = 1 + H[1][1], F22 = 1 + H[2][2];
    double det = F00 * (F11 * F22 - H[1][2] * H[2][1]) - H[0][1] * (H[1][0] * F22 - H[1][2] * H[2][0]) +
                 H[0][2] * (H[1][0] * H[2][1] - F11 * H[2][0]);
    ok = det >= min_det;
  }
  if (!ok) atomicOr(status, NSM_STATUS_BAD_JACOBIAN);
  double sig[6], C[3][3], J;
  neohookean<double>(H, K, G, sig, C, J);
  for (int q = 0; q < 9; q++) X[9 * i + q] = (float)H[q / 3][q % 3];
  for (int q = 0; q < 6; q++) Y[6 * i + q] = (float)(sig[q] / G);
}

// Sum over the training set of |(sigma/G - B(H)) / |x|^3|^2 (per-block
// partials, summed in block order on the host): sets the residual scale.
__global__ void k_residual_moment(long n, const float* __restrict__ X, const float* __restrict__ Y, float k_over_g,
                                  float in_scale, double* __restrict__ partial)
{
  __shared__ double s[256];
  double            acc = 0.0;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    float x[9], xs[9], L[6];
    for (int q = 0; q < 9; q++) {
      x[q]  = X[9 * i + q];
      xs[q] = x[q] * in_scale;
    }
    base_part(x, k_over_g, L);
    const double g = gate(xs);
    for (int q = 0; q < 6; q++) {
      double r = ((double)Y[6 * i + q] - (double)L[q]) / g;
      acc += r * r;
    }
  }
  s[threadIdx.x] = acc;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = s[0];
}

// ---------------------------------------------------------------------------
// BF16 operand images from the FP32 master parameters.
__global__ void k_images(const float* __restrict__ P, uint8_t* __restrict__ img)
{
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  // W1x [64][32]
  if (t < kHid * kInX) {
    int   n = t / kInX, k = t % kInX;
    float w = 0.0f;
    if (k < 9) w = P[oW1 + n * 9 + k];
    else if (k == 9) w = P[ob1 + n];
    else if (k >= 16 && k < 25) w = P[oW1 + n * 9 + (k - 16)];
    store_bf16(img + kOffW1, n, k, kInX, w);
  }
  // W2 [64][64] and W2t [64][64]
  if (t < kHid * kHid) {
    int n = t / kHid, k = t % kHid;
    store_bf16(img + kOffW2, n, k, kHid, P[oW2 + n * kHid + k]);
    store_bf16(img + kOffW2t, n, k, kHid, P[oW2 + k * kHid + n]);
  }
  // W3x [16][64] and W3t [64][16]
  if (t < kOutX * kHid) {
    int n = t / kHid, k = t % kHid;
    store_bf16(img + kOffW3, n, k, kHid, n < kOut ? P[oW3 + n * kHid + k] : 0.0f);
    int n2 = t / kOutX, k2 = t % kOutX;
    store_bf16(img + kOffW3t, n2, k2, kOutX, k2 < kOut ? P[oW3 + k2 * kHid + n2] : 0.0f);
  }
}

// ---------------------------------------------------------------------------
// Training step: one tile of 128 points per CTA (thread r <-> point r, whose
// accumulator row is tensor-memory lane r).  Writes this CTA's gradient of
// the mean-squared residual loss and its loss sum.
namespace tr {
constexpr int X    = 0;                        // [128][32]
constexpr int A1   = X + 128 * kInX * 2;       // [128][64]
constexpr int A2   = A1 + 128 * kHid * 2;      // [128][64]
constexpr int DZ3  = A2 + 128 * kHid * 2;      // [128][16]
constexpr int DZ2  = DZ3 + 128 * kOutX * 2;    // [128][64]
constexpr int AOP  = DZ2 + 128 * kHid * 2;     // [128][128 points]: dZ2^T rows 0-63, dZ1^T 64-127
constexpr int BOP  = AOP + 128 * 128 * 2;      // [112][128]: A1^T 0-63, X^T 64-95, ones 96
constexpr int AOP3 = BOP + 112 * 128 * 2;      // [128][128]: dZ3^T rows 0-5, zeros elsewhere
constexpr int BOP3 = AOP3 + 128 * 128 * 2;     // [80][128]: A2^T 0-63, ones 64
constexpr int W    = BOP3 + 80 * 128 * 2;      // operand images
constexpr int B    = W + kImgBytes;            // b2[64], b3[6]
constexpr int END  = B + 512;
constexpr int SMEM = END + 16384;              // slack past the last operand
// tensor-memory columns
constexpr uint32_t cZ1 = 0, cZ2 = 64, cZ3 = 128, cDA2 = 144, cDA1 = 208, cGW = 272, cGW3 = 384, kCols = 512;
}  // namespace tr

struct Sync {
  uint64_t* mbar;
  uint32_t  phase;
  int*      err;
};

// Issue-side: make operand writes visible to the tensor core and order them
// before the MMAs thread 0 is about to issue.
__device__ __forceinline__ void publish_operands()
{
  fence_proxy_async();
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
}

// Wait for the last commit; false (and the CTA-wide error flag) on timeout.
__device__ __forceinline__ bool await_mma(Sync& s)
{
  const bool ok = mbar_wait(s.mbar, s.phase);
  s.phase ^= 1u;
  if (!ok) atomicOr(s.err, 1);
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  return *s.err == 0;
}

__device__ __forceinline__ void ld_row(uint32_t tbase, uint32_t col, int n16, float* v)
{
  const uint32_t lane_base = (uint32_t)(((threadIdx.x >> 5) & 3) * 32) << 16;  // the warp's lane quarter
  for (int c = 0; c < n16; c++) tmem_ld16(tbase + lane_base + col + 16 * c, v + 16 * c);
  tmem_wait_ld();
}

__device__ __forceinline__ void gemm(uint32_t d, const uint8_t* a, int a_rows_k, const uint8_t* b, int b_rows_k,
                                     int N, int K, bool accumulate_first)
{
  // a, b: K-major tiles whose row pitch per 8-row group is 16*K bytes
  const uint32_t idesc = idesc_bf16_f32(128, N);
  for (int ks = 0; ks < K / 16; ks++) {
    uint64_t ad = smem_desc(smem_addr(a) + ks * 2 * kLBO, kLBO, 16 * a_rows_k);
    uint64_t bd = smem_desc(smem_addr(b) + ks * 2 * kLBO, kLBO, 16 * b_rows_k);
    mma_bf16(d, ad, bd, idesc, accumulate_first || ks > 0);
  }
}

// Two warpgroups per tile: thread t owns row r = t % 128 (tensor-memory lane r)
// and, in the 64-column epilogues, the columns [32 h, 32 h + 32) of half
// h = t / 128, so each thread's share of the activation and gradient work is
// half a row and the tile's dependent MMA rounds wait on half as much
// epilogue each.
constexpr int kTrainThreads = 256;

__global__ void __launch_bounds__(kTrainThreads) k_train(const float* __restrict__ X, const float* __restrict__ Y,
                                                         long n, long first, long stride_a, long offset_b,
                                                         const uint8_t* __restrict__ img, const float* __restrict__ P,
                                                         Scales sc, float inv_batch, float* __restrict__ grad_partial,
                                                         float* __restrict__ loss_partial, int* __restrict__ status)
{
  extern __shared__ __align__(1024) uint8_t sm[];
  __shared__ uint64_t mbar;
  __shared__ uint32_t tslot;
  __shared__ int      err;
  __shared__ float    red[128];
  const int           tid = threadIdx.x, warp = tid >> 5, r = tid & 127, half = tid >> 7;
  const int           c0  = 32 * half;  // this thread's first column in the 64-column epilogues

  // The point's pair (half 0) is gathered first, from its row of the epoch's
  // visiting order, so that the loads' latency passes while the operand
  // regions below are set up.
  const long j     = first + (long)blockIdx.x * 128 + r;
  const bool valid = j < n;
  float      x[9], y[6];
  if (half == 0) {
    const long idx = valid ? (long)((stride_a * j + offset_b) % n) : 0;
#pragma unroll
    for (int q = 0; q < 9; q++) x[q] = X[9 * idx + q];
#pragma unroll
    for (int q = 0; q < 6; q++) y[q] = Y[6 * idx + q];
  }

  if (warp == 0) {
    tmem_alloc(&tslot, tr::kCols);
    tmem_relinquish();
  }
  if (tid == 0) {
    mbar_init(&mbar, 1);
    err = 0;
  }
  // constant operand regions (zero rows, ones rows), weight images, biases
  {
    uint4 z = make_uint4(0, 0, 0, 0);
    for (int i = tid; i < (tr::W - tr::AOP) / 16; i += kTrainThreads) reinterpret_cast<uint4*>(sm + tr::AOP)[i] = z;
    const uint4* src = reinterpret_cast<const uint4*>(img);
    for (int i = tid; i < kImgBytes / 16; i += kTrainThreads) reinterpret_cast<uint4*>(sm + tr::W)[i] = src[i];
    float* bias = reinterpret_cast<float*>(sm + tr::B);
    if (tid < kHid) bias[tid] = P[ob2 + tid];
    if (tid < kOut) bias[64 + tid] = P[ob3 + tid];
  }
  __syncthreads();
  if (half == 0) {
    store_bf16(sm + tr::BOP, 96, r, 128, 1.0f);
    store_bf16(sm + tr::BOP3, 64, r, 128, 1.0f);
  }
  const float* b2 = reinterpret_cast<const float*>(sm + tr::B);
  const float* b3 = b2 + 64;
  const uint32_t tb = tslot;
  Sync           sy{&mbar, 0u, &err};

  // ---- the point (half 0: its input row and target) ----
  float t[6];
  if (half == 0) {
    float xs[9];
    for (int q = 0; q < 9; q++) xs[q] = x[q] * sc.in_scale;
    {
      float L[6];
      base_part(x, sc.k_over_g, L);
      const float g = gate(xs) * sc.res_scale;
      for (int q = 0; q < 6; q++) t[q] = (y[q] - L[q]) / g;
    }
    float row[kInX];
    input_row(xs, row);
    for (int k0 = 0; k0 < kInX; k0 += 8) store_chunk(sm + tr::X, r, k0, kInX, row + k0);
    for (int q = 0; q < kInX; q++)
      if (q < 10 || (q >= 16 && q < 25)) store_bf16(sm + tr::BOP, 64 + q, r, 128, row[q]);
  }
  publish_operands();

  // ---- forward ----
  if (tid == 0) {
    gemm(tb + tr::cZ1, sm + tr::X, kInX, sm + tr::W + kOffW1, kInX, kHid, kInX, false);
    mma_commit(&mbar);
  }
  if (!await_mma(sy)) goto cleanup;
  {
    float z[32];
    ld_row(tb, tr::cZ1 + c0, 2, z);
    for (int q = 0; q < 32; q++) z[q] = act(z[q]);
    for (int k0 = 0; k0 < 32; k0 += 8) store_chunk(sm + tr::A1, r, c0 + k0, kHid, z + k0);
    for (int q = 0; q < 32; q++) store_bf16(sm + tr::BOP, c0 + q, r, 128, z[q]);
  }
  publish_operands();
  if (tid == 0) {
    gemm(tb + tr::cZ2, sm + tr::A1, kHid, sm + tr::W + kOffW2, kHid, kHid, kHid, false);
    mma_commit(&mbar);
  }
  if (!await_mma(sy)) goto cleanup;
  {
    float z[32];
    ld_row(tb, tr::cZ2 + c0, 2, z);
    for (int q = 0; q < 32; q++) z[q] = act(z[q] + b2[c0 + q]);
    for (int k0 = 0; k0 < 32; k0 += 8) store_chunk(sm + tr::A2, r, c0 + k0, kHid, z + k0);
    for (int q = 0; q < 32; q++) store_bf16(sm + tr::BOP3, c0 + q, r, 128, z[q]);
  }
  publish_operands();
  if (tid == 0) {
    gemm(tb + tr::cZ3, sm + tr::A2, kHid, sm + tr::W + kOffW3, kHid, kOutX, kHid, false);
    mma_commit(&mbar);
  }
  if (!await_mma(sy)) goto cleanup;
  if (half == 0) {
    float z[16], g[16];
    ld_row(tb, tr::cZ3, 1, z);
    float lsum = 0.0f;
    for (int q = 0; q < 16; q++) g[q] = 0.0f;
    for (int q = 0; q < kOut; q++) {
      float d = valid ? (z[q] + b3[q] - t[q]) : 0.0f;
      lsum += d * d;
      g[q] = 2.0f * d * inv_batch;
    }
    red[r] = lsum;
    for (int k0 = 0; k0 < 16; k0 += 8) store_chunk(sm + tr::DZ3, r, k0, kOutX, g + k0);
    for (int q = 0; q < kOut; q++) store_bf16(sm + tr::AOP3, q, r, 128, g[q]);
  }
  publish_operands();
  // ---- backward ----
  if (tid == 0) {
    gemm(tb + tr::cDA2, sm + tr::DZ3, kOutX, sm + tr::W + kOffW3t, kOutX, kHid, kOutX, false);
    mma_commit(&mbar);
  }
  if (!await_mma(sy)) goto cleanup;
  {
    float da[32], z[32];
    ld_row(tb, tr::cDA2 + c0, 2, da);
    ld_row(tb, tr::cZ2 + c0, 2, z);
    for (int q = 0; q < 32; q++) da[q] *= act_grad(z[q] + b2[c0 + q]);
    for (int k0 = 0; k0 < 32; k0 += 8) store_chunk(sm + tr::DZ2, r, c0 + k0, kHid, da + k0);
    for (int q = 0; q < 32; q++) store_bf16(sm + tr::AOP, c0 + q, r, 128, da[q]);
  }
  publish_operands();
  if (tid == 0) {
    gemm(tb + tr::cDA1, sm + tr::DZ2, kHid, sm + tr::W + kOffW2t, kHid, kHid, kHid, false);
    mma_commit(&mbar);
  }
  if (!await_mma(sy)) goto cleanup;
  {
    float da[32], z[32];
    ld_row(tb, tr::cDA1 + c0, 2, da);
    ld_row(tb, tr::cZ1 + c0, 2, z);
    for (int q = 0; q < 32; q++) store_bf16(sm + tr::AOP, 64 + c0 + q, r, 128, da[q] * act_grad(z[q]));
  }
  publish_operands();
  // weight gradients: sums over the 128 points of the tile (K = points)
  if (tid == 0) {
    gemm(tb + tr::cGW, sm + tr::AOP, 128, sm + tr::BOP, 128, 112, 128, false);
    gemm(tb + tr::cGW3, sm + tr::AOP3, 128, sm + tr::BOP3, 128, 80, 128, false);
    mma_commit(&mbar);
  }
  if (!await_mma(sy)) goto cleanup;
  {
    float* G = grad_partial + (long)blockIdx.x * kParams;
    if (half == 0) {
      // row r of the [112] block: W2 and b2 gradients (rows < 64), W1 and b1 (rows >= 64)
      float v[112];
      ld_row(tb, tr::cGW, 7, v);
      if (r < 64) {
        for (int q = 0; q < 64; q++) G[oW2 + r * 64 + q] = v[q];
        G[ob2 + r] = v[96];
      } else {
        const int o = r - 64;
        for (int q = 0; q < 9; q++) G[oW1 + o * 9 + q] = v[64 + q] + v[64 + 16 + q];
        G[ob1 + o] = v[64 + 9];
      }
    } else if (warp == 4) {  // rows 0..31 of the W3 block: W3 and b3 gradients of rows < 6
      float w3[80];
      ld_row(tb, tr::cGW3, 5, w3);
      if (r < kOut) {
        for (int q = 0; q < 64; q++) G[oW3 + r * 64 + q] = w3[q];
        G[ob3 + r] = w3[64];
      }
    }
  }
  __syncthreads();
  for (int w = 64; w > 0; w >>= 1) {
    if (tid < w) red[tid] += red[tid + w];
    __syncthreads();
  }
  if (tid == 0) loss_partial[blockIdx.x] = red[0];

cleanup:
  if (tid == 0 && err) {
    mbar_wait(sy.mbar, sy.phase ^ 1u);  // bounded: let a timed-out MMA drain before the columns are freed
    atomicOr(status, NSM_STATUS_TIMEOUT);
  }
  fence_before_sync();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tb, tr::kCols);
}

// The operand-image entries of parameter i (the layout k_images writes), from
// its value w.  The biases b2 and b3 have none (the kernels read them in
// FP32), nor do the images' zero padding entries, which k_images wrote.
__device__ __forceinline__ void store_images(int i, float w, uint8_t* __restrict__ img)
{
  if (i < ob1) {
    const int n = (i - oW1) / kIn, k = (i - oW1) % kIn;
    store_bf16(img + kOffW1, n, k, kInX, w);
    store_bf16(img + kOffW1, n, k + 16, kInX, w);
  } else if (i < oW2) {
    store_bf16(img + kOffW1, i - ob1, 9, kInX, w);
  } else if (i < ob2) {
    const int n = (i - oW2) / kHid, k = (i - oW2) % kHid;
    store_bf16(img + kOffW2, n, k, kHid, w);
    store_bf16(img + kOffW2t, k, n, kHid, w);
  } else if (i >= oW3 && i < ob3) {
    const int n = (i - oW3) / kHid, k = (i - oW3) % kHid;
    store_bf16(img + kOffW3, n, k, kHid, w);
    store_bf16(img + kOffW3t, k, n, kOutX, w);
  }
}

// Deterministic reduction of the per-CTA gradients, an Adam step on the FP32
// master parameters, and the new parameters' BF16 operand-image entries.
// Eight lanes share a parameter: lane j sums the partials of CTAs j, j + 8,
// ... in order (loads issued four at a time ahead of the in-order sum), and
// three butterfly steps combine the eight sums in a fixed order, so every
// run gives the same bits while a launch has many loads in flight.
constexpr int kAdamLanes = 8;
__global__ void k_adam(int ncta, const float* __restrict__ grad_partial, float* __restrict__ P,
                       float* __restrict__ m1, float* __restrict__ m2, float lr, float beta1, float beta2,
                       float eps, float bc1, float bc2, uint8_t* __restrict__ img)
{
  const long t   = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const int  i   = (int)(t / kAdamLanes), sub = (int)(t % kAdamLanes);
  const bool own = i < kParams;
  float      g   = 0.0f;
  if (own) {
    const float* gp = grad_partial + i;
    int          c  = sub;
    for (; c + 3 * kAdamLanes < ncta; c += 4 * kAdamLanes) {
      const float p0 = gp[(long)c * kParams], p1 = gp[(long)(c + kAdamLanes) * kParams],
                  p2 = gp[(long)(c + 2 * kAdamLanes) * kParams], p3 = gp[(long)(c + 3 * kAdamLanes) * kParams];
      g += p0;
      g += p1;
      g += p2;
      g += p3;
    }
    for (; c < ncta; c += kAdamLanes) g += gp[(long)c * kParams];
  }
#pragma unroll
  for (int o = 1; o < kAdamLanes; o <<= 1) g += __shfl_xor_sync(0xffffffffu, g, o);
  if (!own || sub != 0) return;
  float a = beta1 * m1[i] + (1.0f - beta1) * g;
  float b = beta2 * m2[i] + (1.0f - beta2) * g * g;
  m1[i]   = a;
  m2[i]   = b;
  const float w = P[i] - lr * (a / bc1) / (sqrtf(b / bc2) + eps);
  P[i]          = w;
  store_images(i, w, img);
}

__global__ void k_sum_gradient(int ncta, const float* __restrict__ grad_partial, float* __restrict__ g)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kParams) return;
  float s = 0.0f;
  for (int c = 0; c < ncta; c++) s += grad_partial[(long)c * kParams + i];
  g[i] = s;
}

// ---------------------------------------------------------------------------
// Inference on a batch of points: H (row-major, FP32) -> sigma / G.  Points
// outside the training envelope take the plain neo-Hookean stress and are
// counted.
namespace inf {
constexpr int X    = 0;                     // [128][32]
constexpr int A1   = X + 128 * kInX * 2;    // [128][64]
constexpr int A2   = A1 + 128 * kHid * 2;   // [128][64]
constexpr int W    = A2 + 128 * kHid * 2;   // W1x, W2, W3x images
constexpr int B    = W + kOffW2t;           // b2[64], b3[6]
constexpr int END  = B + 512;
constexpr int SMEM = END + 16384;
constexpr uint32_t cZ1 = 0, cZ2 = 64, cZ3 = 128, kCols = 256;
}  // namespace inf

__global__ void __launch_bounds__(128) k_predict(long n, const float* __restrict__ H, const uint8_t* __restrict__ img,
                                                 const float* __restrict__ P, Scales sc, double K, double G,
                                                 double* __restrict__ sigma, int* __restrict__ fallback,
                                                 int* __restrict__ status)
{
  extern __shared__ __align__(1024) uint8_t sm[];
  __shared__ uint64_t mbar;
  __shared__ uint32_t tslot;
  __shared__ int      err;
  const int           r = threadIdx.x, warp = r >> 5;
  if (warp == 0) {
    tmem_alloc(&tslot, inf::kCols);
    tmem_relinquish();
  }
  if (r == 0) {
    mbar_init(&mbar, 1);
    err = 0;
  }
  {
    const uint4* src = reinterpret_cast<const uint4*>(img);
    for (int i = r; i < kOffW2t / 16; i += 128) reinterpret_cast<uint4*>(sm + inf::W)[i] = src[i];
    float* bias = reinterpret_cast<float*>(sm + inf::B);
    if (r < kHid) bias[r] = P[ob2 + r];
    if (r < kOut) bias[64 + r] = P[ob3 + r];
  }
  const float* b2 = reinterpret_cast<const float*>(sm + inf::B);
  const float* b3 = b2 + 64;
  const long   i  = (long)blockIdx.x * 128 + r;
  const bool   valid = i < n;
  float        h[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  if (valid)
    for (int q = 0; q < 9; q++) h[q] = H[9 * i + q];
  float xs[9], row[kInX];
  for (int q = 0; q < 9; q++) xs[q] = h[q] * sc.in_scale;
  input_row(xs, row);
  for (int k0 = 0; k0 < kInX; k0 += 8) store_chunk(sm + inf::X, r, k0, kInX, row + k0);
  publish_operands();
  Sync           sy{&mbar, 0u, &err};
  const uint32_t tb = tslot;
  if (r == 0) {
    gemm(tb + inf::cZ1, sm + inf::X, kInX, sm + inf::W + kOffW1, kInX, kHid, kInX, false);
    mma_commit(&mbar);
  }
  if (!await_mma(sy)) goto cleanup;
  {
    float z[64];
    ld_row(tb, inf::cZ1, 4, z);
    for (int q = 0; q < 64; q++) z[q] = act(z[q]);
    for (int k0 = 0; k0 < 64; k0 += 8) store_chunk(sm + inf::A1, r, k0, kHid, z + k0);
  }
  publish_operands();
  if (r == 0) {
    gemm(tb + inf::cZ2, sm + inf::A1, kHid, sm + inf::W + kOffW2, kHid, kHid, kHid, false);
    mma_commit(&mbar);
  }
  if (!await_mma(sy)) goto cleanup;
  {
    float z[64];
    ld_row(tb, inf::cZ2, 4, z);
    for (int q = 0; q < 64; q++) z[q] = act(z[q] + b2[q]);
    for (int k0 = 0; k0 < 64; k0 += 8) store_chunk(sm + inf::A2, r, k0, kHid, z + k0);
  }
  publish_operands();
  if (r == 0) {
    gemm(tb + inf::cZ3, sm + inf::A2, kHid, sm + inf::W + kOffW3, kHid, kOutX, kHid, false);
    mma_commit(&mbar);
  }
  if (!await_mma(sy)) goto cleanup;
  {
    float z[16];
    ld_row(tb, inf::cZ3, 1, z);
    if (valid) {
      if (in_envelope(h, sc)) {
        float L[6];
        base_part(h, sc.k_over_g, L);
        const float g = gate(xs) * sc.res_scale;
        for (int q = 0; q < kOut; q++) sigma[6 * i + q] = G * (double)(L[q] + g * (z[q] + b3[q]));
      } else {
        double Hd[3][3], s6[6], C[3][3], J;
        for (int q = 0; q < 9; q++) Hd[q / 3][q % 3] = h[q];
        neohookean<double>(Hd, K, G, s6, C, J);
        for (int q = 0; q < kOut; q++) sigma[6 * i + q] = s6[q];
        atomicAdd(fallback, 1);
      }
    }
  }
cleanup:
  if (r == 0 && err) {
    mbar_wait(sy.mbar, sy.phase ^ 1u);  // bounded: let a timed-out MMA drain before the columns are freed
    atomicOr(status, NSM_STATUS_TIMEOUT);
  }
  fence_before_sync();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tslot, inf::kCols);
}

// ---------------------------------------------------------------------------
cudaError_t launch_generate(long n, unsigned long long seed, double sd, double min_det, double K, double G, float* X,
                            float* Y, int* status, cudaStream_t s)
{
  if (n <= 0) return cudaSuccess;
  k_generate<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, seed, sd, min_det, K, G, X, Y, status);
  return cudaGetLastError();
}

cudaError_t launch_residual_moment(long n, const float* X, const float* Y, float k_over_g, float in_scale,
                                   double* partial, int blocks, cudaStream_t s)
{
  k_residual_moment<<<blocks, 256, 0, s>>>(n, X, Y, k_over_g, in_scale, partial);
  return cudaGetLastError();
}

cudaError_t launch_images(const float* P, uint8_t* img, cudaStream_t s)
{
  k_images<<<(kHid * kHid + 127) / 128, 128, 0, s>>>(P, img);
  return cudaGetLastError();
}

cudaError_t setup_kernels()
{
  cudaError_t e = cudaFuncSetAttribute(k_train, cudaFuncAttributeMaxDynamicSharedMemorySize, tr::SMEM);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(k_predict, cudaFuncAttributeMaxDynamicSharedMemorySize, inf::SMEM);
}

cudaError_t launch_train(int tiles, const float* X, const float* Y, long n, long first, long stride_a, long offset_b,
                         const uint8_t* img, const float* P, const Scales& sc, float inv_batch, float* grad_partial,
                         float* loss_partial, int* status, cudaStream_t s)
{
  k_train<<<tiles, kTrainThreads, tr::SMEM, s>>>(X, Y, n, first, stride_a, offset_b, img, P, sc, inv_batch, grad_partial,
                                       loss_partial, status);
  return cudaGetLastError();
}

cudaError_t launch_adam(int ncta, const float* grad_partial, float* P, float* m1, float* m2, float lr, float beta1,
                        float beta2, float eps, float bc1, float bc2, uint8_t* img, cudaStream_t s)
{
  k_adam<<<(kParams * kAdamLanes + 255) / 256, 256, 0, s>>>(ncta, grad_partial, P, m1, m2, lr, beta1, beta2, eps,
                                                             bc1, bc2, img);
  return cudaGetLastError();
}

cudaError_t launch_sum_gradient(int ncta, const float* grad_partial, float* g, cudaStream_t s)
{
  k_sum_gradient<<<(kParams + 255) / 256, 256, 0, s>>>(ncta, grad_partial, g);
  return cudaGetLastError();
}

cudaError_t launch_predict(long n, const float* H, const uint8_t* img, const float* P, const Scales& sc, double K,
                           double G, double* sigma, int* fallback, int* status, cudaStream_t s)
{
  if (n <= 0) return cudaSuccess;
  k_predict<<<(unsigned)((n + 127) / 128), 128, inf::SMEM, s>>>(n, H, img, P, sc, K, G, sigma, fallback, status);
  return cudaGetLastError();
}

}  // namespace mlp
}  // namespace nsm
