// Host side of the learned constitutive closure (C ABI nsm_mlp_*): parameter
// initialisation, training-set generation, the training loop (tensor-core
// forward/backward, deterministic reduction, Adam) and batched inference.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/nimble_gb300.h"
#include "mlp_element.cuh"
#include "mlp_kernels.cuh"
#include "nsm_kernels.cuh"

using namespace nsm::mlp;

struct nsm_mlp {
  int          device = 0;
  cudaStream_t stream = nullptr;
  double       K = 0, G = 0;
  Scales       sc{20.0f, 1.0f, 2.0f, 0.2f, 0.5f};
  float*       d_P = nullptr;
  float*       d_m1 = nullptr;
  float*       d_m2 = nullptr;
  uint8_t*     d_img = nullptr;
  float*       d_X = nullptr;  // training set: H (row-major) [n][9]
  float*       d_Y = nullptr;  // sigma / G [n][6]
  long         n = 0;
  float*       d_grad = nullptr;  // [max_tiles][kParams]
  float*       d_loss = nullptr;  // [max_tiles]
  int          max_tiles = 0;
  int*         d_status = nullptr;
  int*         d_fallback = nullptr;
  long         adam_step = 0;
};

namespace {

thread_local std::string g_mlp_error;

int mlp_fail(int code, const std::string& m)
{
  g_mlp_error = m;
  return code;
}

#define MLP_CUDA(call)                                                                         \
  do {                                                                                         \
    cudaError_t _e = (call);                                                                   \
    if (_e != cudaSuccess) return mlp_fail(NSM_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(_e)); \
  } while (0)

uint64_t mix(uint64_t& s)
{
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z          = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z          = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

int ensure_tiles(nsm_mlp* m, int tiles)
{
  if (tiles <= m->max_tiles) return NSM_OK;
  if (m->d_grad) cudaFree(m->d_grad);
  if (m->d_loss) cudaFree(m->d_loss);
  m->d_grad = nullptr;
  m->d_loss = nullptr;
  MLP_CUDA(cudaMalloc(&m->d_grad, sizeof(float) * kParams * (size_t)tiles));
  MLP_CUDA(cudaMalloc(&m->d_loss, sizeof(float) * (size_t)tiles));
  m->max_tiles = tiles;
  return NSM_OK;
}

int check_status(nsm_mlp* m)
{
  int st = 0;
  MLP_CUDA(cudaMemcpyAsync(&st, m->d_status, sizeof(int), cudaMemcpyDeviceToHost, m->stream));
  MLP_CUDA(cudaMemsetAsync(m->d_status, 0, sizeof(int), m->stream));
  MLP_CUDA(cudaStreamSynchronize(m->stream));
  if (st & NSM_STATUS_TIMEOUT) return mlp_fail(NSM_ERR_CUDA, "tensor-core completion wait timed out");
  if (st & NSM_STATUS_BAD_JACOBIAN) return mlp_fail(NSM_ERR_BAD_JACOBIAN, "training sample rejection failed");
  return NSM_OK;
}

}  // namespace

namespace nsm {
namespace mlp {
bool element_args(nsm_mlp* m, MlpElementArgs* out, double* bulk, double* shear)
{
  if (!m || !out) return false;
  out->img = m->d_img;
  out->P   = m->d_P;
  out->sc  = m->sc;
  out->geo = nullptr;  // the model's (nsm_set_mlp_closure)
  if (bulk) *bulk = m->K;
  if (shear) *shear = m->G;
  return true;
}
}  // namespace mlp
}  // namespace nsm

extern "C" {

const char* nsm_mlp_last_error(void) { return g_mlp_error.c_str(); }

int nsm_mlp_create(double bulk_modulus, double shear_modulus, unsigned long long seed, int device, nsm_mlp** out)
{
  if (!out || !(bulk_modulus > 0) || !(shear_modulus > 0)) return mlp_fail(NSM_ERR_INVALID_ARGUMENT, "invalid argument");
  *out       = nullptr;
  nsm_mlp* m = new nsm_mlp();
  m->device  = device;
  m->K       = bulk_modulus;
  m->G       = shear_modulus;
  m->sc.k_over_g = (float)(bulk_modulus / shear_modulus);
  auto bail = [&](int code) {
    nsm_mlp_destroy(m);
    return code;
  };
  if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaMalloc(&m->d_P, sizeof(float) * kParams) != cudaSuccess ||
      cudaMalloc(&m->d_m1, sizeof(float) * kParams) != cudaSuccess ||
      cudaMalloc(&m->d_m2, sizeof(float) * kParams) != cudaSuccess ||
      cudaMalloc(&m->d_img, kImgBytes) != cudaSuccess || cudaMalloc(&m->d_status, sizeof(int)) != cudaSuccess ||
      cudaMalloc(&m->d_fallback, sizeof(int)) != cudaSuccess || setup_kernels() != cudaSuccess ||
      setup_element_kernel() != cudaSuccess)
    return bail(mlp_fail(NSM_ERR_CUDA, "allocation failed"));
  // Xavier-uniform weights from a seeded generator, zero biases
  std::vector<float> P(kParams, 0.0f);
  uint64_t           s = seed;
  auto uni = [&](double a) { return (float)(a * (2.0 * ((mix(s) >> 11) * (1.0 / 9007199254740992.0)) - 1.0)); };
  for (int i = 0; i < kHid * kIn; i++) P[oW1 + i] = uni(std::sqrt(6.0 / (kIn + kHid)));
  for (int i = 0; i < kHid * kHid; i++) P[oW2 + i] = uni(std::sqrt(6.0 / (kHid + kHid)));
  for (int i = 0; i < kOut * kHid; i++) P[oW3 + i] = uni(std::sqrt(6.0 / (kHid + kOut)));
  if (cudaMemcpy(m->d_P, P.data(), sizeof(float) * kParams, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemset(m->d_m1, 0, sizeof(float) * kParams) != cudaSuccess ||
      cudaMemset(m->d_m2, 0, sizeof(float) * kParams) != cudaSuccess ||
      cudaMemset(m->d_status, 0, sizeof(int)) != cudaSuccess || launch_images(m->d_P, m->d_img, m->stream) != cudaSuccess ||
      cudaStreamSynchronize(m->stream) != cudaSuccess)
    return bail(mlp_fail(NSM_ERR_CUDA, "initialisation failed"));
  *out = m;
  return NSM_OK;
}

int nsm_mlp_destroy(nsm_mlp* m)
{
  if (!m) return NSM_OK;
  cudaSetDevice(m->device);
  if (m->stream) cudaStreamSynchronize(m->stream);
  void* ptrs[] = {m->d_P, m->d_m1, m->d_m2, m->d_img, m->d_X, m->d_Y, m->d_grad, m->d_loss, m->d_status, m->d_fallback};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (m->stream) cudaStreamDestroy(m->stream);
  delete m;
  return NSM_OK;
}

int nsm_mlp_generate(nsm_mlp* m, long n, unsigned long long seed, double perturbation, double min_det)
{
  if (!m || n < 1 || !(perturbation > 0)) return mlp_fail(NSM_ERR_INVALID_ARGUMENT, "invalid argument");
  MLP_CUDA(cudaSetDevice(m->device));
  if (m->d_X) cudaFree(m->d_X);
  if (m->d_Y) cudaFree(m->d_Y);
  m->d_X = m->d_Y = nullptr;
  MLP_CUDA(cudaMalloc(&m->d_X, sizeof(float) * 9 * (size_t)n));
  MLP_CUDA(cudaMalloc(&m->d_Y, sizeof(float) * 6 * (size_t)n));
  m->n = n;
  MLP_CUDA(launch_generate(n, seed, perturbation, min_det, m->K, m->G, m->d_X, m->d_Y, m->d_status, m->stream));
  m->sc.in_scale = (float)(1.0 / perturbation);
  m->sc.envelope = (float)(4.0 * perturbation);
  m->sc.min_det  = (float)min_det;
  const int blocks = 1024;
  double*   d_part = nullptr;
  MLP_CUDA(cudaMalloc(&d_part, sizeof(double) * blocks));
  std::vector<double> part(blocks);
  cudaError_t e = launch_residual_moment(n, m->d_X, m->d_Y, m->sc.k_over_g, m->sc.in_scale, d_part, blocks, m->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(part.data(), d_part, sizeof(double) * blocks, cudaMemcpyDeviceToHost, m->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
  cudaFree(d_part);
  if (e != cudaSuccess) return mlp_fail(NSM_ERR_CUDA, cudaGetErrorString(e));
  double sum = 0.0;
  for (double p : part) sum += p;
  m->sc.res_scale = (float)std::sqrt(sum / (6.0 * (double)n));
  if (!(m->sc.res_scale > 0)) m->sc.res_scale = 1.0f;
  return check_status(m);
}

int nsm_mlp_train(nsm_mlp* m, int epochs, int batch_tiles, double lr, double* final_loss)
{
  if (!m || epochs < 0 || batch_tiles < 1 || !(lr > 0)) return mlp_fail(NSM_ERR_INVALID_ARGUMENT, "invalid argument");
  if (!m->d_X) return mlp_fail(NSM_ERR_STATE, "no training set (nsm_mlp_generate first)");
  MLP_CUDA(cudaSetDevice(m->device));
  int r = ensure_tiles(m, batch_tiles);
  if (r) return r;
  const long   batch       = 128L * batch_tiles;
  const long   steps_epoch = (m->n + batch - 1) / batch;
  const long   total       = steps_epoch * epochs;
  const double beta1 = 0.9, beta2 = 0.999, eps = 1e-8;
  uint64_t     s = 0x5EEDull + (uint64_t)m->adam_step;
  // the last epoch's per-tile losses stay on the device until the epoch ends
  // (no per-step synchronisation), then are summed in step and tile order
  std::vector<float> loss;
  float*             d_epoch_loss = nullptr;
  if (epochs > 0) MLP_CUDA(cudaMalloc(&d_epoch_loss, sizeof(float) * (size_t)steps_epoch * batch_tiles));
  struct Free {
    float* p;
    ~Free() { if (p) cudaFree(p); }
  } free_epoch_loss{d_epoch_loss};
  double epoch_loss = 0.0;
  for (int ep = 0; ep < epochs; ep++) {
    // a fresh pseudo-random visiting order per epoch: j -> (a j + b) mod n, gcd(a, n) = 1
    long a;
    do {
      a = (long)(mix(s) % (uint64_t)m->n);
    } while (a == 0 || std::gcd(a, m->n) != 1);
    const long b = (long)(mix(s) % (uint64_t)m->n);
    epoch_loss   = 0.0;
    for (long st = 0; st < steps_epoch; st++) {
      const long   first = st * batch;
      const long   pts   = std::min(batch, m->n - first);
      const int    tiles = (int)((pts + 127) / 128);
      const long   k     = m->adam_step + 1;
      const double frac  = total > 1 ? (double)(ep * steps_epoch + st) / (double)(total - 1) : 0.0;
      const double lr_t  = lr * (0.01 + 0.99 * 0.5 * (1.0 + std::cos(3.141592653589793 * frac)));
      float* d_loss = ep == epochs - 1 ? d_epoch_loss + st * batch_tiles : m->d_loss;
      MLP_CUDA(launch_train(tiles, m->d_X, m->d_Y, m->n, first, a, b, m->d_img, m->d_P, m->sc, (float)(1.0 / pts),
                            m->d_grad, d_loss, m->d_status, m->stream));
      MLP_CUDA(launch_adam(tiles, m->d_grad, m->d_P, m->d_m1, m->d_m2, (float)lr_t, (float)beta1, (float)beta2,
                           (float)eps, (float)(1.0 - std::pow(beta1, (double)k)), (float)(1.0 - std::pow(beta2, (double)k)),
                           m->d_img, m->stream));
      m->adam_step++;
    }
    if (ep == epochs - 1) {
      loss.resize((size_t)steps_epoch * batch_tiles);
      MLP_CUDA(cudaMemcpyAsync(loss.data(), d_epoch_loss, sizeof(float) * loss.size(), cudaMemcpyDeviceToHost, m->stream));
      MLP_CUDA(cudaStreamSynchronize(m->stream));
      for (long st = 0; st < steps_epoch; st++) {
        const long pts   = std::min(batch, m->n - st * batch);
        const int  tiles = (int)((pts + 127) / 128);
        for (int t = 0; t < tiles; t++) epoch_loss += loss[(size_t)st * batch_tiles + t];
      }
    }
    r = check_status(m);
    if (r) return r;
  }
  if (final_loss) *final_loss = epochs > 0 ? epoch_loss / (6.0 * (double)m->n) : 0.0;
  return NSM_OK;
}

int nsm_mlp_get_params(nsm_mlp* m, float* params, float* scales)
{
  if (!m) return mlp_fail(NSM_ERR_INVALID_ARGUMENT, "null");
  MLP_CUDA(cudaSetDevice(m->device));
  if (params) {
    MLP_CUDA(cudaMemcpyAsync(params, m->d_P, sizeof(float) * kParams, cudaMemcpyDeviceToHost, m->stream));
    MLP_CUDA(cudaStreamSynchronize(m->stream));
  }
  if (scales) {
    scales[0] = m->sc.in_scale;
    scales[1] = m->sc.res_scale;
    scales[2] = m->sc.k_over_g;
    scales[3] = m->sc.envelope;
    scales[4] = m->sc.min_det;
  }
  return NSM_OK;
}

int nsm_mlp_set_params(nsm_mlp* m, const float* params, const float* scales)
{
  if (!m) return mlp_fail(NSM_ERR_INVALID_ARGUMENT, "null");
  MLP_CUDA(cudaSetDevice(m->device));
  if (params) {
    MLP_CUDA(cudaMemcpyAsync(m->d_P, params, sizeof(float) * kParams, cudaMemcpyHostToDevice, m->stream));
    MLP_CUDA(launch_images(m->d_P, m->d_img, m->stream));
    MLP_CUDA(cudaStreamSynchronize(m->stream));
  }
  if (scales) m->sc = Scales{scales[0], scales[1], scales[2], scales[3], scales[4]};
  return NSM_OK;
}

int nsm_mlp_gradient(nsm_mlp* m, long n, const float* H, const float* Y, float* grad, double* loss)
{
  if (!m || n < 1 || !H || !Y || !grad) return mlp_fail(NSM_ERR_INVALID_ARGUMENT, "invalid argument");
  MLP_CUDA(cudaSetDevice(m->device));
  const int tiles = (int)((n + 127) / 128);
  int       r     = ensure_tiles(m, tiles);
  if (r) return r;
  float *dH = nullptr, *dY = nullptr, *dg = nullptr;
  MLP_CUDA(cudaMalloc(&dH, sizeof(float) * 9 * n));
  MLP_CUDA(cudaMalloc(&dY, sizeof(float) * 6 * n));
  MLP_CUDA(cudaMalloc(&dg, sizeof(float) * kParams));
  std::vector<float> lp(tiles);
  cudaError_t        e = cudaMemcpyAsync(dH, H, sizeof(float) * 9 * n, cudaMemcpyHostToDevice, m->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dY, Y, sizeof(float) * 6 * n, cudaMemcpyHostToDevice, m->stream);
  if (e == cudaSuccess)
    e = launch_train(tiles, dH, dY, n, 0, 1, 0, m->d_img, m->d_P, m->sc, (float)(1.0 / n), m->d_grad, m->d_loss,
                     m->d_status, m->stream);
  if (e == cudaSuccess) e = launch_sum_gradient(tiles, m->d_grad, dg, m->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(grad, dg, sizeof(float) * kParams, cudaMemcpyDeviceToHost, m->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(lp.data(), m->d_loss, sizeof(float) * tiles, cudaMemcpyDeviceToHost, m->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
  cudaFree(dH);
  cudaFree(dY);
  cudaFree(dg);
  if (e != cudaSuccess) return mlp_fail(NSM_ERR_CUDA, cudaGetErrorString(e));
  if (loss) {
    double s = 0;
    for (float v : lp) s += v;
    *loss = s / (double)n;
  }
  return check_status(m);
}

int nsm_mlp_training_sample(nsm_mlp* m, long first, long count, float* H, float* Y)
{
  if (!m || first < 0 || count < 0 || first + count > m->n || (count > 0 && (!H || !Y)))
    return mlp_fail(NSM_ERR_INVALID_ARGUMENT, "range outside the training set");
  MLP_CUDA(cudaSetDevice(m->device));
  MLP_CUDA(cudaMemcpyAsync(H, m->d_X + 9 * first, sizeof(float) * 9 * count, cudaMemcpyDeviceToHost, m->stream));
  MLP_CUDA(cudaMemcpyAsync(Y, m->d_Y + 6 * first, sizeof(float) * 6 * count, cudaMemcpyDeviceToHost, m->stream));
  MLP_CUDA(cudaStreamSynchronize(m->stream));
  return NSM_OK;
}

int nsm_mlp_predict(nsm_mlp* m, long n, const double* F, double* sigma, int* fallback_count)
{
  if (!m || n < 1 || !F || !sigma) return mlp_fail(NSM_ERR_INVALID_ARGUMENT, "invalid argument");
  MLP_CUDA(cudaSetDevice(m->device));
  // reference full-tensor slots (xx,yy,zz,xy,yz,zx,yx,zy,xz) -> H row-major
  static const int slot[9] = {0, 3, 8, 6, 1, 4, 5, 7, 2};
  std::vector<float> H((size_t)9 * n);
  for (long i = 0; i < n; i++)
    for (int q = 0; q < 9; q++) H[9 * i + q] = (float)(F[9 * i + slot[q]] - ((q % 4) == 0 ? 1.0 : 0.0));
  float*  dH = nullptr;
  double* dS = nullptr;
  MLP_CUDA(cudaMalloc(&dH, sizeof(float) * 9 * n));
  MLP_CUDA(cudaMalloc(&dS, sizeof(double) * 6 * n));
  int         fb = 0;
  cudaError_t e  = cudaMemcpyAsync(dH, H.data(), sizeof(float) * 9 * n, cudaMemcpyHostToDevice, m->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(m->d_fallback, 0, sizeof(int), m->stream);
  if (e == cudaSuccess) e = launch_predict(n, dH, m->d_img, m->d_P, m->sc, m->K, m->G, dS, m->d_fallback, m->d_status, m->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(sigma, dS, sizeof(double) * 6 * n, cudaMemcpyDeviceToHost, m->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&fb, m->d_fallback, sizeof(int), cudaMemcpyDeviceToHost, m->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
  cudaFree(dH);
  cudaFree(dS);
  if (e != cudaSuccess) return mlp_fail(NSM_ERR_CUDA, cudaGetErrorString(e));
  if (fallback_count) *fallback_count = fb;
  return check_status(m);
}

}  // extern "C"
