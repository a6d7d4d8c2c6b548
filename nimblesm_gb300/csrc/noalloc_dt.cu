// Stable time step of the current configuration for callers that cannot
// allocate GPU memory.
//
// Some callers cannot call cudaMalloc at the point where they need the stable
// time step: a host framework that owns every device buffer through its own
// pool and forbids new allocations once a run has started, code that runs
// while a CUDA stream is being captured into a graph (where an allocation
// would break the capture), or a real-time loop that must not touch the
// allocator.  nsm_critical_time_step_noalloc serves them: the caller passes
// the mesh and displacement and a one-double output, and the per-element time
// steps and the block minima live in a fixed array compiled into this library
// (every GPU that loads the library holds it until the process exits).
//
// The arithmetic is the reference's (src/nimble_block_base.cc:51-84 with
// src/nimble_element.cc:221-260): dt = min over elements of L_e / sqrt(K / rho),
// L_e the smaller of the least node-pair distance and the least bounding-box
// extent of the element in the configuration X + u.  This file is compiled
// without FMA contraction, so with u = 0 the result equals nsm_critical_time_step
// bit for bit.
#include <atomic>
#include <cstdio>

#include <cuda_runtime.h>

#include "../../include/nimble_gb300.h"
#include "nsm_kernels.cuh"

namespace {
constexpr int kMaxBlocks = 1024;
}  // namespace

// The scratch: per-element time steps, then per-block minima.
static __device__ __align__(256) double g_noalloc_scratch[NSM_NOALLOC_MAX_ELEMENTS + kMaxBlocks];

namespace {


// Device address of g_noalloc_scratch per device, looked up once per device
// with that device current.  (In host code the symbol's name is only a
// stand-in, not a device address.)  Atomic, so two host threads making a
// device's first call at once store the same value without a data race.
constexpr int      kMaxDevices = 64;
std::atomic<void*> g_scratch_ptr[kMaxDevices];

int cuda_error(cudaError_t e, const char* where)
{
  char msg[256];
  snprintf(msg, sizeof msg, "nsm_critical_time_step_noalloc: %s: %s", where, cudaGetErrorString(e));
  return nsm::set_last_error(NSM_ERR_CUDA, msg);
}

int invalid(const char* why)
{
  char msg[256];
  snprintf(msg, sizeof msg, "nsm_critical_time_step_noalloc: %s", why);
  return nsm::set_last_error(NSM_ERR_INVALID_ARGUMENT, msg);
}

// An element whose connectivity names a node outside [0, N) reads no
// coordinate and gets the time step -1, so that the minimum, and dt_out, is
// negative: a bad mesh is reported instead of read out of bounds.
__global__ void k_elem_dt(int N, int E, const int* __restrict__ conn, const double* __restrict__ coords,
                          const double* __restrict__ disp, double sound_speed, double* __restrict__ dt_elem)
{
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= E) return;
  int ids[8];
  for (int n = 0; n < 8; n++) {
    ids[n] = conn[8L * e + n];
    if (ids[n] < 0 || ids[n] >= N) {
      dt_elem[e] = -1.0;
      return;
    }
  }
  double x[8][3];
  for (int n = 0; n < 8; n++) {
    const long id = ids[n];
    for (int k = 0; k < 3; k++) x[n][k] = coords[3 * id + k] + (disp ? disp[3 * id + k] : 0.0);
  }
  double x_max = 0.0, y_max = 0.0, z_max = 0.0;  // maxima start at 0, as in the reference
  double x_min = 1.7976931348623157e308, y_min = x_min, z_min = x_min, min_d2 = x_min;
  for (int n = 0; n < 8; n++) {
    const double nx = x[n][0], ny = x[n][1], nz = x[n][2];
    if (nx < x_min) x_min = nx;
    if (nx > x_max) x_max = nx;
    if (ny < y_min) y_min = ny;
    if (ny > y_max) y_max = ny;
    if (nz < z_min) z_min = nz;
    if (nz > z_max) z_max = nz;
    for (int m = n + 1; m < 8; m++) {
      const double dx = nx - x[m][0], dy = ny - x[m][1], dz = nz - x[m][2];
      const double d2 = dx * dx + dy * dy + dz * dz;
      if (d2 < min_d2) min_d2 = d2;
    }
  }
  double len = sqrt(min_d2);
  double box = x_max - x_min;
  if (y_max - y_min < box) box = y_max - y_min;
  if (z_max - z_min < box) box = z_max - z_min;
  if (box < len) len = box;
  dt_elem[e] = len / sound_speed;
}

// Minimum of n values (grid-stride, one result per block).
__global__ void k_block_min(long n, const double* __restrict__ in, double* __restrict__ out)
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

}  // namespace

extern "C" int nsm_critical_time_step_noalloc(int num_nodes, int num_elem, const double* coords,
                                              const double* displacement, const int* conn, double density,
                                              double bulk_modulus, double* dt_out, void* stream)
{
  if (num_elem < 0 || num_nodes < 0) return invalid("negative node or element count");
  if (!dt_out) return invalid("null dt_out");
  if (num_elem > 0 && (!coords || !conn || num_nodes < 1)) return invalid("null mesh array or no nodes");
  if (num_elem > NSM_NOALLOC_MAX_ELEMENTS) return invalid("more elements than NSM_NOALLOC_MAX_ELEMENTS");
  if (!(density > 0.0) || !(bulk_modulus > 0.0)) return invalid("density and bulk modulus must be positive");
  // An error left by earlier work is reported, not cleared: it is the caller's.
  cudaError_t e = cudaPeekAtLastError();
  if (e != cudaSuccess) return cuda_error(e, "an earlier CUDA error is pending");
  int dev = 0;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess) return cuda_error(e, "cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices) return invalid("device ordinal beyond the library's table");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (s) {  // the scratch looked up below is the current device's: the stream must be on it
    int sdev = -1;
    if ((e = cudaStreamGetDevice(s, &sdev)) != cudaSuccess) return cuda_error(e, "cudaStreamGetDevice");
    if (sdev != dev) return invalid("the stream belongs to another device than the current one");
  }
  void* p = g_scratch_ptr[dev].load(std::memory_order_acquire);
  if (!p) {
    if ((e = cudaGetSymbolAddress(&p, g_noalloc_scratch)) != cudaSuccess) return cuda_error(e, "cudaGetSymbolAddress");
    if (!p) return cuda_error(cudaErrorInvalidSymbol, "cudaGetSymbolAddress");
    g_scratch_ptr[dev].store(p, std::memory_order_release);
  }
  double*      dt_elem = static_cast<double*>(p);
  double*      partial = dt_elem + NSM_NOALLOC_MAX_ELEMENTS;
  int          blocks  = (num_elem + 255) / 256;
  if (blocks > kMaxBlocks) blocks = kMaxBlocks;
  if (num_elem > 0) {
    const double c = sqrt(bulk_modulus / density);
    k_elem_dt<<<(num_elem + 127) / 128, 128, 0, s>>>(num_nodes, num_elem, conn, coords, displacement, c, dt_elem);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_error(e, "k_elem_dt launch");
    k_block_min<<<blocks, 256, 0, s>>>(num_elem, dt_elem, partial);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_error(e, "k_block_min launch");
  }
  // With no elements the minimum over nothing is the largest double, the value
  // nsm_critical_time_step gives an empty model.
  k_block_min<<<1, 256, 0, s>>>(blocks, partial, dt_out);
  if ((e = cudaGetLastError()) != cudaSuccess) return cuda_error(e, "k_block_min launch");
  return NSM_OK;
}
