// noalloc.cu — dfsph_density_error_noalloc: the solver's average-density-error
// reduction over a caller's device array, with no device allocation at all.
//
// Why it exists: some callers of this library cannot allocate GPU memory at the point
// where they need the solver's convergence measure — a host embedding that hands the
// whole device memory budget to its own pool at start-up, code running in a real-time
// loop that forbids allocations after initialisation, or code that runs while another
// component holds the allocator. They pass their own input and output buffers; the only
// scratch (the per-block partial sums of the fixed-order reduction) lives in a
// file-scope device array that every GPU loading this library holds until exit.
//
// Limits and sharing:
//  - at most NOALLOC_MAX_BLOCKS blocks of 256 threads, i.e. n <= 4,194,304 particles;
//    larger n is rejected with DFSPH_ERR_INVALID_ARG;
//  - every call on a device shares the one scratch array and leaves its contents
//    behind; a call writes every partial it later reads, so nothing needs clearing,
//    but calls whose kernels overlap on the GPU (different streams, no ordering) race
//    on the scratch and must not be issued;
//  - the first call on each device resolves the scratch array's device address with
//    cudaGetSymbolAddress (device set-up); make that first call before any stream
//    capture on that device;
//  - the resolved address is cached per device index for the life of the process. A
//    reset of the device's primary context (cudaDeviceReset) reloads the module and may
//    move the array, so resetting a device while this library is loaded is not supported
//    by this entry point.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <string>

#include "../../include/dfsph.h"
#include "engine_api.h"

namespace {

constexpr int NOALLOC_THREADS = 256;
constexpr int NOALLOC_MAX_BLOCKS = 16384;
constexpr int NOALLOC_MAX_DEVICES = 64;

static __device__ __align__(256) double g_noalloc_partials[NOALLOC_MAX_BLOCKS];

double *g_partials_ptr[NOALLOC_MAX_DEVICES] = {};
std::mutex g_setup_mutex;

template <class T>
__global__ void __launch_bounds__(NOALLOC_THREADS)
    k_density_error_partials(const T *__restrict__ ra, int n, T rho0, int pressure, double *__restrict__ partials) {
  __shared__ double ws[NOALLOC_THREADS / 32];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double e = 0.0;
  if (i < n) {
    const T r = ra[i];
    // the same per-particle terms as the Jacobi passes: rho0 rho_adv - rho0 (pressure)
    // or rho0 rho_dot (divergence), formed in the fluid scalar type
    e = pressure ? (double)(rho0 * r - rho0) : (double)(rho0 * r);
  }
  for (int o = 16; o > 0; o >>= 1) e += __shfl_xor_sync(0xffffffffu, e, o);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) ws[w] = e;
  __syncthreads();
  if (w == 0) {
    double s = lane < (int)(blockDim.x >> 5) ? ws[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) partials[blockIdx.x] = s;
  }
}

__global__ void __launch_bounds__(NOALLOC_THREADS)
    k_density_error_final(int nparts, const double *__restrict__ partials, double scale, double *__restrict__ out) {
  __shared__ double ws[NOALLOC_THREADS / 32];
  double s = 0.0;
  for (int k = threadIdx.x; k < nparts; k += blockDim.x) s += partials[k];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += ws[w];
    *out = t * scale;
  }
}

int fail(int code, const std::string &m) {
  dfsph::set_last_error(m);  // readable through dfsph_last_error()
  return code;
}

}  // namespace

extern "C" int dfsph_density_error_noalloc(const void *rho_adv, int32_t fluid_precision, int64_t n, double density0,
                                           int32_t pressure_mode, double *out, void *stream) {
  dfsph::set_last_error("");
  if (!rho_adv || !out) return fail(DFSPH_ERR_INVALID_ARG, "rho_adv and out must be device pointers");
  if (n <= 0) return fail(DFSPH_ERR_INVALID_ARG, "n must be positive");
  if (n > (int64_t)NOALLOC_MAX_BLOCKS * NOALLOC_THREADS)
    return fail(DFSPH_ERR_INVALID_ARG, "n exceeds the allocation-free reduction's maximum of 4,194,304 particles");
  if (fluid_precision != DFSPH_FP32 && fluid_precision != DFSPH_FP64)
    return fail(DFSPH_ERR_INVALID_ARG, "fluid_precision");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(DFSPH_ERR_CUDA, cudaGetErrorString(e));
  if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) return fail(DFSPH_ERR_UNSUPPORTED, "device index beyond the set-up table");
  double *scratch = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_partials_ptr[dev]) {
      void *p = nullptr;
      e = cudaGetSymbolAddress(&p, g_noalloc_partials);
      if (e != cudaSuccess) return fail(DFSPH_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      g_partials_ptr[dev] = static_cast<double *>(p);
    }
    scratch = g_partials_ptr[dev];
  }
  const int nn = (int)n;
  const int blocks = (nn + NOALLOC_THREADS - 1) / NOALLOC_THREADS;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (fluid_precision == DFSPH_FP32)
    k_density_error_partials<float><<<blocks, NOALLOC_THREADS, 0, s>>>(static_cast<const float *>(rho_adv), nn,
                                                                       (float)density0, pressure_mode, scratch);
  else
    k_density_error_partials<double><<<blocks, NOALLOC_THREADS, 0, s>>>(static_cast<const double *>(rho_adv), nn,
                                                                        density0, pressure_mode, scratch);
  k_density_error_final<<<1, NOALLOC_THREADS, 0, s>>>(blocks, scratch, 1.0 / (double)n, out);
  e = cudaGetLastError();
  if (e != cudaSuccess) return fail(DFSPH_ERR_CUDA, cudaGetErrorString(e));
  return DFSPH_OK;
}
