// Max-norm of a caller-owned device vector without any device allocation.
//
// Some callers cannot allocate device memory: code that owns all device
// memory through its own pool and forbids stray cudaMalloc calls, and loops
// that must not pay cudaMalloc's implicit device synchronization.  For them
// this entry point keeps its scratch (per-block partial maxima, the result
// and a completion counter) in one file-scope __device__ array that every GPU
// loading the library holds until the process exits.
//
// The array's name is only a host-side stand-in in host code: the device
// address is obtained once per device with cudaGetSymbolAddress (with that
// device current) and passed to the kernel.  The first call on a device does
// this set-up, so it should come before any stream capture.  The cached
// address belongs to the device's primary context: after cudaDeviceReset on
// a device, this entry point must not be called on it again in the same
// process.  Every call shares the one array, so calls that overlap on the GPU
// (two streams, two threads) race; the counter is cleared by each call before
// its kernel.  A NaN anywhere in the input makes the result NaN.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/feng_cuda.h"
#include "fe_common.h"

namespace feng {
namespace {

constexpr int NA_THREADS = 256;
constexpr int NA_PER_THREAD = 16;
constexpr int64_t NA_CHUNK = (int64_t)NA_THREADS * NA_PER_THREAD;  // elements per block
constexpr int NA_MAX_BLOCKS = FE_NOALLOC_MAX_N / (NA_THREADS * NA_PER_THREAD);
static_assert((int64_t)NA_MAX_BLOCKS * NA_CHUNK == FE_NOALLOC_MAX_N, "maximum size must be whole blocks");

struct NoAllocScratch {
  double partial[NA_MAX_BLOCKS];
  double result;
  unsigned int counter;
};

static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

constexpr int MAX_DEVICES = 64;
std::mutex g_mutex;
NoAllocScratch *g_addr[MAX_DEVICES] = {};

// One block per chunk of NA_CHUNK elements: block maximum into partial[b];
// the last block to finish reduces the partials into result and re-arms the
// counter.
__global__ void __launch_bounds__(NA_THREADS) k_max_norm_noalloc(const double *__restrict__ x, int64_t n,
                                                                 NoAllocScratch *sc)
{
  __shared__ double sh[NA_THREADS];
  __shared__ bool last;
  const int64_t base = (int64_t)blockIdx.x * NA_CHUNK;
  double m = 0.;
  for(int k = 0; k < NA_PER_THREAD; ++k) {
    const int64_t i = base + (int64_t)k * NA_THREADS + threadIdx.x;
    if(i < n) m = nan_max(m, fabs(x[i]));
  }
  sh[threadIdx.x] = m;
  __syncthreads();
  for(int o = NA_THREADS / 2; o > 0; o >>= 1) {
    if(threadIdx.x < o) sh[threadIdx.x] = nan_max(sh[threadIdx.x], sh[threadIdx.x + o]);
    __syncthreads();
  }
  if(threadIdx.x == 0) {
    sc->partial[blockIdx.x] = sh[0];
    __threadfence();
    last = atomicAdd(&sc->counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if(!last) return;
  __threadfence();
  double r = 0.;
  for(int b = threadIdx.x; b < (int)gridDim.x; b += NA_THREADS) r = nan_max(r, ((volatile double *)sc->partial)[b]);
  sh[threadIdx.x] = r;
  __syncthreads();
  for(int o = NA_THREADS / 2; o > 0; o >>= 1) {
    if(threadIdx.x < o) sh[threadIdx.x] = nan_max(sh[threadIdx.x], sh[threadIdx.x + o]);
    __syncthreads();
  }
  if(threadIdx.x == 0) {
    sc->result = sh[0];
    sc->counter = 0;
  }
}

}  // namespace
}  // namespace feng

using namespace feng;

extern "C" int fe_cuda_max_norm_noalloc(const double *x, int64_t n, void *stream, double *result)
{
  if(!result || (n > 0 && !x) || n < 0) {
    set_error("fe_cuda_max_norm_noalloc: null pointer or negative size");
    return FE_INVALID_ARG;
  }
  if(n > FE_NOALLOC_MAX_N) {
    set_error("fe_cuda_max_norm_noalloc: %lld elements exceed the maximum of %d held by its static scratch",
              (long long)n, FE_NOALLOC_MAX_N);
    return FE_INVALID_ARG;
  }
  if(n == 0) {
    *result = 0.;
    return FE_OK;
  }
  int dev = 0;
  if(cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEVICES) {
    cudaGetLastError();
    set_error("fe_cuda_max_norm_noalloc: no usable current device");
    return FE_CUDA_DEVICE_FAIL;
  }
  NoAllocScratch *sc = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_mutex);
    if(!g_addr[dev]) {
      // Once per device, with that device current: the device address of
      // the static scratch.
      void *p = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if(e != cudaSuccess || !p) {
        cudaGetLastError();
        set_error("fe_cuda_max_norm_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
        return FE_CUDA_DEVICE_FAIL;
      }
      g_addr[dev] = (NoAllocScratch *)p;
    }
    sc = g_addr[dev];
  }
  cudaStream_t s = (cudaStream_t)stream;
  // The counter must start at zero (a previous call could have been cut short).
  if(cudaMemsetAsync(&sc->counter, 0, sizeof(unsigned int), s) != cudaSuccess) {
    cudaGetLastError();
    set_error("fe_cuda_max_norm_noalloc: clearing the scratch counter failed");
    return FE_CUDA_DEVICE_FAIL;
  }
  const int blocks = (int)((n + NA_CHUNK - 1) / NA_CHUNK);
  (k_max_norm_noalloc<<<blocks, NA_THREADS, 0, s>>>(x, n, sc), ::feng::count_launch());
  cudaError_t e = cudaGetLastError();
  if(e == cudaSuccess) e = cudaMemcpyAsync(result, &sc->result, sizeof(double), cudaMemcpyDeviceToHost, s);
  if(e == cudaSuccess) e = cudaStreamSynchronize(s);
  if(e != cudaSuccess) {
    set_error("fe_cuda_max_norm_noalloc: %s", cudaGetErrorString(e));
    return FE_CUDA_DEVICE_FAIL;
  }
  return FE_OK;
}
