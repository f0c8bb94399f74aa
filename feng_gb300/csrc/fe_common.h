// Common definitions shared by the host setup code, the CUDA kernels and the
// C-ABI.  Status codes mirror feNG's feStatus (src/feMessage.h:44-62):
// 0 is success, negative values are errors.
#pragma once

#include <algorithm>
#include <atomic>
#include <cstdint>
#include <cstdio>
#include <string>
#include <thread>
#include <vector>

namespace feng {

enum Status : int {
  FE_OK = 0,
  FE_ERROR = -1,
  FE_READ_ERROR = -2,
  FE_INVALID_ARG = -3,
  FE_CUDA_FAIL = -4,
  FE_NOT_CONVERGED = -5,
  FE_PC_FAILED = -6,
  FE_NONFINITE = -7,
  FE_BAD_COLORING = -8,
};

// Last error message of the calling thread (read through fe_last_error()).
void set_error(const char *fmt, ...);
const char *last_error();

// Count of the library's kernel launches (graph replays add their kernel
// nodes); launches recorded while a stream is being captured are not counted.
extern std::atomic<long long> g_launches;
extern thread_local int g_capturing;
inline void count_launch()
{
  if(!g_capturing) g_launches.fetch_add(1, std::memory_order_relaxed);
}

// Maximum that propagates NaN (CUDA's fmax returns the non-NaN operand, which
// would let a NaN residual vanish from a max-norm and read as convergence).
#ifdef __CUDACC__
__host__ __device__ __forceinline__ double nan_max(double a, double b) { return (a > b || a != a) ? a : b; }
__host__ __device__ __forceinline__ float nan_maxf(float a, float b) { return (a > b || a != a) ? a : b; }
#endif

// Host loops of the set-up over [0, n) split into contiguous ranges run by
// up to 32 threads (f(begin, end)); small n runs inline.
template <typename F>
void parallel_for(int64_t n, F &&f, int64_t grain = 1 << 14)
{
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  const int64_t T = std::min<int64_t>({(int64_t)hw, 32, (n + grain - 1) / grain});
  if(T <= 1) {
    if(n > 0) f((int64_t)0, n);
    return;
  }
  const int64_t chunk = (n + T - 1) / T;
  std::vector<std::thread> th;
  for(int64_t t = 0; t < T; ++t) {
    const int64_t b = t * chunk, e = std::min(n, b + chunk);
    if(b < e) th.emplace_back([&f, b, e] { f(b, e); });
  }
  for(auto &x : th) x.join();
}

// SplitMix64 (Steele, Lea, Flood 2014): the generator of the mesh jitter,
// so a mesh can be regenerated from its seed alone.
struct SplitMix64 {
  uint64_t s;
  explicit SplitMix64(uint64_t seed) : s(seed) {}
  uint64_t next()
  {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  // Uniform double in [-1, 1) with 53 random bits.
  double uniform_pm1() { return (double)(next() >> 11) * (2.0 / 9007199254740992.0) - 1.0; }
};

#define FE_TRY(expr)                   \
  do {                                 \
    int _s = (expr);                   \
    if(_s != ::feng::FE_OK) return _s; \
  } while(0)

}  // namespace feng
