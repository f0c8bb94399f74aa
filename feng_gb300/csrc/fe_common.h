// Common definitions shared by the host setup code, the CUDA kernels and the
// C-ABI.  Status codes mirror feNG's feStatus (src/feMessage.h:44-62):
// 0 is success, negative values are errors.
#pragma once

#include <atomic>
#include <cstdint>
#include <cstdio>
#include <string>
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

#define FE_TRY(expr)                   \
  do {                                 \
    int _s = (expr);                   \
    if(_s != ::feng::FE_OK) return _s; \
  } while(0)

}  // namespace feng
