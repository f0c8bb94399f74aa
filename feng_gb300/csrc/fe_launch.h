// Kernel launches of the Krylov solver and the multigrid preconditioner with
// programmatic dependent launch (PDL): a kernel may be scheduled while the
// previous kernel of its stream is still running; it first waits
// (griddepcontrol.wait) until that kernel has finished and its writes are
// visible, then lets its own successor be scheduled
// (griddepcontrol.launch_dependents).  The launch latency and the block
// rasterisation of a kernel thereby overlap the tail of the one before it,
// which matters for the chains of short dependent kernels of an Arnoldi step
// (a V-cycle's coarse levels, the Gram-Schmidt reductions).  Every kernel
// launched through launch_k starts with FE_PDL_ENTRY(); kernels launched
// without the attribute keep the plain stream order.  FENG_PDL=0 launches
// without the attribute (the same kernels, fully serialised).
#pragma once

#include <cuda_runtime.h>

#include <cstdlib>
#include <cstring>

#include "fe_common.h"

#ifdef __CUDACC__
#define FE_PDL_ENTRY() asm volatile("griddepcontrol.wait;\n\tgriddepcontrol.launch_dependents;" ::: "memory")
#endif

namespace feng {

inline bool pdl_enabled()
{
  static const bool on = [] {
    const char *e = std::getenv("FENG_PDL");
    return !(e && std::strcmp(e, "0") == 0);
  }();
  return on;
}

// kernel<<<grid, block, smem, stream>>>(args...) with the PDL attribute;
// the error, if any, is left for cudaGetLastError / the stream capture.
template <typename... P, typename... A>
inline void launch_k(void (*kernel)(P...), dim3 grid, dim3 block, size_t smem, cudaStream_t stream, A &&...args)
{
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = stream;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = pdl_enabled() ? 1 : 0;
  cudaLaunchKernelEx(&cfg, kernel, static_cast<P>(args)...);
  count_launch();
}

}  // namespace feng
