// CSR pattern of the system on the device (feEZCompressedRowStorage,
// src/feCompressedRowStorage.cpp:15-135): row r holds its diagonal and every
// unknown DOF coupled to r by a matrix form in an element holding r, sorted
// and unique -- the rule of build_csr_pattern (fe_setup.cpp), with the same
// result bit for bit.
//
// Steps: the DOF -> (element, local index) adjacency (counts by atomics, an
// exclusive scan on the host, a fill whose order inside a row does not
// matter); then one warp per row gathers the candidate columns into shared
// memory (warp-aggregated appends), sorts them (bitonic) and counts the
// distinct ones; a scan of the counts on the host gives the row pointers; a
// second warp pass writes the distinct columns.  A row with more than
// PAT_CAP candidates (element valences far above those of the meshes here)
// makes the build report FE_INVALID_ARG, and the automatic mode then takes
// the host path.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <vector>

#include "fe_common.h"
#include "fe_setup.h"

namespace feng {

namespace {

constexpr int PAT_CAP = 1024;  // candidates per row held in shared memory
constexpr int PAT_WARPS = 8;

#define CKP(x)                                                              \
  do {                                                                      \
    cudaError_t e_ = (x);                                                   \
    if(e_ != cudaSuccess) {                                                 \
      set_error("device pattern: %s (%s)", cudaGetErrorString(e_), #x);     \
      return FE_CUDA_FAIL;                                           \
    }                                                                       \
  } while(0)

__global__ void k_dof_count(int64_t total, const int32_t *__restrict__ adr, int64_t nInc, int32_t *__restrict__ cnt)
{
  for(int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int32_t d = adr[t];
    if(d >= 0 && d < nInc) atomicAdd(cnt + d, 1);
  }
}

__global__ void k_dof_fill(int64_t total, const int32_t *__restrict__ adr, int64_t nInc,
                           const int32_t *__restrict__ dptr, int32_t *__restrict__ fill, int32_t *__restrict__ adj)
{
  for(int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int32_t d = adr[t];
    if(d >= 0 && d < nInc) adj[dptr[d] + atomicAdd(fill + d, 1)] = (int32_t)t;
  }
}

// One warp per row: the row's sorted candidates in buf[0..n), n returned
// (-1: more than PAT_CAP candidates).
__device__ int gather_sorted(int64_t r, int nl, const int32_t *__restrict__ adr, const uint8_t *__restrict__ mask,
                             int64_t nInc, const int32_t *__restrict__ dptr, const int32_t *__restrict__ adj,
                             int32_t *buf)
{
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  const int32_t k0 = dptr[r], deg = dptr[r + 1] - k0;
  const int64_t total = (int64_t)deg * nl;
  if(lane == 0) buf[0] = (int32_t)r;  // the diagonal
  int n = 1;
  for(int64_t base = 0; base < total; base += 32) {
    const int64_t idx = base + lane;
    bool take = false;
    int32_t col = 0;
    if(idx < total) {
      const int32_t a = adj[k0 + idx / nl];  // element * nl + local row
      const int j = (int)(idx % nl);
      const int i = a % nl;
      col = adr[(int64_t)(a - i) + j];
      take = mask[i * nl + j] && col >= 0 && col < nInc;
    }
    const unsigned b = __ballot_sync(0xffffffffu, take);
    const int pos = n + __popc(b & lt);
    if(take && pos < PAT_CAP) buf[pos] = col;
    n += __popc(b);
  }
  __syncwarp();
  if(n > PAT_CAP) return -1;
  int N = 32;
  while(N < n) N <<= 1;
  for(int i = n + lane; i < N; i += 32) buf[i] = INT_MAX;
  __syncwarp();
  // bitonic sort of buf[0..N)
  for(int k = 2; k <= N; k <<= 1)
    for(int j = k >> 1; j > 0; j >>= 1) {
      for(int i = lane; i < N; i += 32) {
        const int p = i ^ j;
        if(p > i) {
          const int32_t x = buf[i], y = buf[p];
          if((x > y) == ((i & k) == 0)) {
            buf[i] = y;
            buf[p] = x;
          }
        }
      }
      __syncwarp();
    }
  return n;
}

__global__ void __launch_bounds__(PAT_WARPS * 32) k_row_count(int64_t nInc, int nl, const int32_t *__restrict__ adr,
                                                              const uint8_t *__restrict__ mask,
                                                              const int32_t *__restrict__ dptr,
                                                              const int32_t *__restrict__ adj, int32_t *__restrict__ len,
                                                              int *overflow)
{
  __shared__ int32_t sbuf[PAT_WARPS][PAT_CAP];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int32_t *buf = sbuf[warp];
  for(int64_t r = (int64_t)blockIdx.x * PAT_WARPS + warp; r < nInc; r += (int64_t)gridDim.x * PAT_WARPS) {
    const int n = gather_sorted(r, nl, adr, mask, nInc, dptr, adj, buf);
    if(n < 0) {
      if(lane == 0) {
        atomicOr(overflow, 1);
        len[r] = 0;
      }
      __syncwarp();
      continue;
    }
    int u = 0;
    for(int base = 0; base < n; base += 32) {
      const int i = base + lane;
      const bool f = i < n && (i == 0 || buf[i] != buf[i - 1]);
      u += __popc(__ballot_sync(0xffffffffu, f));
    }
    if(lane == 0) len[r] = u;
    __syncwarp();
  }
}

__global__ void __launch_bounds__(PAT_WARPS * 32) k_row_fill(int64_t nInc, int nl, const int32_t *__restrict__ adr,
                                                             const uint8_t *__restrict__ mask,
                                                             const int32_t *__restrict__ dptr,
                                                             const int32_t *__restrict__ adj,
                                                             const int64_t *__restrict__ ia, int32_t *__restrict__ ja)
{
  __shared__ int32_t sbuf[PAT_WARPS][PAT_CAP];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  int32_t *buf = sbuf[warp];
  for(int64_t r = (int64_t)blockIdx.x * PAT_WARPS + warp; r < nInc; r += (int64_t)gridDim.x * PAT_WARPS) {
    const int n = gather_sorted(r, nl, adr, mask, nInc, dptr, adj, buf);
    if(n < 0) continue;  // reported by the count pass
    int64_t o = ia[r];
    for(int base = 0; base < n; base += 32) {
      const int i = base + lane;
      const bool f = i < n && (i == 0 || buf[i] != buf[i - 1]);
      const unsigned b = __ballot_sync(0xffffffffu, f);
      if(f) ja[o + __popc(b & lt)] = buf[i];
      o += __popc(b);
    }
    __syncwarp();
  }
}

int grid_of(int64_t work, int per, int maxBlocks)
{
  return (int)std::max<int64_t>(1, std::min<int64_t>((work + per - 1) / per, maxBlocks));
}

}  // namespace

int build_csr_pattern_device(const ElementTables &et, int64_t nInc, CSRPattern &pat)
{
  const int nl = et.nloc;
  const int64_t nE = et.nElm, total = nE * nl;
  if(nl <= 0 || nl > 64 || total >= (int64_t)INT32_MAX || nInc >= (int64_t)INT32_MAX - 1) {
    set_error("device pattern: element tables out of range");
    return FE_INVALID_ARG;
  }
  std::vector<int32_t> adr32((size_t)total);
  parallel_for(total, [&](int64_t a, int64_t b) {
    for(int64_t k = a; k < b; ++k) adr32[k] = et.adr[k] < nInc ? (int32_t)et.adr[k] : -1;
  });
  int dev = 0, nsm = 1;
  CKP(cudaGetDevice(&dev));
  CKP(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  cudaStream_t s = nullptr;
  CKP(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  int32_t *dAdr = nullptr, *dCnt = nullptr, *dPtr = nullptr, *dAdj = nullptr, *dLen = nullptr, *dJa = nullptr;
  int64_t *dIa = nullptr;
  uint8_t *dMask = nullptr;
  int *dOver = nullptr;
  int status = FE_OK;
  auto run = [&]() -> int {
    CKP(cudaMalloc(&dAdr, sizeof(int32_t) * std::max<int64_t>(total, 1)));
    CKP(cudaMalloc(&dMask, (size_t)nl * nl));
    CKP(cudaMalloc(&dCnt, sizeof(int32_t) * (nInc + 1)));
    CKP(cudaMalloc(&dPtr, sizeof(int32_t) * (nInc + 1)));
    CKP(cudaMalloc(&dOver, sizeof(int)));
    CKP(cudaMemcpyAsync(dAdr, adr32.data(), sizeof(int32_t) * total, cudaMemcpyHostToDevice, s));
    CKP(cudaMemcpyAsync(dMask, et.mask.data(), (size_t)nl * nl, cudaMemcpyHostToDevice, s));
    CKP(cudaMemsetAsync(dCnt, 0, sizeof(int32_t) * (nInc + 1), s));
    CKP(cudaMemsetAsync(dOver, 0, sizeof(int), s));
    const int g = grid_of(total, 256, nsm * 32);
    (k_dof_count<<<g, 256, 0, s>>>(total, dAdr, nInc, dCnt), ::feng::count_launch());
    CKP(cudaGetLastError());
    std::vector<int32_t> cnt((size_t)nInc + 1);
    CKP(cudaMemcpyAsync(cnt.data(), dCnt, sizeof(int32_t) * nInc, cudaMemcpyDeviceToHost, s));
    CKP(cudaStreamSynchronize(s));
    std::vector<int32_t> dptr((size_t)nInc + 1, 0);
    for(int64_t r = 0; r < nInc; ++r) dptr[r + 1] = dptr[r] + cnt[r];
    CKP(cudaMalloc(&dAdj, sizeof(int32_t) * std::max<int32_t>(dptr[nInc], 1)));
    CKP(cudaMemcpyAsync(dPtr, dptr.data(), sizeof(int32_t) * (nInc + 1), cudaMemcpyHostToDevice, s));
    CKP(cudaMemsetAsync(dCnt, 0, sizeof(int32_t) * (nInc + 1), s));
    (k_dof_fill<<<g, 256, 0, s>>>(total, dAdr, nInc, dPtr, dCnt, dAdj), ::feng::count_launch());
    CKP(cudaGetLastError());
    dLen = dCnt;  // reused: row lengths
    const int gr = grid_of(nInc, PAT_WARPS, nsm * 16);
    (k_row_count<<<gr, PAT_WARPS * 32, 0, s>>>(nInc, nl, dAdr, dMask, dPtr, dAdj, dLen, dOver), ::feng::count_launch());
    CKP(cudaGetLastError());
    int over = 0;
    CKP(cudaMemcpyAsync(cnt.data(), dLen, sizeof(int32_t) * nInc, cudaMemcpyDeviceToHost, s));
    CKP(cudaMemcpyAsync(&over, dOver, sizeof(int), cudaMemcpyDeviceToHost, s));
    CKP(cudaStreamSynchronize(s));
    if(over) {
      set_error("device pattern: a row has more than %d candidate columns", PAT_CAP);
      return FE_INVALID_ARG;
    }
    pat = CSRPattern();
    pat.n = nInc;
    pat.ia.assign(nInc + 1, 0);
    for(int64_t r = 0; r < nInc; ++r) pat.ia[r + 1] = pat.ia[r] + cnt[r];
    if(pat.ia[nInc] >= (int64_t)INT32_MAX) {
      set_error("more than 2^31 nonzeros: 32-bit scatter map does not fit");
      return FE_INVALID_ARG;
    }
    CKP(cudaMalloc(&dIa, sizeof(int64_t) * (nInc + 1)));
    CKP(cudaMalloc(&dJa, sizeof(int32_t) * std::max<int64_t>(pat.ia[nInc], 1)));
    CKP(cudaMemcpyAsync(dIa, pat.ia.data(), sizeof(int64_t) * (nInc + 1), cudaMemcpyHostToDevice, s));
    (k_row_fill<<<gr, PAT_WARPS * 32, 0, s>>>(nInc, nl, dAdr, dMask, dPtr, dAdj, dIa, dJa), ::feng::count_launch());
    CKP(cudaGetLastError());
    pat.ja.resize(pat.ia[nInc]);
    CKP(cudaMemcpyAsync(pat.ja.data(), dJa, sizeof(int32_t) * pat.ia[nInc], cudaMemcpyDeviceToHost, s));
    CKP(cudaStreamSynchronize(s));
    return FE_OK;
  };
  status = run();
  cudaFree(dAdr); cudaFree(dMask); cudaFree(dCnt); cudaFree(dPtr); cudaFree(dAdj); cudaFree(dIa); cudaFree(dJa);
  cudaFree(dOver);
  cudaStreamDestroy(s);
  return status;
}

namespace {
int g_patternMode = -1;  // -1: the device when one is present, 0: host, 1: device
}

int set_pattern_mode(int mode)
{
  if(mode < -1 || mode > 1) {
    set_error("pattern mode must be -1 (auto), 0 (host) or 1 (device)");
    return FE_INVALID_ARG;
  }
  g_patternMode = mode;
  return FE_OK;
}

int pattern_mode() { return g_patternMode; }

int build_csr_pattern_auto(const ElementTables &et, int64_t nInc, CSRPattern &pat, int *onDevice)
{
  int nDev = 0;
  const bool haveDevice = cudaGetDeviceCount(&nDev) == cudaSuccess && nDev > 0;
  if(!haveDevice) cudaGetLastError();  // clear the no-device status
  if(onDevice) *onDevice = 0;
  if(g_patternMode == 0 || (g_patternMode == -1 && !haveDevice)) return build_csr_pattern(et, nInc, pat);
  if(!haveDevice) {
    set_error("device pattern requested but no CUDA device is present");
    return FE_CUDA_FAIL;
  }
  const int s = build_csr_pattern_device(et, nInc, pat);
  if(s == FE_OK) {
    if(onDevice) *onDevice = 1;
    return FE_OK;
  }
  // rows beyond the shared-memory capacity: the host builds the same pattern
  if(s == FE_INVALID_ARG && g_patternMode == -1) return build_csr_pattern(et, nInc, pat);
  return s;
}

}  // namespace feng
