// Device V-cycle of the smoothed-aggregation hierarchy (see fe_amg.h).
// Each level: Chebyshev smoothing on D^-1 A (polynomial, SpMV-only),
// residual, restriction, coarse correction, prolongation, Chebyshev again;
// the coarsest level is a dense inverse applied as a mat-vec.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "fe_amg.h"
#include "fe_common.h"
#include "fe_launch.h"

namespace feng {

#define CKA(x)                                                                         \
  do {                                                                                 \
    cudaError_t _e = (x);                                                              \
    if(_e != cudaSuccess) {                                                            \
      set_error("CUDA error %s at %s:%d", cudaGetErrorString(_e), __FILE__, __LINE__); \
      return FE_CUDA_FAIL;                                                             \
    }                                                                                  \
  } while(0)

namespace {

int grid(int64_t n, int per = 256) { return (int)std::max<int64_t>(1, std::min<int64_t>((n + per - 1) / per, 1 << 20)); }

// Vectors hold NV interleaved components per row (NV = 2: both velocity
// components of a node share one pass over the matrix).
template <typename V, int NV>
struct Vals {
  V v[NV];
};

template <typename V, int NV>
__device__ __forceinline__ Vals<V, NV> ldv(const V *__restrict__ p, int64_t i)
{
  Vals<V, NV> r;
  if constexpr(NV == 2 && sizeof(V) == 4) {
    const float2 t = *reinterpret_cast<const float2 *>(p + 2 * i);
    r.v[0] = t.x;
    r.v[1] = t.y;
  } else if constexpr(NV == 2 && sizeof(V) == 8) {
    const double2 t = *reinterpret_cast<const double2 *>(p + 2 * i);
    r.v[0] = t.x;
    r.v[1] = t.y;
  } else {
#pragma unroll
    for(int c = 0; c < NV; ++c) r.v[c] = p[i * NV + c];
  }
  return r;
}

// Row dot products acc[c] = sum_k a[k] x[ja[k]][c] over LANES lanes per row
// (butterfly reduction: the sums are valid in every lane of the row).  The
// row is walked UNR segments of LANES entries at a time: the column indices
// and values of all UNR segments are loaded first (streaming: each matrix
// entry is used once per product), then the gathers of x.
template <typename V, int LANES, int NV>
__device__ __forceinline__ void row_dot(int32_t beg, int32_t end, int sub, const int32_t *__restrict__ ja,
                                        const V *__restrict__ a, const V *__restrict__ x, V (&acc)[NV])
{
  constexpr int UNR = LANES >= 8 ? 4 : 2;
#pragma unroll
  for(int c = 0; c < NV; ++c) acc[c] = 0;
  for(int32_t k0 = beg + sub; k0 < end; k0 += LANES * UNR) {
    int32_t j[UNR];
    V av[UNR];
#pragma unroll
    for(int u = 0; u < UNR; ++u) {
      const int32_t k = k0 + u * LANES;
      const bool ok = k < end;
      j[u] = ok ? __ldcs(ja + k) : -1;
      av[u] = ok ? __ldcs(a + k) : (V)0;
    }
#pragma unroll
    for(int u = 0; u < UNR; ++u)
      if(j[u] >= 0) {
        const Vals<V, NV> xv = ldv<V, NV>(x, j[u]);
#pragma unroll
        for(int c = 0; c < NV; ++c) acc[c] += av[u] * xv.v[c];
      }
  }
#pragma unroll
  for(int c = 0; c < NV; ++c)
#pragma unroll
    for(int o = LANES / 2; o > 0; o >>= 1) acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], o, LANES);
}

// Lane sums acc[c] = sum_k (a[k] w[ja[k]]) x[ja[k]][c] over the entries
// k = beg + sub, beg + sub + LANES, ... of a row (in that order; no
// reduction across the lanes), walked as row_dot: the column indices and
// values of UNR segments first, then their gathers.
template <typename V, int LANES, int NV>
__device__ __forceinline__ void row_dot_w(int32_t beg, int32_t end, int sub, const int32_t *__restrict__ ja,
                                          const V *__restrict__ a, const V *__restrict__ w,
                                          const V *__restrict__ x, V (&acc)[NV])
{
  constexpr int UNR = LANES >= 8 ? 4 : 2;
#pragma unroll
  for(int c = 0; c < NV; ++c) acc[c] = 0;
  for(int32_t k0 = beg + sub; k0 < end; k0 += LANES * UNR) {
    int32_t j[UNR];
    V av[UNR];
#pragma unroll
    for(int u = 0; u < UNR; ++u) {
      const int32_t k = k0 + u * LANES;
      const bool ok = k < end;
      j[u] = ok ? __ldcs(ja + k) : -1;
      av[u] = ok ? __ldcs(a + k) : (V)0;
    }
#pragma unroll
    for(int u = 0; u < UNR; ++u)
      if(j[u] >= 0) {
        const V ak = av[u] * w[j[u]];
        const Vals<V, NV> xv = ldv<V, NV>(x, j[u]);
#pragma unroll
        for(int c = 0; c < NV; ++c) acc[c] += ak * xv.v[c];
      }
  }
}

// y = A x (MODE 0), y = b - A x (MODE 1), y += A x (MODE 2),
// y = A (b .* x) with b a per-row scale of x (MODE 3), y = b + A x (MODE 4);
// csr_row: the LANES lanes of virtual thread t's row (row t / LANES).
template <typename V, int LANES, int MODE, int NV>
__device__ __forceinline__ void csr_row(int64_t t, int64_t n, const int32_t *__restrict__ ia,
                                        const int32_t *__restrict__ ja, const V *__restrict__ a,
                                        const V *__restrict__ x, const V *__restrict__ b, V *__restrict__ y)
{
  const int64_t row = t / LANES;
  const int sub = (int)(t % LANES);
  const bool live = row < n;
  const int32_t beg = live ? ia[row] : 0, end = live ? ia[row + 1] : 0;
  V acc[NV];
  if(MODE == 3) {
    row_dot_w<V, LANES, NV>(beg, end, sub, ja, a, b, x, acc);
#pragma unroll
    for(int c = 0; c < NV; ++c)
#pragma unroll
      for(int o = LANES / 2; o > 0; o >>= 1) acc[c] += __shfl_down_sync(0xffffffffu, acc[c], o, LANES);
  } else {
    row_dot<V, LANES, NV>(beg, end, sub, ja, a, x, acc);
  }
  if(live && sub == 0) {
#pragma unroll
    for(int c = 0; c < NV; ++c) {
      const int64_t o = row * NV + c;
      if(MODE == 0 || MODE == 3) y[o] = acc[c];
      else if(MODE == 1) y[o] = b[o] - acc[c];
      else if(MODE == 4) y[o] = b[o] + acc[c];
      else y[o] += acc[c];
    }
  }
}

template <typename V, int LANES, int MODE, int NV>
__global__ void __launch_bounds__(256) k_csr(int64_t n, const int32_t *__restrict__ ia,
                                             const int32_t *__restrict__ ja, const V *__restrict__ a,
                                             const V *__restrict__ x, const V *__restrict__ b,
                                             V *__restrict__ y, const int *__restrict__ skip)
{
  FE_PDL_ENTRY();
  if(skip && *skip) return;
  csr_row<V, LANES, MODE, NV>((int64_t)blockIdx.x * blockDim.x + threadIdx.x, n, ia, ja, a, x, b, y);
}

template <typename V, int MODE, int NV>
void csr(int lanes, int64_t n, const int32_t *ia, const int32_t *ja, const V *a, const V *x, const V *b,
         V *y, cudaStream_t s, const int *skip)
{
  const int g = grid(n * lanes);
  if(lanes == 8) ::feng::launch_k(k_csr<V, 8, MODE, NV>, g, 256, 0, s, n, ia, ja, a, x, b, y, skip);
  else if(lanes == 16) ::feng::launch_k(k_csr<V, 16, MODE, NV>, g, 256, 0, s, n, ia, ja, a, x, b, y, skip);
  else ::feng::launch_k(k_csr<V, 4, MODE, NV>, g, 256, 0, s, n, ia, ja, a, x, b, y, skip);
}

// Chebyshev start (x = 0): r = D^-1 b, d = r / theta, x = 0.
template <typename V, int NV>
__global__ void k_cheb_start(int64_t n, const V *__restrict__ dinv, const V *__restrict__ b, V *__restrict__ r,
                             V *__restrict__ d, V *__restrict__ x, V inv_theta, const int *__restrict__ skip)
{
  FE_PDL_ENTRY();
  if(skip && *skip) return;
  for(int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n * NV; i += (int64_t)gridDim.x * blockDim.x) {
    const V ri = dinv[i / NV] * b[i];
    r[i] = ri;
    d[i] = ri * inv_theta;
    x[i] = 0;
  }
}

// Chebyshev start from a nonzero x: r = D^-1 (b - A x), d = r / theta.
template <typename V, int LANES, int NV>
__global__ void __launch_bounds__(256) k_cheb_restart(int64_t n, const int32_t *__restrict__ ia,
                                                      const int32_t *__restrict__ ja, const V *__restrict__ a,
                                                      const V *__restrict__ dinv, const V *__restrict__ b,
                                                      const V *__restrict__ x, V *__restrict__ r,
                                                      V *__restrict__ d, V inv_theta, const int *__restrict__ skip)
{
  FE_PDL_ENTRY();
  if(skip && *skip) return;
  const int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / LANES;
  const int sub = threadIdx.x % LANES;
  const bool live = row < n;
  const int32_t beg = live ? ia[row] : 0, end = live ? ia[row + 1] : 0;
  V acc[NV];
  row_dot<V, LANES, NV>(beg, end, sub, ja, a, x, acc);
  if(live && sub == 0) {
    const V di = dinv[row];
#pragma unroll
    for(int c = 0; c < NV; ++c) {
      const int64_t o = row * NV + c;
      const V ri = di * (b[o] - acc[c]);
      r[o] = ri;
      d[o] = ri * inv_theta;
    }
  }
}

// One Chebyshev step: x += d; r -= D^-1 A d; dn = c1 d + c2 r.
template <typename V, int LANES, int NV>
__global__ void __launch_bounds__(256) k_cheb_step(int64_t n, const int32_t *__restrict__ ia,
                                                   const int32_t *__restrict__ ja, const V *__restrict__ a,
                                                   const V *__restrict__ dinv, const V *__restrict__ d,
                                                   V *__restrict__ dn, V *__restrict__ r,
                                                   V *__restrict__ x, V c1, V c2, const int *__restrict__ skip)
{
  FE_PDL_ENTRY();
  if(skip && *skip) return;
  const int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / LANES;
  const int sub = threadIdx.x % LANES;
  const bool live = row < n;
  const int32_t beg = live ? ia[row] : 0, end = live ? ia[row + 1] : 0;
  V acc[NV];
  row_dot<V, LANES, NV>(beg, end, sub, ja, a, d, acc);
  if(live && sub < NV) {
    // lane c of the row updates component c
    const V dv = dinv[row];
    V ac = acc[0];
#pragma unroll
    for(int c = 1; c < NV; ++c)
      if(sub == c) ac = acc[c];
    const int64_t o = row * NV + sub;
    const V di = d[o];
    x[o] += di;
    const V ri = r[o] - dv * ac;
    r[o] = ri;
    dn[o] = c1 * di + c2 * ri;
  }
}

// Start from x = 0 fused with the first step: with d = D^-1 b / theta
// (formed on the fly for the neighbours), x = d, r = D^-1 b - D^-1 A d,
// dn = c1 d + c2 r.
template <typename V, int LANES, int NV>
__device__ __forceinline__ void cheb_first_row(int64_t t, int64_t n, const int32_t *__restrict__ ia,
                                               const int32_t *__restrict__ ja, const V *__restrict__ a,
                                               const V *__restrict__ dinv, const V *__restrict__ b,
                                               V *__restrict__ dn, V *__restrict__ r, V *__restrict__ x,
                                               V inv_theta, V c1, V c2)
{
  const int64_t row = t / LANES;
  const int sub = (int)(t % LANES);
  const bool live = row < n;
  const int32_t beg = live ? ia[row] : 0, end = live ? ia[row + 1] : 0;
  V acc[NV];
  row_dot_w<V, LANES, NV>(beg, end, sub, ja, a, dinv, b, acc);
#pragma unroll
  for(int c = 0; c < NV; ++c)
#pragma unroll
    for(int o = LANES / 2; o > 0; o >>= 1) acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], o, LANES);
  if(live && sub < NV) {
    const V dv = dinv[row];
    V ac = acc[0];
#pragma unroll
    for(int c = 1; c < NV; ++c)
      if(sub == c) ac = acc[c];
    const int64_t o = row * NV + sub;
    const V r0 = dv * b[o];
    const V di = r0 * inv_theta;
    x[o] = di;
    const V ri = r0 - dv * ac * inv_theta;
    r[o] = ri;
    dn[o] = c1 * di + c2 * ri;
  }
}

template <typename V, int LANES, int NV>
__global__ void __launch_bounds__(256) k_cheb_first(int64_t n, const int32_t *__restrict__ ia,
                                                    const int32_t *__restrict__ ja, const V *__restrict__ a,
                                                    const V *__restrict__ dinv, const V *__restrict__ b,
                                                    V *__restrict__ dn, V *__restrict__ r, V *__restrict__ x,
                                                    V inv_theta, V c1, V c2, const int *__restrict__ skip)
{
  FE_PDL_ENTRY();
  if(skip && *skip) return;
  cheb_first_row<V, LANES, NV>((int64_t)blockIdx.x * blockDim.x + threadIdx.x, n, ia, ja, a, dinv, b, dn, r, x,
                               inv_theta, c1, c2);
}

// Degree-1 post-smoothing from the prolongated y = x + P xc:
// x = y + D^-1 (b - A y) / theta (x and y distinct).
// OUT (the finest level of a paired V-cycle whose result goes straight to
// the caller's vector): component c of row i is written, times *scale, to
// out[dof[c][i]] instead of x.
template <typename V, int LANES, int NV, bool OUT>
__device__ __forceinline__ void cheb_post_row(int64_t t, int64_t n, const int32_t *__restrict__ ia,
                                              const int32_t *__restrict__ ja, const V *__restrict__ a,
                                              const V *__restrict__ dinv, const V *__restrict__ b,
                                              const V *__restrict__ y, V *__restrict__ x, V inv_theta,
                                              const int32_t *__restrict__ dofX, const int32_t *__restrict__ dofY,
                                              const double *__restrict__ scale, V *__restrict__ out)
{
  const int64_t row = t / LANES;
  const int sub = (int)(t % LANES);
  const bool live = row < n;
  const int32_t beg = live ? ia[row] : 0, end = live ? ia[row + 1] : 0;
  V acc[NV];
  row_dot<V, LANES, NV>(beg, end, sub, ja, a, y, acc);
  if(live && sub < NV) {
    V ac = acc[0];
#pragma unroll
    for(int c = 1; c < NV; ++c)
      if(sub == c) ac = acc[c];
    const int64_t o = row * NV + sub;
    const V ri = dinv[row] * (b[o] - ac);
    const V xo = y[o] + ri * inv_theta;
    if(OUT) out[sub == 0 ? dofX[row] : dofY[row]] = xo * (V)*scale;
    else x[o] = xo;
  }
}

template <typename V, int LANES, int NV, bool OUT>
__global__ void __launch_bounds__(256) k_cheb_post(int64_t n, const int32_t *__restrict__ ia,
                                                   const int32_t *__restrict__ ja, const V *__restrict__ a,
                                                   const V *__restrict__ dinv, const V *__restrict__ b,
                                                   const V *__restrict__ y, V *__restrict__ x, V inv_theta,
                                                   const int *__restrict__ skip, const int32_t *__restrict__ dofX,
                                                   const int32_t *__restrict__ dofY, const double *__restrict__ scale,
                                                   V *__restrict__ out)
{
  FE_PDL_ENTRY();
  if(skip && *skip) return;
  cheb_post_row<V, LANES, NV, OUT>((int64_t)blockIdx.x * blockDim.x + threadIdx.x, n, ia, ja, a, dinv, b, y, x,
                                   inv_theta, dofX, dofY, scale, out);
}

// Walks the len entries of row lane of a sliced-ELL slice (entry k at
// base + 32 k + lane) in order, calling f(column, value) for each, in steps
// of UNR entries, software-pipelined: the next step's columns and values are
// loaded before this step's gathers, so a step waits for one memory latency
// instead of two.
template <int UNR, typename V, typename F>
__device__ __forceinline__ void sell_walk(int32_t base, int32_t len, int lane, const int32_t *__restrict__ sc,
                                          const V *__restrict__ sv, F &&f)
{
  int32_t c[UNR];
  V a[UNR];
#pragma unroll
  for(int u = 0; u < UNR; ++u) {
    const bool ok = u < len;
    const int32_t e = base + (u << 5) + lane;
    c[u] = ok ? __ldcs(sc + e) : -1;
    a[u] = ok ? __ldcs(sv + e) : (V)0;
  }
  for(int32_t k = 0; k < len; k += UNR) {
    int32_t cn[UNR];
    V an[UNR];
#pragma unroll
    for(int u = 0; u < UNR; ++u) {
      const bool ok = k + UNR + u < len;
      const int32_t e = base + ((k + UNR + u) << 5) + lane;
      cn[u] = ok ? __ldcs(sc + e) : -1;
      an[u] = ok ? __ldcs(sv + e) : (V)0;
    }
#pragma unroll
    for(int u = 0; u < UNR; ++u)
      if(c[u] >= 0) f(c[u], a[u]);
#pragma unroll
    for(int u = 0; u < UNR; ++u) {
      c[u] = cn[u];
      a[u] = an[u];
    }
  }
}

// k_cheb_first on the sliced-ELL copy of A: thread = row, both components.
template <typename V, int NV>
__global__ void __launch_bounds__(256) k_cheb_first_sell(int64_t n, const int32_t *__restrict__ sp,
                                                         const int32_t *__restrict__ sc, const V *__restrict__ sv,
                                                         const V *__restrict__ dinv, const V *__restrict__ b,
                                                         V *__restrict__ dn, V *__restrict__ r, V *__restrict__ x,
                                                         V inv_theta, V c1, V c2, const int *__restrict__ skip)
{
  FE_PDL_ENTRY();
  if(skip && *skip) return;
  const int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if(row >= n) return;
  const int64_t sl = row >> 5;
  const int lane = (int)(row & 31);
  const int32_t base = sp[sl], len = (sp[sl + 1] - base) >> 5;
  V acc[NV];
#pragma unroll
  for(int c = 0; c < NV; ++c) acc[c] = 0;
  sell_walk<8, V>(base, len, lane, sc, sv, [&](int32_t j, V a) {
    const V ak = a * dinv[j];
    const Vals<V, NV> bv = ldv<V, NV>(b, j);
#pragma unroll
    for(int c = 0; c < NV; ++c) acc[c] += ak * bv.v[c];
  });
  const V dv = dinv[row];
#pragma unroll
  for(int c = 0; c < NV; ++c) {
    const int64_t o = row * NV + c;
    const V r0 = dv * b[o];
    const V di = r0 * inv_theta;
    x[o] = di;
    const V ri = r0 - dv * acc[c] * inv_theta;
    r[o] = ri;
    dn[o] = c1 * di + c2 * ri;
  }
}

// k_cheb_post on the sliced-ELL copy of A: thread = row, both components.
template <typename V, int NV, bool OUT>
__global__ void __launch_bounds__(256) k_cheb_post_sell(int64_t n, const int32_t *__restrict__ sp,
                                                        const int32_t *__restrict__ sc, const V *__restrict__ sv,
                                                        const V *__restrict__ dinv, const V *__restrict__ b,
                                                        const V *__restrict__ y, V *__restrict__ x, V inv_theta,
                                                        const int *__restrict__ skip, AMGDevice::OutMap om)
{
  FE_PDL_ENTRY();
  if(skip && *skip) return;
  int64_t blk = blockIdx.x;
  if constexpr(OUT) {
    // the pressure rows of the folded saddle-point preconditioner in the
    // leading blocks (scheduled first, overlapping the rows)
    const int64_t pBlocks = om.bgu ? (om.nP + 255) / 256 : 0;
    if(blk < pBlocks) {
      const int64_t k = blk * 256 + threadIdx.x;
      if(k >= om.nP) return;
      const double c = *om.cr, cSc = om.consts[1], cMc = om.consts[2];
      const double shift = cMc > 0 ? c / cMc : 0., lift = cSc != 0. ? c / cSc : 0.;
      const int32_t i = om.pRows[k];
      const double rp = (double)((const V *)om.r)[i] - shift * om.pMass[k];
      ((V *)om.z)[i] = (V)((double)((const V *)om.pScale)[k] * rp + lift);
      return;
    }
    blk -= pBlocks;
  }
  const int64_t row = blk * blockDim.x + threadIdx.x;
  if(row >= n) return;
  const int64_t sl = row >> 5;
  const int lane = (int)(row & 31);
  const int32_t base = sp[sl], len = (sp[sl + 1] - base) >> 5;
  V acc[NV];
#pragma unroll
  for(int c = 0; c < NV; ++c) acc[c] = 0;
  sell_walk<8, V>(base, len, lane, sc, sv, [&](int32_t j, V ak) {
    const Vals<V, NV> yv = ldv<V, NV>(y, j);
#pragma unroll
    for(int c = 0; c < NV; ++c) acc[c] += ak * yv.v[c];
  });
  const V dv = dinv[row];
  V cf = 0;
  if constexpr(OUT)
    if(om.bgu) cf = (V)*om.cr;
#pragma unroll
  for(int c = 0; c < NV; ++c) {
    const int64_t o = row * NV + c;
    const V ri = dv * (b[o] - acc[c]);
    const V xo = y[o] + ri * inv_theta;
    if constexpr(OUT) {
      const V xf = om.bgu ? xo - cf * ((const V *)om.bgu)[o] : xo;
      ((V *)om.z)[c == 0 ? om.dofX[row] : om.dofY[row]] = xf * (V)*om.scale;
    } else {
      x[o] = xo;
    }
  }
}

// y = b + P xc on the sliced-ELL copy of P (thread = fine row).
template <typename V, int NV>
__global__ void __launch_bounds__(256) k_prolong_sell(int64_t n, const int32_t *__restrict__ sp,
                                                      const int32_t *__restrict__ sc, const V *__restrict__ sv,
                                                      const V *__restrict__ xc, const V *__restrict__ b,
                                                      V *__restrict__ y, const int *__restrict__ skip)
{
  FE_PDL_ENTRY();
  if(skip && *skip) return;
  const int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if(row >= n) return;
  const int64_t sl = row >> 5;
  const int lane = (int)(row & 31);
  const int32_t base = sp[sl], len = (sp[sl + 1] - base) >> 5;
  V acc[NV];
#pragma unroll
  for(int c = 0; c < NV; ++c) acc[c] = 0;
  sell_walk<8, V>(base, len, lane, sc, sv, [&](int32_t j, V a) {
    const Vals<V, NV> xv = ldv<V, NV>(xc, j);
#pragma unroll
    for(int c = 0; c < NV; ++c) acc[c] += a * xv.v[c];
  });
#pragma unroll
  for(int c = 0; c < NV; ++c) y[row * NV + c] = b[row * NV + c] + acc[c];
}

// Last step of a smoothing whose residual is not needed afterwards: x += d
// only (the step's product with A would be discarded).
template <typename V>
__global__ void k_cheb_last(int64_t m, const V *__restrict__ d, V *__restrict__ x, const int *__restrict__ skip)
{
  FE_PDL_ENTRY();
  if(skip && *skip) return;
  for(int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x)
    x[i] += d[i];
}

// x = Minv b for the coarsest level (dense, row-major): one block of
// DENSE_T threads per row, so that every load of the row is in flight at
// once; warp sums, then the warps' sums in order (deterministic).
constexpr int DENSE_T = 128;
template <typename V, int NV>
__global__ void __launch_bounds__(DENSE_T) k_dense(int64_t n, const V *__restrict__ M, const V *__restrict__ b,
                                                   V *__restrict__ x, const int *__restrict__ skip)
{
  FE_PDL_ENTRY();
  if(skip && *skip) return;
  __shared__ V red[DENSE_T / 32][NV];
  const int64_t row = blockIdx.x;
  V acc[NV];
#pragma unroll
  for(int c = 0; c < NV; ++c) acc[c] = 0;
#pragma unroll 4
  for(int64_t k = threadIdx.x; k < n; k += DENSE_T) {
    const V m = M[row * n + k];
#pragma unroll
    for(int c = 0; c < NV; ++c) acc[c] += m * b[k * NV + c];
  }
#pragma unroll
  for(int c = 0; c < NV; ++c) {
    for(int o = 16; o > 0; o >>= 1) acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], o);
    if((threadIdx.x & 31) == 0) red[threadIdx.x >> 5][c] = acc[c];
  }
  __syncthreads();
  if(threadIdx.x < NV) {
    V t = red[0][threadIdx.x];
#pragma unroll
    for(int w = 1; w < DENSE_T / 32; ++w) t += red[w][threadIdx.x];
    x[row * NV + threadIdx.x] = t;
  }
}

template <typename V>
int upload_vec(void **dst, const std::vector<double> &src)
{
  std::vector<V> tmp(src.begin(), src.end());
  CKA(cudaMalloc(dst, sizeof(V) * std::max<size_t>(1, tmp.size())));
  CKA(cudaMemcpy(*dst, tmp.data(), sizeof(V) * tmp.size(), cudaMemcpyHostToDevice));
  return FE_OK;
}

int upload_idx(int32_t **dst, const std::vector<int64_t> &src)
{
  std::vector<int32_t> tmp(src.begin(), src.end());
  CKA(cudaMalloc(dst, sizeof(int32_t) * std::max<size_t>(1, tmp.size())));
  CKA(cudaMemcpy(*dst, tmp.data(), sizeof(int32_t) * tmp.size(), cudaMemcpyHostToDevice));
  return FE_OK;
}

int upload_idx(int32_t **dst, const std::vector<int32_t> &src)
{
  CKA(cudaMalloc(dst, sizeof(int32_t) * std::max<size_t>(1, src.size())));
  CKA(cudaMemcpy(*dst, src.data(), sizeof(int32_t) * src.size(), cudaMemcpyHostToDevice));
  return FE_OK;
}

// The sliced-ELL copy of A (AMGDevice::Lev::sellPtr).
template <typename V>
int upload_sell(const HostCSR &A, int32_t **sellPtr, int32_t **sellCol, void **sellVal)
{
  const int64_t n = A.n, ns = (n + 31) / 32;
  const int64_t mcols = A.m > 0 ? A.m : n;
  std::vector<int32_t> ptr(ns + 1, 0);
  for(int64_t sl = 0; sl < ns; ++sl) {
    int64_t len = 0;
    for(int64_t r = sl * 32; r < std::min<int64_t>(n, sl * 32 + 32); ++r) len = std::max<int64_t>(len, A.ia[r + 1] - A.ia[r]);
    if(ptr[sl] + 32 * len >= (int64_t)INT32_MAX) return FE_OK;  // keep the CSR kernels
    ptr[sl + 1] = (int32_t)(ptr[sl] + 32 * len);
  }
  std::vector<int32_t> col(std::max<int32_t>(ptr[ns], 1));
  std::vector<V> val(col.size(), (V)0);
  for(int64_t sl = 0; sl < ns; ++sl) {
    const int32_t len = (ptr[sl + 1] - ptr[sl]) / 32;
    for(int lane = 0; lane < 32; ++lane) {
      const int64_t r = sl * 32 + lane;
      for(int32_t k = 0; k < len; ++k) {
        const int64_t e = ptr[sl] + (int64_t)k * 32 + lane;
        const int64_t src = r < n ? A.ia[r] + k : -1;
        if(r < n && src < A.ia[r + 1]) {
          col[e] = (int32_t)A.ja[src];
          val[e] = (V)A.a[src];
        } else {
          col[e] = (int32_t)std::min<int64_t>(r, mcols - 1);  // padding: value 0 on an existing column
          val[e] = (V)0;
        }
      }
    }
  }
  CKA(cudaMalloc(sellPtr, sizeof(int32_t) * ptr.size()));
  CKA(cudaMalloc(sellCol, sizeof(int32_t) * col.size()));
  CKA(cudaMalloc(sellVal, sizeof(V) * val.size()));
  CKA(cudaMemcpy(*sellPtr, ptr.data(), sizeof(int32_t) * ptr.size(), cudaMemcpyHostToDevice));
  CKA(cudaMemcpy(*sellCol, col.data(), sizeof(int32_t) * col.size(), cudaMemcpyHostToDevice));
  CKA(cudaMemcpy(*sellVal, val.data(), sizeof(V) * val.size(), cudaMemcpyHostToDevice));
  return FE_OK;
}

int lanes_for(const HostCSR &M)
{
  const double avg = M.n ? (double)M.nnz() / M.n : 0;
  // 4 lanes per row on the P2 stiffness (~11 entries per row): 21 us per
  // finest smoother step against 27 us with 8 lanes
  return avg > 24 ? 16 : avg > 12 ? 8 : 4;
}

}  // namespace

AMGDevice::~AMGDevice()
{
  for(Lev &L : lv_) {
    cudaFree(L.Aia); cudaFree(L.Aja); cudaFree(L.Pia); cudaFree(L.Pja); cudaFree(L.Ria); cudaFree(L.Rja);
    cudaFree(L.Aa); cudaFree(L.Pa); cudaFree(L.Ra); cudaFree(L.dinv); cudaFree(L.diag);
    cudaFree(L.x); cudaFree(L.b); cudaFree(L.r); cudaFree(L.d0); cudaFree(L.d1);
    cudaFree(L.sellPtr); cudaFree(L.sellCol); cudaFree(L.sellVal);
    cudaFree(L.sellPPtr); cudaFree(L.sellPCol); cudaFree(L.sellPVal);
  }
  cudaFree(coarseInv_);
}

int AMGDevice::upload(const AMGHierarchy &H, const AMGParams &p, int fp32, cudaStream_t s)
{
  p_ = p;
  fp32_ = fp32;
  s_ = s;
  const size_t vs = fp32 ? sizeof(float) : sizeof(double);
  lv_.resize(H.levels.size());
  n0_ = H.levels.empty() ? 0 : H.levels[0].A.n;
  diagSum_ = 0;
  for(int64_t i = 0; i < n0_; ++i) diagSum_ += 1.0 / H.levels[0].dinv[i];
  for(size_t l = 0; l < H.levels.size(); ++l) {
    const AMGLevel &h = H.levels[l];
    Lev &L = lv_[l];
    L.n = h.A.n;
    L.lmax = h.lmax;
    L.lanesA = lanes_for(h.A);
    FE_TRY(upload_idx(&L.Aia, h.A.ia));
    FE_TRY(upload_idx(&L.Aja, h.A.ja));
    FE_TRY(fp32 ? upload_vec<float>(&L.Aa, h.A.a) : upload_vec<double>(&L.Aa, h.A.a));
    if(l == 0 && h.A.n >= 32 * 152)
      FE_TRY(fp32 ? upload_sell<float>(h.A, &L.sellPtr, &L.sellCol, &L.sellVal)
                  : upload_sell<double>(h.A, &L.sellPtr, &L.sellCol, &L.sellVal));
    FE_TRY(fp32 ? upload_vec<float>(&L.dinv, h.dinv) : upload_vec<double>(&L.dinv, h.dinv));
    std::vector<double> dg(h.dinv.size());
    for(size_t i = 0; i < dg.size(); ++i) dg[i] = 1.0 / h.dinv[i];
    FE_TRY(fp32 ? upload_vec<float>(&L.diag, dg) : upload_vec<double>(&L.diag, dg));
    // room for two interleaved components (vcycle2)
    // room for up to three interleaved components per row
    for(void **v : {&L.x, &L.b, &L.r, &L.d0, &L.d1}) CKA(cudaMalloc(v, 3 * vs * std::max<int64_t>(1, L.n)));
    if(l + 1 < H.levels.size()) {
      L.nc = h.P.m;
      L.lanesP = lanes_for(h.P);
      L.lanesR = lanes_for(h.R);
      FE_TRY(upload_idx(&L.Pia, h.P.ia));
      FE_TRY(upload_idx(&L.Pja, h.P.ja));
      FE_TRY(fp32 ? upload_vec<float>(&L.Pa, h.P.a) : upload_vec<double>(&L.Pa, h.P.a));
      if(l == 0 && h.P.n >= 32 * 152)
        FE_TRY(fp32 ? upload_sell<float>(h.P, &L.sellPPtr, &L.sellPCol, &L.sellPVal)
                    : upload_sell<double>(h.P, &L.sellPPtr, &L.sellPCol, &L.sellPVal));
      FE_TRY(upload_idx(&L.Ria, h.R.ia));
      FE_TRY(upload_idx(&L.Rja, h.R.ja));
      FE_TRY(fp32 ? upload_vec<float>(&L.Ra, h.R.a) : upload_vec<double>(&L.Ra, h.R.a));
    }
  }
  nCoarse_ = lv_.empty() ? 0 : lv_.back().n;
  nnz0_ = H.levels.empty() ? 0 : H.levels[0].A.nnz();
  FE_TRY(fp32 ? upload_vec<float>(&coarseInv_, H.coarseInv) : upload_vec<double>(&coarseInv_, H.coarseInv));
  return FE_OK;
}

// needResidual: r = D^-1 (b - A x) must hold for the final x (the
// pre-smoothing, whose residual is restricted); otherwise the last step only
// moves x.
template <typename V, int NV>
static void chebyshev(int lanes, int64_t n, const int32_t *ia, const int32_t *ja, const V *a, const int32_t *sp,
                      const int32_t *sc, const V *sv, const V *dinv, const V *b, V *x, V *r, V *d0, V *d1,
                      double lmax, const AMGParams &p, bool zeroStart, bool needResidual, cudaStream_t s,
                      const int *skip)
{
  // Chebyshev iteration on D^-1 A over [low, high] * lmax (Saad, Alg. 12.1).
  const double lo = p.chebyLow * lmax, hi = p.chebyHigh * lmax;
  const double theta = 0.5 * (hi + lo), delta = 0.5 * (hi - lo), sigma = theta / delta;
  double rho = 1.0 / sigma;
  const int g = grid(n * lanes);
  int k0 = 0;
  V *d = d0, *dn = d1;
  if(zeroStart && (needResidual || p.chebyDegree > 1)) {
    // start + first step in one pass
    const double rhoN = 1.0 / (2.0 * sigma - rho);
    const V c1 = (V)(rhoN * rho), c2 = (V)(2.0 * rhoN / delta);
    const V it = (V)(1.0 / theta);
    if(sp) ::feng::launch_k(k_cheb_first_sell<V, NV>, grid(n), 256, 0, s, n, sp, sc, sv, dinv, b, dn, r, x, it, c1, c2, skip);
    else if(lanes == 16) ::feng::launch_k(k_cheb_first<V, 16, NV>, g, 256, 0, s, n, ia, ja, a, dinv, b, dn, r, x, it, c1, c2, skip);
    else if(lanes == 8) ::feng::launch_k(k_cheb_first<V, 8, NV>, g, 256, 0, s, n, ia, ja, a, dinv, b, dn, r, x, it, c1, c2, skip);
    else ::feng::launch_k(k_cheb_first<V, 4, NV>, g, 256, 0, s, n, ia, ja, a, dinv, b, dn, r, x, it, c1, c2, skip);
    rho = rhoN;
    std::swap(d, dn);
    k0 = 1;
  } else if(zeroStart) {
    ::feng::launch_k(k_cheb_start<V, NV>, grid(n * NV), 256, 0, s, n, dinv, b, r, d0, x, (V)(1.0 / theta), skip);
  } else {
    if(lanes == 16) ::feng::launch_k(k_cheb_restart<V, 16, NV>, g, 256, 0, s, n, ia, ja, a, dinv, b, x, r, d0, (V)(1.0 / theta), skip);
    else if(lanes == 8) ::feng::launch_k(k_cheb_restart<V, 8, NV>, g, 256, 0, s, n, ia, ja, a, dinv, b, x, r, d0, (V)(1.0 / theta), skip);
    else ::feng::launch_k(k_cheb_restart<V, 4, NV>, g, 256, 0, s, n, ia, ja, a, dinv, b, x, r, d0, (V)(1.0 / theta), skip);
  }
  for(int k = k0; k < p.chebyDegree; ++k) {
    if(!needResidual && k == p.chebyDegree - 1) {
      ::feng::launch_k(k_cheb_last<V>, grid(n * NV), 256, 0, s, n * NV, d, x, skip);
      break;
    }
    const double rhoN = 1.0 / (2.0 * sigma - rho);
    const V c1 = (V)(rhoN * rho), c2 = (V)(2.0 * rhoN / delta);
    if(lanes == 16) ::feng::launch_k(k_cheb_step<V, 16, NV>, g, 256, 0, s, n, ia, ja, a, dinv, d, dn, r, x, c1, c2, skip);
    else if(lanes == 8) ::feng::launch_k(k_cheb_step<V, 8, NV>, g, 256, 0, s, n, ia, ja, a, dinv, d, dn, r, x, c1, c2, skip);
    else ::feng::launch_k(k_cheb_step<V, 4, NV>, g, 256, 0, s, n, ia, ja, a, dinv, d, dn, r, x, c1, c2, skip);
    rho = rhoN;
    std::swap(d, dn);
  }
}

template <typename V, int NV>
void AMGDevice::vcycle_t(int l, const V *b, V *x)
{
  Lev &L = lv_[l];
  if(l == (int)lv_.size() - 1) {
    if(L.n > 0) ::feng::launch_k(k_dense<V, NV>, (int)L.n, DENSE_T, 0, s_, L.n, (const V *)coarseInv_, b, x, skip_);
    return;
  }
  Lev &C = lv_[l + 1];
  const V *A = (const V *)L.Aa;
  chebyshev<V, NV>(L.lanesA, L.n, L.Aia, L.Aja, A, L.sellPtr, L.sellCol, (const V *)L.sellVal, (const V *)L.dinv, b,
                   x, (V *)L.r, (V *)L.d0, (V *)L.d1, L.lmax, p_, true, true, s_, skip_);
  // Chebyshev keeps r = D^-1 (b - A x): restrict the residual D r directly
  // (no extra pass over A).
  csr<V, 3, NV>(L.lanesR, C.n, L.Ria, L.Rja, (const V *)L.Ra, (const V *)L.r, (const V *)L.diag, (V *)C.b, s_,
                skip_);
  vcycle_t<V, NV>(l + 1, (const V *)C.b, (V *)C.x);
  if(p_.chebyDegree == 1) {
    // y = x + P xc into this level's free scratch, then one pass
    // x = y + D^-1 (b - A y) / theta (the restart and the step in one)
    V *y = (V *)L.d1;
    if(L.sellPPtr)
      ::feng::launch_k(k_prolong_sell<V, NV>, grid(L.n), 256, 0, s_, L.n, L.sellPPtr, L.sellPCol, (const V *)L.sellPVal,
                                                        (const V *)C.x, x, y, skip_);
    else
      csr<V, 4, NV>(L.lanesP, L.n, L.Pia, L.Pja, (const V *)L.Pa, (const V *)C.x, x, y, s_, skip_);
    const double lo = p_.chebyLow * L.lmax, hi = p_.chebyHigh * L.lmax, theta = 0.5 * (hi + lo);
    const V it = (V)(1.0 / theta);
    const int g = grid(L.n * L.lanesA);
    const V *dinv = (const V *)L.dinv;
    if(L.sellPtr) {
      const V *sv = (const V *)L.sellVal;
      if(l == 0 && NV == 2 && out_.z) {
        const int extra = out_.bgu ? (int)((out_.nP + 255) / 256) : 0;
        ::feng::launch_k(k_cheb_post_sell<V, NV, true>, grid(L.n) + extra, 256, 0, s_, L.n, L.sellPtr, L.sellCol, sv, dinv,
                         b, y, x, it, skip_, out_);
        outWritten_ = true;
      } else {
        ::feng::launch_k(k_cheb_post_sell<V, NV, false>, grid(L.n), 256, 0, s_, L.n, L.sellPtr, L.sellCol, sv, dinv, b, y, x, it,
                         skip_, AMGDevice::OutMap());
      }
      return;
    }
    if(l == 0 && NV == 2 && out_.z) {
      const int32_t *dx = out_.dofX, *dy = out_.dofY;
      const double *sc = out_.scale;
      V *z = (V *)out_.z;
      if(L.lanesA == 16) ::feng::launch_k(k_cheb_post<V, 16, NV, true>, g, 256, 0, s_, L.n, L.Aia, L.Aja, A, dinv, b, y, x, it, skip_, dx, dy, sc, z);
      else if(L.lanesA == 8) ::feng::launch_k(k_cheb_post<V, 8, NV, true>, g, 256, 0, s_, L.n, L.Aia, L.Aja, A, dinv, b, y, x, it, skip_, dx, dy, sc, z);
      else ::feng::launch_k(k_cheb_post<V, 4, NV, true>, g, 256, 0, s_, L.n, L.Aia, L.Aja, A, dinv, b, y, x, it, skip_, dx, dy, sc, z);
      outWritten_ = true;
      return;
    }
    if(L.lanesA == 16) ::feng::launch_k(k_cheb_post<V, 16, NV, false>, g, 256, 0, s_, L.n, L.Aia, L.Aja, A, dinv, b, y, x, it, skip_, nullptr, nullptr, nullptr, nullptr);
    else if(L.lanesA == 8) ::feng::launch_k(k_cheb_post<V, 8, NV, false>, g, 256, 0, s_, L.n, L.Aia, L.Aja, A, dinv, b, y, x, it, skip_, nullptr, nullptr, nullptr, nullptr);
    else ::feng::launch_k(k_cheb_post<V, 4, NV, false>, g, 256, 0, s_, L.n, L.Aia, L.Aja, A, dinv, b, y, x, it, skip_, nullptr, nullptr, nullptr, nullptr);
    return;
  }
  csr<V, 2, NV>(L.lanesP, L.n, L.Pia, L.Pja, (const V *)L.Pa, (const V *)C.x, nullptr, x, s_, skip_);
  chebyshev<V, NV>(L.lanesA, L.n, L.Aia, L.Aja, A, L.sellPtr, L.sellCol, (const V *)L.sellVal, (const V *)L.dinv, b,
                   x, (V *)L.r, (V *)L.d0, (V *)L.d1, L.lmax, p_, false, false, s_, skip_);
}

void AMGDevice::vcycle64(const double *b, double *x) { vcycle_t<double, 1>(0, b, x); }
void AMGDevice::vcycle32(const float *b, float *x) { vcycle_t<float, 1>(0, b, x); }
bool AMGDevice::vcycle2_64(const double *b, double *x, const OutMap *om)
{
  out_ = om ? *om : OutMap();
  outWritten_ = false;
  vcycle_t<double, 2>(0, b, x);
  out_ = OutMap();
  return outWritten_;
}

bool AMGDevice::vcycle2_32(const float *b, float *x, const OutMap *om)
{
  out_ = om ? *om : OutMap();
  outWritten_ = false;
  vcycle_t<float, 2>(0, b, x);
  out_ = OutMap();
  return outWritten_;
}

void AMGDevice::vcycle3_64(const double *b, double *x)
{
  out_ = OutMap();
  vcycle_t<double, 3>(0, b, x);
}

void AMGDevice::vcycle3_32(const float *b, float *x)
{
  out_ = OutMap();
  vcycle_t<float, 3>(0, b, x);
}

void AMGDevice::fineStep2()
{
  // The finest-level pre-smoothing pass of a V-cycle (k_cheb_first) on the
  // level's scratch vectors: b = d0 (finite values of earlier cycles), x, r,
  // dn = d1 written.
  const Lev &L = lv_[0];
  const int g = grid(L.n * L.lanesA);
  auto go = [&](auto tag) {
    using V = decltype(tag);
    const V *a = (const V *)L.Aa, *dinv = (const V *)L.dinv, *b = (const V *)L.d0;
    V *dn = (V *)L.d1, *r = (V *)L.r, *x = (V *)L.x;
    const V it = (V)0.5, c1 = (V)0.5, c2 = (V)0.5;
    if(L.sellPtr)
      ::feng::launch_k(k_cheb_first_sell<V, 2>, grid(L.n), 256, 0, s_, L.n, L.sellPtr, L.sellCol, (const V *)L.sellVal, dinv, b, dn,
                                                          r, x, it, c1, c2, skip_);
    else if(L.lanesA == 16) ::feng::launch_k(k_cheb_first<V, 16, 2>, g, 256, 0, s_, L.n, L.Aia, L.Aja, a, dinv, b, dn, r, x, it, c1, c2, skip_);
    else if(L.lanesA == 8) ::feng::launch_k(k_cheb_first<V, 8, 2>, g, 256, 0, s_, L.n, L.Aia, L.Aja, a, dinv, b, dn, r, x, it, c1, c2, skip_);
    else ::feng::launch_k(k_cheb_first<V, 4, 2>, g, 256, 0, s_, L.n, L.Aia, L.Aja, a, dinv, b, dn, r, x, it, c1, c2, skip_);
  };
  if(fp32_) go(float());
  else go(double());
}

int64_t AMGDevice::fineStep2Bytes() const
{
  if(lv_.empty()) return 0;
  const Lev &L = lv_[0];
  const int64_t vs = fp32_ ? 4 : 8;
  // values + columns, row pointers, dinv, and per component: b read, x, r,
  // dn written
  return nnz0_ * (vs + 4) + (L.n + 1) * 4 + L.n * vs + 2 * L.n * vs * 4;
}

void AMGDevice::spmv64(const double *x, double *y)
{
  const Lev &L = lv_[0];
  csr<double, 0, 1>(L.lanesA, L.n, L.Aia, L.Aja, (const double *)L.Aa, x, nullptr, y, s_, skip_);
}

void AMGDevice::spmv32(const float *x, float *y)
{
  const Lev &L = lv_[0];
  csr<float, 0, 1>(L.lanesA, L.n, L.Aia, L.Aja, (const float *)L.Aa, x, nullptr, y, s_, skip_);
}

}  // namespace feng
