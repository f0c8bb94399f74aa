#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "fe_common.h"
#include "fe_df.h"
#include "fe_launch.h"
#include "fe_krylov.h"

namespace feng {

#define CK(x)                                                                          \
  do {                                                                                 \
    cudaError_t _e = (x);                                                              \
    if(_e != cudaSuccess) {                                                            \
      set_error("CUDA error %s at %s:%d", cudaGetErrorString(_e), __FILE__, __LINE__); \
      return FE_CUDA_FAIL;                                                             \
    }                                                                                  \
  } while(0)

namespace {

constexpr int RB = 256;        // threads per reduction block
constexpr int MAXRED = 1024;   // maximum number of reduction blocks
constexpr int MAXM = 128;      // maximum restart length

// ---------------------------------------------------------------------------
// SpMV: y = A x (or y = b - A x), LANES consecutive lanes per row.
// ---------------------------------------------------------------------------
template <typename VA, typename VX, typename VY, typename ACC, int LANES, bool RESID>
__global__ void __launch_bounds__(256) k_spmv(int64_t n, const int32_t *__restrict__ ia,
                                              const int32_t *__restrict__ ja,
                                              const VA *__restrict__ a, const VX *__restrict__ x,
                                              const double *__restrict__ b, VY *__restrict__ y,
                                              const int *__restrict__ done)
{
  FE_PDL_ENTRY();
  if(done && *done) return;
  const int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / LANES;
  const int sub = threadIdx.x % LANES;
  // Rows past n keep their lanes alive (zero work) so the shuffles below
  // always run with the full warp.
  const bool live = row < n;
  const int32_t beg = live ? ia[row] : 0, end = live ? ia[row + 1] : 0;
  // UNR segments of LANES entries per step: the column indices and values
  // (streamed, used once) are loaded before the gathers of x.
  constexpr int UNR = LANES >= 8 ? 4 : 2;
  ACC acc = 0;
  for(int32_t k0 = beg + sub; k0 < end; k0 += LANES * UNR) {
    int32_t j[UNR];
    VA av[UNR];
#pragma unroll
    for(int u = 0; u < UNR; ++u) {
      const int32_t k = k0 + u * LANES;
      const bool ok = k < end;
      j[u] = ok ? __ldcs(ja + k) : -1;
      av[u] = ok ? __ldcs(a + k) : (VA)0;
    }
#pragma unroll
    for(int u = 0; u < UNR; ++u)
      if(j[u] >= 0) acc += (ACC)av[u] * (ACC)x[j[u]];
  }
#pragma unroll
  for(int o = LANES / 2; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o, LANES);
  if(live && sub == 0) {
    if(RESID) y[row] = (VY)(b[row] - (double)acc);
    else y[row] = (VY)acc;
  }
}

// ---------------------------------------------------------------------------
// Reductions with in-kernel finalisation: every block writes a partial, the
// last block to finish sums the partials in block order (deterministic).
// ---------------------------------------------------------------------------
struct RedState {
  unsigned int counter;
  float finv;   // 1 / ||w|| of the last FP32 Gram-Schmidt norm pass
  int reorth;   // the last Gram-Schmidt pass asks for a second one
  double result[4];
};

__device__ double block_sum(double v, double *sh)
{
  for(int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x / 32, l = threadIdx.x % 32;
  if(l == 0) sh[w] = v;
  __syncthreads();
  v = 0;
  if(threadIdx.x < blockDim.x / 32) v = sh[threadIdx.x];
  if(w == 0)
    for(int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  __syncthreads();
  return v;  // valid in thread 0
}

__device__ double block_max(double v, double *sh)
{
  for(int o = 16; o > 0; o >>= 1) v = nan_max(v, __shfl_down_sync(0xffffffffu, v, o));
  const int w = threadIdx.x / 32, l = threadIdx.x % 32;
  if(l == 0) sh[w] = v;
  __syncthreads();
  v = 0;
  if(threadIdx.x < blockDim.x / 32) v = sh[threadIdx.x];
  if(w == 0)
    for(int o = 16; o > 0; o >>= 1) v = nan_max(v, __shfl_down_sync(0xffffffffu, v, o));
  __syncthreads();
  return v;
}

// Finishes a reduction of K values: writes partials, last block sums them.
template <int K, bool MAX>
__device__ void finish_reduction(const double (&v)[K], double *partials, RedState *st,
                                 double *out)
{
  __shared__ double sh[RB / 32];
  __shared__ bool last;
  double tot[K];
#pragma unroll
  for(int k = 0; k < K; ++k) tot[k] = MAX ? block_max(v[k], sh) : block_sum(v[k], sh);
  if(threadIdx.x == 0) {
#pragma unroll
    for(int k = 0; k < K; ++k) partials[k * MAXRED + blockIdx.x] = tot[k];
    __threadfence();
    unsigned int prev = atomicAdd(&st->counter, 1u);
    last = (prev == gridDim.x - 1);
  }
  __syncthreads();
  if(!last) return;
  __threadfence();
#pragma unroll
  for(int k = 0; k < K; ++k) {
    // L2-coherent loads (the partials come from other blocks), independent
    // so that they overlap.
    double s = 0.;
    for(int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) {
      const double p = __ldcg(partials + k * MAXRED + i);
      s = MAX ? nan_max(s, p) : s + p;
    }
    s = MAX ? block_max(s, sh) : block_sum(s, sh);
    if(threadIdx.x == 0) {
      st->result[k] = s;
      if(out) out[k] = s;
    }
  }
  if(threadIdx.x == 0) st->counter = 0;
}

__global__ void k_dot(int64_t n, const double *__restrict__ x, const double *__restrict__ y,
                      double *partials, RedState *st, double *out)
{
  FE_PDL_ENTRY();
  double v[1] = {0.};
  for(int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
      i += (int64_t)gridDim.x * blockDim.x)
    v[0] += x[i] * y[i];
  finish_reduction<1, false>(v, partials, st, out);
}

__global__ void k_absmax(int64_t n, const double *__restrict__ x, double *partials, RedState *st,
                         double *out)
{
  FE_PDL_ENTRY();
  double v[1] = {0.};
  for(int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
      i += (int64_t)gridDim.x * blockDim.x)
    v[0] = nan_max(v[0], fabs(x[i]));
  finish_reduction<1, true>(v, partials, st, out);
}

// h[c] (+)= V_c . w for c < ncols; grid (parts, ncols).  Partials per column.
__global__ void k_mdot_partial(int64_t n, const double *__restrict__ V, int ncols,
                               const double *__restrict__ w, double *partials,
                               const int *__restrict__ done)
{
  FE_PDL_ENTRY();
  if(*done) return;
  __shared__ double sh[RB / 32];
  const int c = blockIdx.y;
  const double *vc = V + (int64_t)c * n;
  double v = 0.;
  for(int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
      i += (int64_t)gridDim.x * blockDim.x)
    v += vc[i] * w[i];
  v = block_sum(v, sh);
  if(threadIdx.x == 0) partials[(int64_t)c * MAXRED + blockIdx.x] = v;
}

// Sums the partials of each column c (block c) into hcol[c] (and H column).
__global__ void k_mdot_final(int nparts, double *partials, double *hcur, double *Hcol, int accum,
                             const int *__restrict__ done)
{
  FE_PDL_ENTRY();
  if(*done) return;
  __shared__ double sh[RB / 32];
  const int c = blockIdx.x;
  double s = 0.;
  for(int i = threadIdx.x; i < nparts; i += blockDim.x) s += partials[(int64_t)c * MAXRED + i];
  s = block_sum(s, sh);
  if(threadIdx.x == 0) {
    hcur[c] = s;
    Hcol[c] = accum ? Hcol[c] + s : s;
  }
}

// w -= sum_c h[c] V_c
__global__ void k_mupdate(int64_t n, const double *__restrict__ V, int ncols,
                          const double *__restrict__ h, double *__restrict__ w,
                          const int *__restrict__ done)
{
  FE_PDL_ENTRY();
  if(*done) return;
  __shared__ double sh[MAXM + 1];
  for(int c = threadIdx.x; c < ncols; c += blockDim.x) sh[c] = h[c];
  __syncthreads();
  for(int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
      i += (int64_t)gridDim.x * blockDim.x) {
    double acc = w[i];
    for(int c = 0; c < ncols; ++c) acc -= sh[c] * V[(int64_t)c * n + i];
    w[i] = acc;
  }
}

// Sum of squares of w into st->result[0] (k_scale_from takes the root).
__global__ void k_norm_to(int64_t n, const double *__restrict__ w, double *partials, RedState *st,
                          const int *__restrict__ done)
{
  FE_PDL_ENTRY();
  if(*done) return;
  double v[1] = {0.};
  for(int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
      i += (int64_t)gridDim.x * blockDim.x)
    v[0] += w[i] * w[i];
  finish_reduction<1, false>(v, partials, st, nullptr);
}

// v = w / sqrt(ss), and H[j+1][j] = sqrt(ss).  ss read from st->result[0].
__global__ void k_scale_from(int64_t n, const double *__restrict__ w, double *__restrict__ v,
                             const RedState *st, double *Hsub, const int *__restrict__ done)
{
  FE_PDL_ENTRY();
  if(*done) return;
  const double nrm = sqrt(st->result[0]);
  if(blockIdx.x == 0 && threadIdx.x == 0) *Hsub = nrm;
  const double inv = nrm > 0 ? 1.0 / nrm : 0.0;
  for(int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
      i += (int64_t)gridDim.x * blockDim.x)
    v[i] = w[i] * inv;
}

template <typename VO>
__global__ void k_scale_vec(int64_t n, const double *__restrict__ w, VO *__restrict__ v,
                            const double *__restrict__ s, int invert)
{
  FE_PDL_ENTRY();
  const double f = invert ? (*s > 0 ? 1.0 / *s : 0.0) : *s;
  for(int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
      i += (int64_t)gridDim.x * blockDim.x)
    v[i] = (VO)(w[i] * f);
}

__global__ void k_to_f32(int64_t n, const double *__restrict__ x, float *__restrict__ y,
                         const int *__restrict__ done)
{
  FE_PDL_ENTRY();
  if(done && *done) return;
  for(int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
      i += (int64_t)gridDim.x * blockDim.x)
    y[i] = (float)x[i];
}

// Givens rotations on Hessenberg column j (device, one thread).  H is stored
// column-major with leading dimension MAXM+1.
struct GmresHead {
  int done;       // set once the estimate reaches tol or on breakdown
  int k;          // number of basis vectors in use
  double est;     // |g[k]|: residual norm estimate
  double tol;
  double beta;    // ||r|| at the start of the cycle
};
struct GmresState : GmresHead {
  double H[MAXM * (MAXM + 1)];
  double cs[MAXM], sn[MAXM], g[MAXM + 1], y[MAXM];
  double hcur[MAXM + 1];
};

// One warp: the column and the previous rotations are staged in shared
// memory, the (inherently sequential) rotation chain runs on lane 0 out of
// registers and shared memory, and the column is written back by the warp.
// Applies the previous rotations to Hessenberg column j, forms rotation j,
// updates g and the residual estimate, sets done (one warp; sh, scs, ssn:
// shared arrays of MAXM + 1, MAXM, MAXM doubles).
__device__ void givens_warp(GmresState *gs, int j, int lane, double *sh, double *scs, double *ssn)
{
  double *h = gs->H + (int64_t)j * (MAXM + 1);
  for(int i = lane; i <= j + 1; i += 32) sh[i] = h[i];
  for(int i = lane; i < j; i += 32) {
    scs[i] = gs->cs[i];
    ssn[i] = gs->sn[i];
  }
  __syncwarp();
  // The chain t_0 = h_0, t_{i+1} = -s_i t_i + c_i h_{i+1}, h_i <- c_i t_i +
  // s_i h_{i+1}, h_j <- t_j is an affine recurrence: lane l composes the
  // maps t -> -s_i t + c_i h_{i+1} of its GCH consecutive rotations, a warp
  // scan composes the lanes' maps (Hillis-Steele, five shuffle rounds), and
  // each lane replays its rotations from its start value: ~25 dependent FP64
  // operations instead of two per rotation in sequence.
  {
    constexpr int GCH = (MAXM + 31) / 32;
    const int i0 = lane * GCH;
    const double h0 = sh[0];
    double cv[GCH], sv[GCH], hv[GCH];
    double A = 1., B = 0.;  // the lane's map t -> A t + B
#pragma unroll
    for(int u = 0; u < GCH; ++u) {
      const bool ok = i0 + u < j;
      cv[u] = ok ? scs[i0 + u] : 1.;
      sv[u] = ok ? ssn[i0 + u] : 0.;
      hv[u] = ok ? sh[i0 + u + 1] : 0.;
      if(ok) {
        const double al = -sv[u], be = cv[u] * hv[u];
        A = al * A;
        B = al * B + be;
      }
    }
    // inclusive scan: (A, B) <- (A, B) o (lane - off's map)
#pragma unroll
    for(int off = 1; off < 32; off <<= 1) {
      const double Ap = __shfl_up_sync(0xffffffffu, A, off), Bp = __shfl_up_sync(0xffffffffu, B, off);
      if(lane >= off) {
        B = A * Bp + B;
        A = A * Ap;
      }
    }
    // exclusive: the composition of the lanes before this one
    double Ae = __shfl_up_sync(0xffffffffu, A, 1), Be = __shfl_up_sync(0xffffffffu, B, 1);
    if(lane == 0) {
      Ae = 1.;
      Be = 0.;
    }
    __syncwarp();  // every read of sh before the writes below
    double t = Ae * h0 + Be;
#pragma unroll
    for(int u = 0; u < GCH; ++u)
      if(i0 + u < j) {
        sh[i0 + u] = cv[u] * t + sv[u] * hv[u];
        t = -sv[u] * t + cv[u] * hv[u];
        if(i0 + u == j - 1) sh[j] = t;
      }
  }
  __syncwarp();
  for(int i = lane; i < j; i += 32) h[i] = sh[i];
  if(lane != 0) return;
  const double a = sh[j], b = sh[j + 1];
  const double r = hypot(a, b);
  double c = 1., s = 0.;
  if(r > 0) { c = a / r; s = b / r; }
  gs->cs[j] = c;
  gs->sn[j] = s;
  h[j] = r;
  h[j + 1] = 0.;
  gs->g[j + 1] = -s * gs->g[j];
  gs->g[j] = c * gs->g[j];
  gs->k = j + 1;
  gs->est = fabs(gs->g[j + 1]);
  if(!(gs->est > gs->tol) || b == 0.0 || !isfinite(gs->est)) gs->done = 1;
}

__global__ void k_givens(GmresState *gs, int j)
{
  FE_PDL_ENTRY();
  if(gs->done) return;
  __shared__ double sh[MAXM + 1], scs[MAXM], ssn[MAXM];
  givens_warp(gs, j, threadIdx.x, sh, scs, ssn);
}

// y = R^-1 g with R the upper triangle of H (k x k), by columns: the block
// stages R in shared memory (all loads in flight at once), then one warp
// sweeps c = k-1 .. 0: the lane holding row c divides, broadcasts y_c, and
// every lane subtracts column c times y_c from its rows above c (lane l
// holds rows l, l + 32, ...; fixed order, deterministic).
__global__ void k_backsolve(GmresState *gs)
{
  FE_PDL_ENTRY();
  // dynamic: the column-major upper triangle of the restart length m
  // (m (m + 1) / 2 doubles), sized at launch
  extern __shared__ double sR[];
  const int k = gs->k;
  auto idx = [](int i, int c) { return c * (c + 1) / 2 + i; };  // i <= c
  for(int e = threadIdx.x; e < k * k; e += blockDim.x) {
    const int c = e / k, i = e - c * k;
    if(i <= c) sR[idx(i, c)] = gs->H[(int64_t)c * (MAXM + 1) + i];
  }
  __syncthreads();
  if(threadIdx.x >= 32) return;
  const int lane = threadIdx.x;
  constexpr int RPL = MAXM / 32;  // rows per lane
  double s[RPL];
#pragma unroll
  for(int t = 0; t < RPL; ++t) s[t] = lane + 32 * t < k ? gs->g[lane + 32 * t] : 0.;
  for(int c = k - 1; c >= 0; --c) {
    const int owner = c & 31, tc = c >> 5;
    double sc = 0.;
#pragma unroll
    for(int t = 0; t < RPL; ++t)
      if(t == tc) sc = s[t];
    double yc = 0.;
    if(lane == owner) {
      const double d = sR[idx(c, c)];
      yc = d != 0 ? sc / d : 0.;
      gs->y[c] = yc;
    }
    yc = __shfl_sync(0xffffffffu, yc, owner);
#pragma unroll
    for(int t = 0; t < RPL; ++t) {
      const int i = lane + 32 * t;
      if(i < c) s[t] -= sR[idx(i, c)] * yc;
    }
  }
}

// x += Z y.  FP64 basis: FP64 products and sums.  FP32 basis (mixed path):
// the products and the running sum in double-float on the FP32 pipes (the
// FP64 pipe of the GB300 would bound the pass at ~50 us for 50 columns of
// 588 k rows; double-float keeps it at the bytes), added to x in FP64.
template <typename VZ>
__global__ void k_xupdate(int64_t n, int64_t ld, const VZ *__restrict__ Z, const GmresState *gs,
                          double *__restrict__ x)
{
  FE_PDL_ENTRY();
  const int k = gs->k;
  if constexpr(sizeof(VZ) == 8) {
    __shared__ double sy[MAXM];
    for(int c = threadIdx.x; c < k; c += blockDim.x) sy[c] = gs->y[c];
    __syncthreads();
    for(int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
        i += (int64_t)gridDim.x * blockDim.x) {
      double acc = x[i];
      for(int c = 0; c < k; ++c) acc += sy[c] * (double)Z[(int64_t)c * ld + i];
      x[i] = acc;
    }
  } else {
    __shared__ dfl sy[MAXM];
    for(int c = threadIdx.x; c < k; c += blockDim.x) sy[c] = df_from(gs->y[c]);
    __syncthreads();
    constexpr int U = 8;
    for(int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
        i += (int64_t)gridDim.x * blockDim.x) {
      dfl acc = df_zero();
      for(int c0 = 0; c0 < k; c0 += U) {
        float z[U];
#pragma unroll
        for(int u = 0; u < U; ++u) z[u] = c0 + u < k ? (float)Z[(int64_t)(c0 + u) * ld + i] : 0.f;
#pragma unroll
        for(int u = 0; u < U; ++u)
          if(c0 + u < k) {
            const dfl y = sy[c0 + u];
            const float p = __fmul_rn(z[u], y.hi);
            float e = __fmaf_rn(z[u], y.hi, -p);
            e = __fmaf_rn(z[u], y.lo, e);
            acc = df_add(acc, df_fast2(p, e));
          }
      }
      x[i] += df_to(acc);
    }
  }
}

// ---------------------------------------------------------------------------
// Classical Gram-Schmidt passes on the FP32 Krylov basis of the mixed cycle
// (V column-major with leading dimension n, columns c < ncols <= CMAX):
//   MODE 0: h_c = V_c . w
//   MODE 1: w -= V hprev, then h_c = V_c . w   (the second CGS pass)
//   MODE 2: w -= V hprev, then ss = w . w
// One read of V and w per pass, FP32 products, per-block partial sums in
// FP64; the last block sums the partials in block order (deterministic) and
// writes hcur / Hcol (MODE 0: Hcol = h, MODE 1: Hcol += h) or ss into
// st->result[0].  The FP64 pipe of the GB300 is too slow for these loops.
// ---------------------------------------------------------------------------

// The FP32 Arnoldi basis of the mixed path is stored in row blocks of VBLK
// rows: column c of row block k at V + (k m1 + c) VBLK (m1 = restart + 1
// columns per block), so that a block of threads streaming several columns
// over the same rows reads one contiguous region.  vidx4: the float4 index
// of float4 row g (rows 4g..4g+3) of column c.
constexpr int VBLK = 1024;
__host__ __device__ __forceinline__ int64_t vidx4(int64_t g, int c, int m1)
{
  return ((g >> 8) * m1 + c) * (VBLK / 4) + (g & (VBLK / 4 - 1));
}

// A second read of a line this thread has just read (served by L1): a
// separate load, so that the compiler does not keep the first read in
// registers (which costs occupancy).
__device__ __forceinline__ float4 ld4_l1(const float4 *p)
{
  float4 r;
  asm volatile("ld.global.ca.v4.f32 {%0, %1, %2, %3}, [%4];" : "=f"(r.x), "=f"(r.y), "=f"(r.z), "=f"(r.w) : "l"(p));
  return r;
}

template <int CMAX, int MODE>
__global__ void __launch_bounds__(RB, 3) k_gs32(int64_t n4, int m1, const float *__restrict__ V, int ncols,
                                             const double *__restrict__ hprev, float *__restrict__ w,
                                             double *partials, RedState *st, double *hcur, double *Hcol,
                                             const int *__restrict__ done, int pass)
{
  FE_PDL_ENTRY();
  // Rows are taken four at a time (16-byte loads); the basis is in row
  // blocks (vidx4) and rows n..ld-1 hold zeros.
  // MODE 2, pass 0: decides whether a second pass is needed (the update kept
  // less than a tenth of ||w||, i.e. severe cancellation: the test of
  // Daniel, Gragg, Kaufman and Stewart with eta = 0.1; ||w||^2 from the dot
  // pass); pass 1 runs only when it was asked for.
  if(*done || (MODE == 2 && pass == 1 && !st->reorth)) return;
  constexpr int NACC = MODE == 2 ? 1 : CMAX;
  __shared__ float hs[CMAX];
  __shared__ float red[RB / 32][NACC];
  __shared__ bool last;
  if(MODE > 0) {
    for(int c = threadIdx.x; c < CMAX; c += RB) hs[c] = c < ncols ? (float)hprev[c] : 0.f;
    __syncthreads();
  }
  float acc[NACC];
#pragma unroll
  for(int c = 0; c < NACC; ++c) acc[c] = 0.f;
  float4 *w4 = reinterpret_cast<float4 *>(w);
  for(int64_t g = (int64_t)blockIdx.x * RB + threadIdx.x; g < n4; g += (int64_t)gridDim.x * RB) {
    float4 wv = w4[g];
    if(MODE > 0) {
#pragma unroll
      for(int c = 0; c < CMAX; ++c)
        if(c < ncols) {
          const float4 v = reinterpret_cast<const float4 *>(V)[vidx4(g, c, m1)];
          const float h = hs[c];
          wv.x = fmaf(-h, v.x, wv.x);
          wv.y = fmaf(-h, v.y, wv.y);
          wv.z = fmaf(-h, v.z, wv.z);
          wv.w = fmaf(-h, v.w, wv.w);
        }
      w4[g] = wv;
    }
    if(MODE < 2) {
      // (MODE 1 reads the columns again: the same lines, from L1.)
#pragma unroll
      for(int c = 0; c < CMAX; ++c)
        if(c < ncols) {
          const float4 *pv = reinterpret_cast<const float4 *>(V) + vidx4(g, c, m1);
          const float4 v = MODE == 1 ? ld4_l1(pv) : *pv;
          acc[c] = fmaf(v.x, wv.x, fmaf(v.y, wv.y, fmaf(v.z, wv.z, fmaf(v.w, wv.w, acc[c]))));
        }
    } else {
      acc[0] = fmaf(wv.x, wv.x, fmaf(wv.y, wv.y, fmaf(wv.z, wv.z, fmaf(wv.w, wv.w, acc[0]))));
    }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nr = MODE == 2 ? 1 : ncols;
#pragma unroll
  for(int c = 0; c < NACC; ++c) {
    if(c < nr) {
      float v = acc[c];
      for(int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if(lane == 0) red[warp][c] = v;
    }
  }
  __syncthreads();
  for(int c = threadIdx.x; c < nr; c += RB) {
    double sum = 0.;
    for(int k = 0; k < RB / 32; ++k) sum += (double)red[k][c];
    partials[(int64_t)c * MAXRED + blockIdx.x] = sum;
    __threadfence();
  }
  __syncthreads();
  if(threadIdx.x == 0) last = atomicAdd(&st->counter, 1u) == gridDim.x - 1;
  __syncthreads();
  if(!last) return;
  __threadfence();
  for(int c = warp; c < nr; c += RB / 32) {
    // L2-coherent loads (written by other blocks), eight independent chains.
    const double *pc = partials + (int64_t)c * MAXRED;
    double s8[8] = {0., 0., 0., 0., 0., 0., 0., 0.};
    const int nb = (int)gridDim.x;
    for(int b0 = lane; b0 < nb; b0 += 256) {
      double v[8];
#pragma unroll
      for(int q = 0; q < 8; ++q) v[q] = __ldcg(pc + (b0 + 32 * q < nb ? b0 + 32 * q : 0));
#pragma unroll
      for(int q = 0; q < 8; ++q) s8[q] += b0 + 32 * q < nb ? v[q] : 0.;
    }
    double sum = ((s8[0] + s8[1]) + (s8[2] + s8[3])) + ((s8[4] + s8[5]) + (s8[6] + s8[7]));
    for(int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    if(lane == 0) {
      if(MODE == 2) {
        // ||w||: H[j+1][j] (through Hcol) and the FP32 scale of the next basis vector.
        const double nrm = sqrt(sum);
        st->result[0] = sum;
        *Hcol = nrm;
        st->finv = nrm > 0 ? (float)(1.0 / nrm) : 0.f;
        if(pass == 0) st->reorth = sum < 1e-2 * st->result[2] ? 1 : 0;
      } else {
        hcur[c] = sum;
        Hcol[c] = MODE == 0 ? sum : Hcol[c] + sum;
      }
    }
  }
  __syncthreads();
  if(threadIdx.x == 0) st->counter = 0;
}

// h_c = V_c . w for c < ncols and ||w||^2.  Grid: x = blocks of rows (each
// thread takes groups of 4 rows, two groups per step, grid-stride), y =
// groups of eight columns, so every thread keeps eight FP32 accumulators and
// issues its sixteen basis loads together; the ||w||^2 column belongs to y = 0.  Per warp a butterfly
// sums the eight accumulators over the lanes (the last three steps as a
// reduce-scatter: lane l ends with column l % 8), the warps are summed in
// FP64, one partial per row block and column; the last block sums the
// partials in row-block order.
// pyth (first pass only): the last block also forms ||w - V h||^2 =
// ||w||^2 - ||h||^2 (Pythagoras, V orthonormal) and, unless that kept less
// than a hundredth of ||w||^2 (severe cancellation: the
// Daniel-Gragg-Kaufman-Stewart test with eta = 0.1), takes it as the norm of
// the update: H[j+1][j] = its root (through Hcol[ncols]), st->finv its
// inverse; otherwise st->reorth asks for the second pass.
// second = 1: the reorthogonalisation pass, run only when it was asked for;
// its coefficients are added to the Hessenberg column.
__global__ void __launch_bounds__(RB) k_gs_dots(int64_t n4, int m1, const float *__restrict__ V, int ncols,
                                                const float *__restrict__ w, double *partials, RedState *st,
                                                double *hcur, double *Hcol, const int *__restrict__ done,
                                                int second, int pyth)
{
  FE_PDL_ENTRY();
  if(*done || (second && !st->reorth)) return;
  __shared__ float red[RB / 32][9];
  __shared__ double hsum[MAXM + 1];
  __shared__ bool last;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int c0 = blockIdx.y * 8;
  const bool wcol = blockIdx.y == 0;
  float acc[8];
#pragma unroll
  for(int u = 0; u < 8; ++u) acc[u] = 0.f;
  float wq = 0.f;
  const float4 *w4 = reinterpret_cast<const float4 *>(w);
  const float4 *V4 = reinterpret_cast<const float4 *>(V);
  const int64_t stride = (int64_t)gridDim.x * RB;
  for(int64_t g = (int64_t)blockIdx.x * RB + threadIdx.x; g < n4; g += 2 * stride) {
    const int64_t g2 = g + stride;
    const bool two = g2 < n4;
    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 x = w4[g];
    const float4 x2 = two ? w4[g2] : z4;
    if(wcol) {
      wq = fmaf(x.x, x.x, fmaf(x.y, x.y, fmaf(x.z, x.z, fmaf(x.w, x.w, wq))));
      wq = fmaf(x2.x, x2.x, fmaf(x2.y, x2.y, fmaf(x2.z, x2.z, fmaf(x2.w, x2.w, wq))));
    }
    float4 v[8], v2[8];
#pragma unroll
    for(int u = 0; u < 8; ++u) {
      v[u] = c0 + u < ncols ? __ldcs(V4 + vidx4(g, c0 + u, m1)) : z4;
      v2[u] = (two && c0 + u < ncols) ? __ldcs(V4 + vidx4(g2, c0 + u, m1)) : z4;
    }
#pragma unroll
    for(int u = 0; u < 8; ++u) {
      acc[u] = fmaf(v[u].x, x.x, fmaf(v[u].y, x.y, fmaf(v[u].z, x.z, fmaf(v[u].w, x.w, acc[u]))));
      acc[u] = fmaf(v2[u].x, x2.x, fmaf(v2[u].y, x2.y, fmaf(v2[u].z, x2.z, fmaf(v2[u].w, x2.w, acc[u]))));
    }
  }
  // lanes l, l^8, l^16, l^24 first, then a reduce-scatter over the low bits
#pragma unroll
  for(int h = 16; h >= 8; h >>= 1)
#pragma unroll
    for(int u = 0; u < 8; ++u) acc[u] += __shfl_xor_sync(0xffffffffu, acc[u], h);
#pragma unroll
  for(int h = 4; h > 0; h >>= 1) {
    const bool hi = lane & h;
#pragma unroll
    for(int i = 0; i < h; ++i) {
      const float keep = hi ? acc[i + h] : acc[i];
      const float send = hi ? acc[i] : acc[i + h];
      acc[i] = keep + __shfl_xor_sync(0xffffffffu, send, h);
    }
  }
  for(int o = 16; o > 0; o >>= 1) wq += __shfl_xor_sync(0xffffffffu, wq, o);
  if(lane < 8) red[warp][lane] = acc[0];
  if(lane == 0) red[warp][8] = wq;
  __syncthreads();
  if(threadIdx.x < 9) {
    const int t = threadIdx.x;
    const int col = t < 8 ? c0 + t : ncols;
    if((t < 8 && col < ncols) || (t == 8 && wcol)) {
      double sum = 0.;
      for(int k = 0; k < RB / 32; ++k) sum += (double)red[k][t];
      partials[(int64_t)col * MAXRED + blockIdx.x] = sum;
    }
    // only the threads that wrote partials order them before the counter
    __threadfence();
  }
  __syncthreads();
  if(threadIdx.x == 0) last = atomicAdd(&st->counter, 1u) == gridDim.x * gridDim.y - 1;
  __syncthreads();
  if(!last) return;
  __threadfence();
  for(int c = warp; c <= ncols; c += RB / 32) {
    const double *pc = partials + (int64_t)c * MAXRED;
    double s8[8] = {0., 0., 0., 0., 0., 0., 0., 0.};
    const int nb = (int)gridDim.x;
    for(int b0 = lane; b0 < nb; b0 += 256) {
      double v[8];
#pragma unroll
      for(int q = 0; q < 8; ++q) v[q] = __ldcg(pc + (b0 + 32 * q < nb ? b0 + 32 * q : 0));
#pragma unroll
      for(int q = 0; q < 8; ++q) s8[q] += b0 + 32 * q < nb ? v[q] : 0.;
    }
    double sum = ((s8[0] + s8[1]) + (s8[2] + s8[3])) + ((s8[4] + s8[5]) + (s8[6] + s8[7]));
    for(int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    if(lane == 0) {
      hsum[c] = sum;
      if(c == ncols) {
        st->result[2] = sum;
      } else {
        hcur[c] = sum;
        Hcol[c] = second ? Hcol[c] + sum : sum;
      }
    }
  }
  __syncthreads();
  if(threadIdx.x == 0) {
    st->counter = 0;
    if(pyth && !second) {
      const double ww = hsum[ncols];
      double hh = 0.;
      for(int c = 0; c < ncols; ++c) hh += hsum[c] * hsum[c];
      const double est = ww - hh;
      if(est > 1e-2 * ww) {
        const double nrm = sqrt(est);
        Hcol[ncols] = nrm;
        st->finv = (float)(1.0 / nrm);
        st->reorth = 0;
      } else {
        st->reorth = 1;
      }
    }
  }
}

// h_c = V_c . w for c < ncols and ||w||^2 in one pass over w and the
// columns, shaped as the update pass: thread = one float4 row of w at a
// time (grid-stride over one wave of blocks), the columns in batches of 8
// loads, CMAX FP32 accumulators per thread (64 registers: four blocks per
// SM): block (x, y) takes the columns CMAX y .. CMAX y + CMAX - 1 (more than
// 16 columns: grid y > 1, each slice re-reading w).  Per block each accumulator is summed over the lanes
// (butterfly) and the warps (FP64, warp order) into one partial per row
// block x and column (||w||^2: column ncols, from y = 0); the last block to
// finish sums the partials (RB / (ncols + 1) threads per column, each over a
// fixed stride of row blocks in rounds of 32 loads, then in thread order)
// into hcur / Hcol (second = 0: Hcol = h; 1: the reorthogonalisation pass,
// run only when it was asked for, adds h to Hcol) and st->result[2].
// gridDim.x <= MAXRED.
template <int CMAX>
__global__ void __launch_bounds__(RB, 4) k_gs_dots_all(int64_t n4, int m1, const float *__restrict__ V,
                                                      int ncols, const float *__restrict__ w, double *partials,
                                                      RedState *st, double *hcur, double *Hcol,
                                                      const int *__restrict__ done, int second)
{
  FE_PDL_ENTRY();
  if(*done || (second && !st->reorth)) return;
  __shared__ double red[RB / 32][CMAX + 1];
  __shared__ double flat[RB];
  __shared__ bool last;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int cb = CMAX * blockIdx.y, cn = min(CMAX, ncols - cb);
  const bool wcol = blockIdx.y == 0;
  const float4 *w4 = reinterpret_cast<const float4 *>(w);
  const float4 *V4 = reinterpret_cast<const float4 *>(V);
  float acc[CMAX];
#pragma unroll
  for(int c = 0; c < CMAX; ++c) acc[c] = 0.f;
  float wq = 0.f;
  for(int64_t g = (int64_t)blockIdx.x * RB + tid; g < n4; g += (int64_t)gridDim.x * RB) {
    const float4 x = w4[g];
    if(wcol) wq = fmaf(x.x, x.x, fmaf(x.y, x.y, fmaf(x.z, x.z, fmaf(x.w, x.w, wq))));
#pragma unroll
    for(int c0 = 0; c0 < CMAX; c0 += 8) {
      if(c0 < cn) {
        // one batch of eight loads in flight (clamped columns, the extra
        // products dropped by selects)
        float4 v[8];
#pragma unroll
        for(int u = 0; u < 8; ++u) v[u] = __ldcs(V4 + vidx4(g, cb + (c0 + u < cn ? c0 + u : c0), m1));
#pragma unroll
        for(int u = 0; u < 8; ++u) {
          const float t = fmaf(v[u].x, x.x, fmaf(v[u].y, x.y, fmaf(v[u].z, x.z, v[u].w * x.w)));
          acc[c0 + u] += c0 + u < cn ? t : 0.f;
        }
      }
    }
  }
#pragma unroll
  for(int c = 0; c < CMAX; ++c) {
    if(c < cn) {
      float t = acc[c];
      for(int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
      if(lane == 0) red[warp][c] = (double)t;
    }
  }
  for(int o = 16; o > 0; o >>= 1) wq += __shfl_xor_sync(0xffffffffu, wq, o);
  if(lane == 0) red[warp][CMAX] = (double)wq;
  __syncthreads();
  if(tid < cn || (wcol && tid == CMAX)) {
    const int col = tid < cn ? cb + tid : ncols;
    double sum = 0.;
    for(int k = 0; k < RB / 32; ++k) sum += red[k][tid];
    partials[(int64_t)col * MAXRED + blockIdx.x] = sum;
    // only the threads that wrote partials order them before the counter
    __threadfence();
  }
  __syncthreads();
  if(tid == 0) last = atomicAdd(&st->counter, 1u) == gridDim.x * gridDim.y - 1;
  __syncthreads();
  if(!last) return;
  __threadfence();
  const int nc = ncols + 1, T = max(1, RB / nc), nb = (int)gridDim.x;
  const int c = tid / T, s = tid - c * T;
  double part = 0.;
  if(c < nc) {
    const double *pc = partials + (int64_t)c * MAXRED;
    double v4[4] = {0., 0., 0., 0.};
    for(int k0 = 0; s + T * k0 < nb; k0 += 24) {
      // straight-line loads (indices clamped into the array, the extra ones
      // zeroed by selects), so that all 24 are in flight at once
      double v[24];
#pragma unroll
      for(int k = 0; k < 24; ++k) {
        const int b = s + T * (k0 + k);
        v[k] = __ldcg(pc + (b < nb ? b : 0));
      }
#pragma unroll
      for(int k = 0; k < 24; ++k) v4[k & 3] += s + T * (k0 + k) < nb ? v[k] : 0.;
    }
    part = (v4[0] + v4[1]) + (v4[2] + v4[3]);
  }
  flat[tid] = part;
  __syncthreads();
  if(tid < nc) {
    double sum = 0.;
    for(int k = 0; k < T; ++k) sum += flat[tid * T + k];
    if(tid == ncols) {
      st->result[2] = sum;
    } else {
      hcur[tid] = sum;
      Hcol[tid] = second ? Hcol[tid] + sum : sum;
    }
  }
  if(tid == 0) st->counter = 0;
}

// The update pass w - V h over c < ncols.
// NORM: the result goes back to w and its squared norm is reduced (one FP64
// partial per block, the last block sums them in block order): H[j+1][j] =
// the norm (through Hnext), st->finv its inverse; on the first pass
// (second = 0) st->reorth asks for a second pass when the update kept less
// than a tenth of ||w|| (||w||^2 in st->result[2] from the dot pass); the
// second pass runs only when it was asked for.
// !NORM (after a dot pass that took the norm by Pythagoras): unless a second
// pass was asked for, the result times st->finv is the next basis vector
// (column ncols of the row-blocked basis, and its contiguous copy vcopy, the
// preconditioner's next input); otherwise it goes back to w.
template <int CMAX, bool NORM>
__global__ void __launch_bounds__(RB, 4) k_gs_upd(int64_t n4, int m1, float *__restrict__ V, int ncols,
                                                  const double *__restrict__ hprev, float *__restrict__ w,
                                                  float *__restrict__ vcopy, RedState *st, double *partials,
                                                  double *Hnext, const int *__restrict__ done, int second)
{
  FE_PDL_ENTRY();
  if(*done || (NORM && second && !st->reorth)) return;
  __shared__ float hs[CMAX];
  __shared__ double wred[RB / 32];
  __shared__ bool last;
  for(int c = threadIdx.x; c < CMAX; c += RB) hs[c] = c < ncols ? (float)hprev[c] : 0.f;
  __syncthreads();
  const bool again = NORM || st->reorth != 0;
  const float inv = NORM ? 1.f : st->finv;
  float4 *w4 = reinterpret_cast<float4 *>(w);
  float4 *V4 = reinterpret_cast<float4 *>(V);
  float4 *c4 = reinterpret_cast<float4 *>(vcopy);
  float q = 0.f;
  for(int64_t g = (int64_t)blockIdx.x * RB + threadIdx.x; g < n4; g += (int64_t)gridDim.x * RB) {
    float4 wv = w4[g];
    // one batch of eight column loads in flight at a time (unrolled
    // batches would hoist every load and spill)
#pragma unroll 1
    for(int c0 = 0; c0 < CMAX; c0 += 8) {
      if(c0 < ncols) {
        float4 v[8];
#pragma unroll
        for(int u = 0; u < 8; ++u)
          v[u] = c0 + u < ncols ? __ldcs(V4 + vidx4(g, c0 + u, m1)) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for(int u = 0; u < 8; ++u) {
          const float h = hs[c0 + u];
          wv.x = fmaf(-h, v[u].x, wv.x);
          wv.y = fmaf(-h, v[u].y, wv.y);
          wv.z = fmaf(-h, v[u].z, wv.z);
          wv.w = fmaf(-h, v[u].w, wv.w);
        }
      }
    }
    if(NORM) {
      q = fmaf(wv.x, wv.x, fmaf(wv.y, wv.y, fmaf(wv.z, wv.z, fmaf(wv.w, wv.w, q))));
    } else if(!again) {
      wv.x *= inv;
      wv.y *= inv;
      wv.z *= inv;
      wv.w *= inv;
      V4[vidx4(g, ncols, m1)] = wv;
      c4[g] = wv;
      continue;
    }
    w4[g] = wv;
  }
  if(!NORM) return;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for(int o = 16; o > 0; o >>= 1) q += __shfl_xor_sync(0xffffffffu, q, o);
  if(lane == 0) wred[warp] = (double)q;
  __syncthreads();
  if(threadIdx.x == 0) {
    double sum = 0.;
    for(int k = 0; k < RB / 32; ++k) sum += wred[k];
    partials[blockIdx.x] = sum;
    __threadfence();
    last = atomicAdd(&st->counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if(!last) return;
  __threadfence();
  {
    // every thread of the last block: partials t, t + RB, t + 2 RB, ... (one
    // round of straight-line loads for up to 4 RB blocks), then the warps'
    // sums in warp order
    const int nb = (int)gridDim.x;
    double t = 0.;
    for(int b0 = threadIdx.x; b0 < nb; b0 += 4 * RB) {
      double v[4];
#pragma unroll
      for(int k = 0; k < 4; ++k) v[k] = __ldcg(partials + (b0 + RB * k < nb ? b0 + RB * k : 0));
#pragma unroll
      for(int k = 0; k < 4; ++k) t += b0 + RB * k < nb ? v[k] : 0.;
    }
    for(int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    __syncthreads();
    if(lane == 0) wred[warp] = t;
    __syncthreads();
  }
  if(threadIdx.x == 0) {
    double sum = 0.;
    for(int k = 0; k < RB / 32; ++k) sum += wred[k];
    const double nrm = sqrt(sum);
    st->result[0] = sum;
    *Hnext = nrm;
    st->finv = nrm > 0 ? (float)(1.0 / nrm) : 0.f;
    if(!second) st->reorth = sum < 1e-2 * st->result[2] ? 1 : 0;
    st->counter = 0;
  }
}

// v = w * (1 / ||w||) in FP32, 4 rows per thread; the scale comes from the
// last update + norm pass (k_gs_upd<., true> or k_gs32<., 2>).
// gated: only after a second Gram-Schmidt pass (otherwise k_gs_upd wrote v).
// gs (ungated only): the last block does not scale; its warp 0 applies the
// Givens rotations of step j meanwhile (k_givens folded in; a block that
// starts after the step converged skips its share of v, which the cycle no
// longer reads).
// The result goes to column col of the row-blocked basis V and to its
// contiguous copy vcopy (the preconditioner's next input).
__global__ void k_scale32(int64_t n4, const float *__restrict__ w, float *__restrict__ V, int m1, int col,
                          float *__restrict__ vcopy, const RedState *st, const int *__restrict__ done, int gated,
                          GmresState *gs, int j)
{
  FE_PDL_ENTRY();
  __shared__ double sh[MAXM + 1], scs[MAXM], ssn[MAXM];
  if(*done || (gated && !st->reorth)) return;
  if(gs && blockIdx.x == gridDim.x - 1) {
    if(threadIdx.x < 32) givens_warp(gs, j, threadIdx.x, sh, scs, ssn);
    return;
  }
  const int nb = gs ? (int)gridDim.x - 1 : (int)gridDim.x;
  const float inv = st->finv;
  const float4 *w4 = reinterpret_cast<const float4 *>(w);
  float4 *V4 = reinterpret_cast<float4 *>(V);
  float4 *c4 = reinterpret_cast<float4 *>(vcopy);
  for(int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < n4; g += (int64_t)nb * blockDim.x) {
    float4 t = w4[g];
    t.x *= inv;
    t.y *= inv;
    t.z *= inv;
    t.w *= inv;
    V4[vidx4(g, col, m1)] = t;
    c4[g] = t;
  }
}

// V_0 = r / ||r|| rounded to FP32 (start of a mixed cycle; column 0 of the
// row-blocked basis V and its contiguous copy vcopy), beta = ||r||.
__global__ void k_scale_r32(int64_t n, const double *__restrict__ r, float *__restrict__ V, int m1,
                            float *__restrict__ vcopy, const RedState *st, double *beta, const int *__restrict__ done)
{
  FE_PDL_ENTRY();
  if(*done) return;
  const double nrm = sqrt(st->result[0]);
  if(blockIdx.x == 0 && threadIdx.x == 0) *beta = nrm;
  const double inv = nrm > 0 ? 1.0 / nrm : 0.0;
  for(int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float v = (float)(r[i] * inv);
    V[(i / VBLK) * m1 * VBLK + (i % VBLK)] = v;
    vcopy[i] = v;
  }
}

__global__ void k_gmres_init(GmresState *gs, const RedState *st)
{
  FE_PDL_ENTRY();
  const double beta = sqrt(st->result[0]);
  const double tol = gs->tol;
  gs->g[0] = beta;
  for(int i = 1; i <= MAXM; ++i) gs->g[i] = 0.;
  gs->done = (beta <= tol || !isfinite(beta)) ? 1 : 0;
  gs->k = 0;
  gs->est = beta;
}

// ---------------------------------------------------------------------------
// Block-Jacobi ILU(0) (Saad Alg. 10.4, IKJ variant restricted to the pattern),
// level-scheduled: one warp per row, the rows of a level in parallel.  The
// factorisation applies each row's updates in the serial order (ascending
// pivots k, each entry once per k), so the factors equal the serial ones bit
// for bit; the triangular solves sum each row in a warp-tree order.
// ---------------------------------------------------------------------------
constexpr int ILU_NARROW_THREADS = 1024;  // one block of 32 warps runs a run of narrow levels

template <typename VF>
__global__ void k_ilu_copy(int64_t lnnz, const int32_t *__restrict__ srcPos, const double *__restrict__ v64,
                           const float *__restrict__ v32, VF *__restrict__ f)
{
  FE_PDL_ENTRY();
  for(int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < lnnz; k += (int64_t)gridDim.x * blockDim.x)
    f[k] = v64 ? (VF)v64[srcPos[k]] : (VF)v32[srcPos[k]];
}

// Row i (one warp): for each pivot k of its L part in ascending order,
// l_ik = a_ik / u_kk, then a_ij -= l_ik u_kj for the entries j > k of row i
// that row k holds (binary search in row k's U part, lanes over j).
template <typename VF>
__device__ __forceinline__ void ilu_factor_row(int32_t i, const int32_t *__restrict__ lia,
                                               const int32_t *__restrict__ lja, const int32_t *__restrict__ ldiag,
                                               VF *__restrict__ f, int *__restrict__ status)
{
  const int lane = threadIdx.x & 31;
  const int32_t rb = lia[i], re = lia[i + 1], rd = ldiag[i];
  for(int32_t kk = rb; kk < rd; ++kk) {
    const int32_t kr = lja[kk];
    const VF piv = f[ldiag[kr]];
    if(piv == (VF)0) {
      if(lane == 0) atomicExch(status, 1);
      return;
    }
    const VF lik = f[kk] / piv;
    __syncwarp();
    if(lane == 0) f[kk] = lik;
    const int32_t ub = ldiag[kr] + 1, ue = lia[kr + 1];
    for(int32_t jj = kk + 1 + lane; jj < re; jj += 32) {
      const int32_t col = lja[jj];
      int32_t lo = ub, hi = ue - 1;
      while(lo <= hi) {
        const int32_t mid = (lo + hi) >> 1, c = lja[mid];
        if(c == col) {
          f[jj] -= lik * f[mid];
          break;
        }
        if(c < col) lo = mid + 1;
        else hi = mid - 1;
      }
    }
    __syncwarp();
  }
  if(lane == 0) {
    const VF d = f[rd];
    if(d == (VF)0) atomicExch(status, 1);
    else if(!isfinite((double)d)) atomicExch(status, 2);
  }
}

// z_i = r_i - sum_{k < i} l_ik z_k (lower) or z_i = (z_i - sum_{k > i} u_ik z_k) / u_ii (upper).
template <typename VF, typename VV, bool LOWER>
__device__ __forceinline__ void ilu_solve_row(int32_t i, const int32_t *__restrict__ lia,
                                              const int32_t *__restrict__ lja, const int32_t *__restrict__ ldiag,
                                              const VF *__restrict__ f, const VV *__restrict__ r, VV *__restrict__ z)
{
  const int lane = threadIdx.x & 31;
  const int32_t d = ldiag[i];
  const int32_t b = LOWER ? lia[i] : d + 1, e = LOWER ? d : lia[i + 1];
  VF s = 0;
  for(int32_t k = b + lane; k < e; k += 32) s += f[k] * (VF)z[lja[k]];
  for(int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if(lane == 0) {
    if(LOWER) z[i] = (VV)((VF)r[i] - s);
    else z[i] = (VV)(((VF)z[i] - s) / f[d]);
  }
}

// A run of narrow levels: one block, levels in order, a barrier between them.
template <typename VF>
__global__ void __launch_bounds__(ILU_NARROW_THREADS) k_ilu_factor_run(
    int32_t lv0, int32_t lv1, const int32_t *__restrict__ lvl, const int32_t *__restrict__ rows,
    const int32_t *__restrict__ lia, const int32_t *__restrict__ lja, const int32_t *__restrict__ ldiag,
    VF *__restrict__ f, int *__restrict__ status)
{
  FE_PDL_ENTRY();
  const int warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for(int32_t lv = lv0; lv < lv1; ++lv) {
    for(int32_t q = lvl[lv] + warp; q < lvl[lv + 1]; q += nw) ilu_factor_row<VF>(rows[q], lia, lja, ldiag, f, status);
    __syncthreads();
  }
}

// One wide level over many blocks (warp per row).
template <typename VF>
__global__ void k_ilu_factor_level(int32_t q0, int32_t q1, const int32_t *__restrict__ rows,
                                   const int32_t *__restrict__ lia, const int32_t *__restrict__ lja,
                                   const int32_t *__restrict__ ldiag, VF *__restrict__ f, int *__restrict__ status)
{
  FE_PDL_ENTRY();
  const int64_t q = q0 + ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32;
  if(q < q1) ilu_factor_row<VF>(rows[q], lia, lja, ldiag, f, status);
}

template <typename VF, typename VV, bool LOWER>
__global__ void __launch_bounds__(ILU_NARROW_THREADS) k_ilu_solve_run(
    int32_t lv0, int32_t lv1, const int32_t *__restrict__ lvl, const int32_t *__restrict__ rows,
    const int32_t *__restrict__ lia, const int32_t *__restrict__ lja, const int32_t *__restrict__ ldiag,
    const VF *__restrict__ f, const VV *__restrict__ r, VV *__restrict__ z, const int *__restrict__ done)
{
  FE_PDL_ENTRY();
  if(done && *done) return;
  const int warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for(int32_t lv = lv0; lv < lv1; ++lv) {
    for(int32_t q = lvl[lv] + warp; q < lvl[lv + 1]; q += nw)
      ilu_solve_row<VF, VV, LOWER>(rows[q], lia, lja, ldiag, f, r, z);
    __syncthreads();
  }
}

template <typename VF, typename VV, bool LOWER>
__global__ void k_ilu_solve_level(int32_t q0, int32_t q1, const int32_t *__restrict__ rows,
                                  const int32_t *__restrict__ lia, const int32_t *__restrict__ lja,
                                  const int32_t *__restrict__ ldiag, const VF *__restrict__ f,
                                  const VV *__restrict__ r, VV *__restrict__ z, const int *__restrict__ done)
{
  FE_PDL_ENTRY();
  if(done && *done) return;
  const int64_t q = q0 + ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32;
  if(q < q1) ilu_solve_row<VF, VV, LOWER>(rows[q], lia, lja, ldiag, f, r, z);
}

template <typename VV, typename VD>
__global__ void k_jacobi(int64_t n, const VD *__restrict__ dinv, const VV *__restrict__ r,
                         VV *__restrict__ z, const int *__restrict__ done)
{
  FE_PDL_ENTRY();
  if(done && *done) return;
  for(int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
      i += (int64_t)gridDim.x * blockDim.x)
    z[i] = (VV)((VD)r[i] * dinv[i]);
}

template <typename VA, typename VD>
__global__ void k_inv_diag(int64_t n, const int32_t *__restrict__ diag, const VA *__restrict__ a,
                           VD *__restrict__ dinv, int *__restrict__ status)
{
  FE_PDL_ENTRY();
  for(int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
      i += (int64_t)gridDim.x * blockDim.x) {
    const VA d = a[diag[i]];
    if(d == (VA)0) { atomicExch(status, 1); dinv[i] = 0; }
    else dinv[i] = (VD)(1.0 / (double)d);
  }
}

// CG helpers operating on device scalars (CGState) so that the host need not
// read back anything inside an iteration.
struct CGState {
  double rz, rzOld, pq, rr;
  double tol;
  int done;
  int it;
};

__global__ void k_cg_xr(int64_t n, CGState *cs, const double *__restrict__ p,
                        const double *__restrict__ q, double *__restrict__ x,
                        double *__restrict__ r, double *partials, RedState *st)
{
  FE_PDL_ENTRY();
  // alpha = rz / pq ; x += alpha p ; r -= alpha q ; accumulate rr
  double v[1] = {0.};
  if(!cs->done) {
    const double alpha = cs->rz / cs->pq;
    for(int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
        i += (int64_t)gridDim.x * blockDim.x) {
      x[i] += alpha * p[i];
      const double ri = r[i] - alpha * q[i];
      r[i] = ri;
      v[0] += ri * ri;
    }
  }
  finish_reduction<1, false>(v, partials, st, nullptr);
}

__global__ void k_cg_check(CGState *cs, const RedState *st)
{
  FE_PDL_ENTRY();
  if(cs->done) return;
  cs->rr = st->result[0];
  cs->it++;
  if(!(sqrt(cs->rr) > cs->tol) || !isfinite(cs->rr)) cs->done = 1;
}

__global__ void k_cg_p(int64_t n, CGState *cs, const RedState *st, const double *__restrict__ z,
                       double *__restrict__ p, int first)
{
  FE_PDL_ENTRY();
  if(cs->done) return;
  const double rzNew = st->result[0];
  const double beta = first ? 0. : rzNew / cs->rz;
  for(int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
      i += (int64_t)gridDim.x * blockDim.x)
    p[i] = z[i] + beta * p[i];
  __syncthreads();
  // the scalar update happens in k_cg_rz once every block is done
}

__global__ void k_cg_rz(CGState *cs, const RedState *st)
{
  FE_PDL_ENTRY();
  if(cs->done) return;
  cs->rz = st->result[0];
}

__global__ void k_cg_pq(CGState *cs, const RedState *st)
{
  FE_PDL_ENTRY();
  if(cs->done) return;
  cs->pq = st->result[0];
  if(cs->pq == 0.0 || !isfinite(cs->pq)) cs->done = 1;
}

__global__ void k_dot_if(int64_t n, const double *__restrict__ x, const double *__restrict__ y,
                         double *partials, RedState *st, const CGState *cs)
{
  FE_PDL_ENTRY();
  double v[1] = {0.};
  if(!cs->done)
    for(int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
        i += (int64_t)gridDim.x * blockDim.x)
      v[0] += x[i] * y[i];
  finish_reduction<1, false>(v, partials, st, nullptr);
}

__global__ void k_zero(int64_t n, double *x)
{
  FE_PDL_ENTRY();
  for(int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
      i += (int64_t)gridDim.x * blockDim.x)
    x[i] = 0.;
}

__global__ void k_copy(int64_t n, const double *__restrict__ a, double *__restrict__ b)
{
  FE_PDL_ENTRY();
  for(int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
      i += (int64_t)gridDim.x * blockDim.x)
    b[i] = a[i];
}

__global__ void k_axpy(int64_t n, double alpha, const double *__restrict__ x, double *__restrict__ y)
{
  FE_PDL_ENTRY();
  for(int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
      i += (int64_t)gridDim.x * blockDim.x)
    y[i] += alpha * x[i];
}

}  // namespace

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
namespace {
struct Ws {
  RedState *st;
  GmresState *gs, *hgs;
  CGState *cg, *hcg;
};
}  // namespace
#define Ws_INIT(k) {(RedState *)(k)->red_state_, (GmresState *)(k)->gmres_, (GmresState *)(k)->h_gmres_, (CGState *)(k)->cg_, (CGState *)(k)->h_cg_}
Krylov::~Krylov()
{
  cudaFree(V_); cudaFree(Z_); cudaFree(Z32_); cudaFree(V32_); cudaFree(vc32_); cudaFree(xs2_); cudaFree(v32_); cudaFree(w32_);
  cudaFree(zeroFlag_);
  cudaFree(sellPtr_); cudaFree(sellCol_); cudaFree(sellSrc_); cudaFree(sellVal_);
  cudaFree(w_); cudaFree(r_); cudaFree(t_); cudaFree(p_); cudaFree(q_);
  cudaFree(diag_); cudaFree(diag32_); cudaFree(red_); cudaFree(dsum_);
  cudaFreeHost(hred_);
  cudaFree(ilu_.blockStart); cudaFree(ilu_.perm); cudaFree(ilu_.lia); cudaFree(ilu_.lja);
  cudaFree(ilu_.ldiag); cudaFree(ilu_.srcPos); cudaFree(ilu_.vals); cudaFree(ilu_.status);
  cudaFree(ilu_.rowsL); cudaFree(ilu_.rowsU); cudaFree(ilu_.lvlL); cudaFree(ilu_.lvlU);
  cudaFree(red_state_); cudaFree(gmres_); cudaFree(cg_);
  cudaFreeHost(h_gmres_); cudaFreeHost(h_cg_); cudaFreeHost(hflag_); cudaFreeHost(htol_); cudaFreeHost(hdone_);
  for(auto e : evs_) cudaEventDestroy(e);
  for(auto &g : graphs_) cudaGraphExecDestroy(g.second);
  delete mg_;
}

static int grid_for(int64_t n, int threads, int maxBlocks)
{
  int64_t b = (n + threads - 1) / threads;
  return (int)std::max<int64_t>(1, std::min<int64_t>(b, maxBlocks));
}

static size_t backsolveSmem(int m) { return sizeof(double) * (size_t)m * (m + 1) / 2; }

// Stops launching the iterations of a restart cycle once the device has set
// its done flag (read every 4 iterations; skipped kernels would no-op anyway).
bool Krylov::poll_done(const int *dflag, int j)
{
  if((j & 3) != 3) return false;
  cudaMemcpyAsync(hflag_, dflag, sizeof(int), cudaMemcpyDeviceToHost, s_);
  cudaStreamSynchronize(s_);
  return *hflag_ != 0;
}

int Krylov::setup(const DeviceCSR &A, const std::vector<int32_t> &blockOfRow, int64_t nBlocksHint,
                  const KrylovOptions &o, cudaStream_t s, const PrecondInfo *pinfo)
{
  A_ = A;
  opt = o;
  // FENG_CUDA_GRAPHS=0 launches the restart cycles kernel by kernel (the same
  // kernels, in the same order) -- for profilers that cannot replay graphs.
  if(const char *e = std::getenv("FENG_CUDA_GRAPHS")) useGraphs_ = std::strcmp(e, "0") != 0;
  s_ = s;
  n_ = A.n;
  if(opt.restart < 1 || opt.restart > MAXM) {
    set_error("restart must be in [1, %d]", MAXM);
    return FE_INVALID_ARG;
  }
  CK(cudaFuncSetAttribute(k_backsolve, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)backsolveSmem(MAXM)));
  const double avg = n_ > 0 ? (double)A.nnz / n_ : 0;
  // 8 lanes per row beat 16 on the Taylor-Hood Jacobian (~29 entries per row)
  lanes_ = avg > 64 ? 16 : (avg > 12 ? 8 : 4);
  nParts_ = grid_for(n_, RB, MAXRED);
  const int m = opt.restart;
  CK(cudaMalloc(&red_, sizeof(double) * MAXRED * (MAXM + 2)));
  CK(cudaMalloc(&dsum_, sizeof(double) * 8));
  CK(cudaMallocHost(&hred_, sizeof(double) * 8));
  CK(cudaMalloc(&w_, sizeof(double) * n_));
  CK(cudaMalloc(&r_, sizeof(double) * n_));
  CK(cudaMalloc(&t_, sizeof(double) * n_));
  CK(cudaMalloc(&p_, sizeof(double) * n_));
  CK(cudaMalloc(&q_, sizeof(double) * n_));
  if(opt.method == 1) {
    if(opt.mixed) {
      if(m > 64) {
        set_error("mixed-precision FGMRES supports restart lengths up to 64 (got %d)", m);
        return FE_INVALID_ARG;
      }
      // whole row blocks of the basis (rows n..ld-1 stay zero)
      ld32_ = (n_ + VBLK - 1) / VBLK * VBLK;
      CK(cudaMalloc(&V32_, sizeof(float) * ld32_ * (m + 1)));
      CK(cudaMalloc(&Z32_, sizeof(float) * ld32_ * m));
      CK(cudaMalloc(&vc32_, sizeof(float) * ld32_));
      CK(cudaMalloc(&xs2_, sizeof(float2) * ld32_));
      CK(cudaMemset(V32_, 0, sizeof(float) * ld32_ * (m + 1)));
      CK(cudaMemset(Z32_, 0, sizeof(float) * ld32_ * m));
      CK(cudaMemset(vc32_, 0, sizeof(float) * ld32_));
      if(n_ >= 32 * 152) FE_TRY(build_sell());
    } else {
      CK(cudaMalloc(&V_, sizeof(double) * n_ * (m + 1)));
      CK(cudaMalloc(&Z_, sizeof(double) * n_ * m));
    }
  }
  // one group of 4 rows per thread: the whole pass is one wave of loads
  {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    nSM_ = std::max(1, sms);
  }
  // whole waves of the update passes (three blocks per SM)
  gsParts_ = grid_for((n_ + 3) / 4, RB, std::min(MAXRED, 3 * nSM_));
  // dot pass: one pass over all columns (k_gs_dots_all); FENG_GS_DOTS=groups
  // keeps the column-group grid of k_gs_dots (the same products, summed in
  // another order; for comparisons)
  if(const char *e = std::getenv("FENG_GS_DOTS")) allDots_ = std::strcmp(e, "groups") != 0;
  CK(cudaMalloc(&v32_, sizeof(float) * n_));
  {
    const int64_t lw = std::max<int64_t>(ld32_, (n_ + 63) / 64 * 64);
    CK(cudaMalloc(&w32_, sizeof(float) * lw));
    CK(cudaMemset(w32_, 0, sizeof(float) * lw));
  }
  CK(cudaMalloc(&red_state_, sizeof(RedState)));
  CK(cudaMemset(red_state_, 0, sizeof(RedState)));
  CK(cudaMalloc(&gmres_, sizeof(GmresState)));
  CK(cudaMemset(gmres_, 0, sizeof(GmresState)));
  CK(cudaMalloc(&cg_, sizeof(CGState)));
  CK(cudaMemset(cg_, 0, sizeof(CGState)));
  CK(cudaMallocHost(&h_gmres_, sizeof(GmresState)));
  CK(cudaMallocHost(&h_cg_, sizeof(CGState)));
  CK(cudaMallocHost(&hflag_, sizeof(int)));
  CK(cudaMallocHost(&htol_, sizeof(double)));
  CK(cudaMallocHost(&hdone_, sizeof(int) * (MAXM + 1)));
  {
    // Arnoldi steps per part graph of a mixed cycle (0: one graph per cycle)
    const char *e = std::getenv("FENG_GMRES_CHUNK");
    chunk_ = e ? std::atoi(e) : 5;
  }

  if(opt.precond == 3 || opt.precond == 4) {
    if(!pinfo) {
      set_error("multigrid preconditioner without set-up information");
      return FE_INVALID_ARG;
    }
    FE_TRY(setup_mg(*pinfo));
  } else if(opt.precond == 2) {
    if(opt.mixed) CK(cudaMalloc(&diag32_, sizeof(float) * n_));
    else CK(cudaMalloc(&diag_, sizeof(double) * n_));
    CK(cudaMalloc(&ilu_.status, sizeof(int)));
  } else if(opt.precond == 1) {
    // Host: gather the block-diagonal part of the pattern.
    std::vector<int32_t> hia(n_ + 1), hja(A.nnz);
    CK(cudaMemcpy(hia.data(), A.ia, sizeof(int32_t) * (n_ + 1), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(hja.data(), A.ja, sizeof(int32_t) * A.nnz, cudaMemcpyDeviceToHost));
    std::vector<int32_t> blk(n_);
    int64_t nb = 1;
    if((int64_t)blockOfRow.size() == n_) {
      nb = 0;
      for(int64_t i = 0; i < n_; ++i) {
        blk[i] = blockOfRow[i];
        nb = std::max<int64_t>(nb, blk[i] + 1);
      }
    } else {
      nb = std::max<int64_t>(1, std::min<int64_t>(nBlocksHint, n_));
      for(int64_t i = 0; i < n_; ++i) blk[i] = (int32_t)((i * nb) / n_);
    }
    std::vector<int32_t> bstart(nb + 1, 0), perm(n_);
    for(int64_t i = 0; i < n_; ++i) bstart[blk[i] + 1]++;
    for(int64_t b = 0; b < nb; ++b) bstart[b + 1] += bstart[b];
    std::vector<int32_t> fillp(bstart.begin(), bstart.end() - 1);
    for(int64_t i = 0; i < n_; ++i) perm[fillp[blk[i]]++] = (int32_t)i;
    std::vector<int32_t> lia(n_ + 1, 0), lja, ldiag(n_, -1), src;
    lja.reserve(A.nnz);
    src.reserve(A.nnz);
    for(int64_t i = 0; i < n_; ++i) {
      for(int32_t k = hia[i]; k < hia[i + 1]; ++k) {
        const int32_t j = hja[k];
        if(blk[j] != blk[i]) continue;
        if(j == i) ldiag[i] = (int32_t)lja.size();
        lja.push_back(j);
        src.push_back(k);
      }
      lia[i + 1] = (int32_t)lja.size();
      if(ldiag[i] < 0) {
        set_error("row %lld has no diagonal entry in the pattern", (long long)i);
        return FE_INVALID_ARG;
      }
    }
    ilu_.nBlocks = nb;
    ilu_.lnnz = (int64_t)lja.size();
    CK(cudaMalloc(&ilu_.blockStart, sizeof(int32_t) * (nb + 1)));
    CK(cudaMalloc(&ilu_.perm, sizeof(int32_t) * n_));
    CK(cudaMalloc(&ilu_.lia, sizeof(int32_t) * (n_ + 1)));
    CK(cudaMalloc(&ilu_.lja, sizeof(int32_t) * ilu_.lnnz));
    CK(cudaMalloc(&ilu_.ldiag, sizeof(int32_t) * n_));
    CK(cudaMalloc(&ilu_.srcPos, sizeof(int32_t) * ilu_.lnnz));
    CK(cudaMalloc(&ilu_.vals, (opt.mixed ? sizeof(float) : sizeof(double)) * ilu_.lnnz));
    CK(cudaMalloc(&ilu_.status, sizeof(int)));
    CK(cudaMemcpy(ilu_.blockStart, bstart.data(), sizeof(int32_t) * (nb + 1), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(ilu_.perm, perm.data(), sizeof(int32_t) * n_, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(ilu_.lia, lia.data(), sizeof(int32_t) * (n_ + 1), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(ilu_.lja, lja.data(), sizeof(int32_t) * ilu_.lnnz, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(ilu_.ldiag, ldiag.data(), sizeof(int32_t) * n_, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(ilu_.srcPos, src.data(), sizeof(int32_t) * ilu_.lnnz, cudaMemcpyHostToDevice));
    FE_TRY(build_ilu_levels(lia, lja, ldiag));
  }
  return FE_OK;
}

// Level schedules of the factor's L and U parts and their segments (see
// DeviceBlockILU).  A level is wide when its rows would keep one block of
// 32 warps busy for several rounds.
int Krylov::build_ilu_levels(const std::vector<int32_t> &lia, const std::vector<int32_t> &lja,
                             const std::vector<int32_t> &ldiag)
{
  const int64_t n = n_;
  constexpr int32_t WIDE = 256;  // rows
  auto schedule = [&](bool lower, std::vector<int32_t> &rows, std::vector<int32_t> &lvl,
                      std::vector<DeviceBlockILU::Segment> &seg) {
    std::vector<int32_t> level(n, 0);
    int32_t nl = 0;
    if(lower) {
      for(int64_t i = 0; i < n; ++i) {
        int32_t m = 0;
        for(int32_t k = lia[i]; k < ldiag[i]; ++k) m = std::max(m, level[lja[k]] + 1);
        level[i] = m;
        nl = std::max(nl, m + 1);
      }
    } else {
      for(int64_t i = n - 1; i >= 0; --i) {
        int32_t m = 0;
        for(int32_t k = ldiag[i] + 1; k < lia[i + 1]; ++k) m = std::max(m, level[lja[k]] + 1);
        level[i] = m;
        nl = std::max(nl, m + 1);
      }
    }
    lvl.assign(nl + 1, 0);
    for(int64_t i = 0; i < n; ++i) lvl[level[i] + 1]++;
    for(int32_t l = 0; l < nl; ++l) lvl[l + 1] += lvl[l];
    rows.resize(n);
    std::vector<int32_t> fill(lvl.begin(), lvl.end() - 1);
    for(int64_t i = 0; i < n; ++i) rows[fill[level[i]]++] = (int32_t)i;  // ascending within a level
    seg.clear();
    for(int32_t l = 0; l < nl;) {
      const int32_t cnt = lvl[l + 1] - lvl[l];
      if(cnt > WIDE) {
        seg.push_back({1, l, l + 1, cnt, lvl[l], lvl[l + 1]});
        ++l;
        continue;
      }
      int32_t e = l, r = 0;
      while(e < nl && lvl[e + 1] - lvl[e] <= WIDE) {
        r += lvl[e + 1] - lvl[e];
        ++e;
      }
      seg.push_back({0, l, e, r, lvl[l], lvl[e]});
      l = e;
    }
    return nl;
  };
  std::vector<int32_t> rl, ll, ru, lu;
  ilu_.nLevL = schedule(true, rl, ll, ilu_.segL);
  ilu_.nLevU = schedule(false, ru, lu, ilu_.segU);
  CK(cudaMalloc(&ilu_.rowsL, sizeof(int32_t) * n));
  CK(cudaMalloc(&ilu_.rowsU, sizeof(int32_t) * n));
  CK(cudaMalloc(&ilu_.lvlL, sizeof(int32_t) * ll.size()));
  CK(cudaMalloc(&ilu_.lvlU, sizeof(int32_t) * lu.size()));
  CK(cudaMemcpy(ilu_.rowsL, rl.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ilu_.rowsU, ru.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ilu_.lvlL, ll.data(), sizeof(int32_t) * ll.size(), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ilu_.lvlU, lu.data(), sizeof(int32_t) * lu.size(), cudaMemcpyHostToDevice));
  return FE_OK;
}

template <typename VF>
void Krylov::ilu_factor_levels(const double *values64, const float *values32)
{
  VF *f = (VF *)ilu_.vals;
  ::feng::launch_k(k_ilu_copy<VF>, grid_for(ilu_.lnnz, 256, 4096), 256, 0, s_, ilu_.lnnz, ilu_.srcPos, values64, values32, f);
  for(const auto &sg : ilu_.segL) {
    if(sg.wide)
      ::feng::launch_k(k_ilu_factor_level<VF>, (unsigned)(((int64_t)sg.rows * 32 + 255) / 256), 256, 0, s_, 
           sg.q0, sg.q1, ilu_.rowsL, ilu_.lia, ilu_.lja, ilu_.ldiag, f, ilu_.status);
    else
      ::feng::launch_k(k_ilu_factor_run<VF>, 1, ILU_NARROW_THREADS, 0, s_, sg.lv0, sg.lv1, ilu_.lvlL, ilu_.rowsL, ilu_.lia,
                                                                ilu_.lja, ilu_.ldiag, f, ilu_.status);
  }
}

template <typename VF, typename VV>
void Krylov::ilu_solve_levels(const VV *r, VV *z, const int *done)
{
  const VF *f = (const VF *)ilu_.vals;
  for(const auto &sg : ilu_.segL) {
    if(sg.wide)
      ::feng::launch_k(k_ilu_solve_level<VF, VV, true>, (unsigned)(((int64_t)sg.rows * 32 + 255) / 256), 256, 0, s_, 
           sg.q0, sg.q1, ilu_.rowsL, ilu_.lia, ilu_.lja, ilu_.ldiag, f, r, z, done);
    else
      ::feng::launch_k(k_ilu_solve_run<VF, VV, true>, 1, ILU_NARROW_THREADS, 0, s_, sg.lv0, sg.lv1, ilu_.lvlL, ilu_.rowsL,
                                                                         ilu_.lia, ilu_.lja, ilu_.ldiag, f, r, z,
                                                                         done);
  }
  for(const auto &sg : ilu_.segU) {
    if(sg.wide)
      ::feng::launch_k(k_ilu_solve_level<VF, VV, false>, (unsigned)(((int64_t)sg.rows * 32 + 255) / 256), 256, 0, s_, 
           sg.q0, sg.q1, ilu_.rowsU, ilu_.lia, ilu_.lja, ilu_.ldiag, f, r, z, done);
    else
      ::feng::launch_k(k_ilu_solve_run<VF, VV, false>, 1, ILU_NARROW_THREADS, 0, s_, sg.lv0, sg.lv1, ilu_.lvlU, ilu_.rowsU,
                                                                          ilu_.lia, ilu_.lja, ilu_.ldiag, f, r, z,
                                                                          done);
  }
}

namespace {
// y = A x on the sliced-ELL copy, FP32, thread = row (rows of a warp are one
// slice, so every column and value load is one full line).  Steps of UNR
// entries, software-pipelined: the next step's columns and values are
// loaded before this step's gathers of x, so a step waits for one memory
// latency instead of two (29.4 us against 35.0 us with plain unrolled steps
// of 4 on the 256 x 256 Kovasznay Jacobian).
template <int UNR>
__global__ void __launch_bounds__(256) k_spmv_sell(int64_t n, const int32_t *__restrict__ sp,
                                                   const int32_t *__restrict__ sc, const float *__restrict__ sv,
                                                   const float *__restrict__ x, float *__restrict__ y,
                                                   const int *__restrict__ done)
{
  FE_PDL_ENTRY();
  if(done && *done) return;
  const int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if(row >= n) return;
  const int64_t sl = row >> 5;
  const int lane = (int)(row & 31);
  const int32_t base = sp[sl], len = (sp[sl + 1] - base) >> 5;
  float acc = 0.f;
  int32_t c[UNR];
  float a[UNR];
#pragma unroll
  for(int u = 0; u < UNR; ++u) {
    const bool ok = u < len;
    const int32_t e = base + (u << 5) + lane;
    c[u] = ok ? __ldcs(sc + e) : -1;
    a[u] = ok ? __ldcs(sv + e) : 0.f;
  }
  for(int32_t k = 0; k < len; k += UNR) {
    int32_t cn[UNR];
    float an[UNR];
#pragma unroll
    for(int u = 0; u < UNR; ++u) {
      const bool ok = k + UNR + u < len;
      const int32_t e = base + ((k + UNR + u) << 5) + lane;
      cn[u] = ok ? __ldcs(sc + e) : -1;
      an[u] = ok ? __ldcs(sv + e) : 0.f;
    }
#pragma unroll
    for(int u = 0; u < UNR; ++u)
      if(c[u] >= 0) acc = fmaf(a[u], x[c[u]], acc);
#pragma unroll
    for(int u = 0; u < UNR; ++u) {
      c[u] = cn[u];
      a[u] = an[u];
    }
  }
  y[row] = acc;
}

// r = b - A x on the sliced-ELL copy of the FP32 matrix with FP64 x and
// FP64 accumulation (the mixed FGMRES's restart residual: iterative
// refinement), thread = row, the pipelined walk of k_spmv_sell.
template <int UNR>
__global__ void __launch_bounds__(256) k_resid_sell(int64_t n, const int32_t *__restrict__ sp,
                                                    const int32_t *__restrict__ sc, const float *__restrict__ sv,
                                                    const double *__restrict__ x, const double *__restrict__ b,
                                                    double *__restrict__ y)
{
  FE_PDL_ENTRY();
  const int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if(row >= n) return;
  const int64_t sl = row >> 5;
  const int lane = (int)(row & 31);
  const int32_t base = sp[sl], len = (sp[sl + 1] - base) >> 5;
  double acc = 0.;
  int32_t c[UNR];
  float a[UNR];
#pragma unroll
  for(int u = 0; u < UNR; ++u) {
    const bool ok = u < len;
    const int32_t e = base + (u << 5) + lane;
    c[u] = ok ? __ldcs(sc + e) : -1;
    a[u] = ok ? __ldcs(sv + e) : 0.f;
  }
  for(int32_t k = 0; k < len; k += UNR) {
    int32_t cn[UNR];
    float an[UNR];
#pragma unroll
    for(int u = 0; u < UNR; ++u) {
      const bool ok = k + UNR + u < len;
      const int32_t e = base + ((k + UNR + u) << 5) + lane;
      cn[u] = ok ? __ldcs(sc + e) : -1;
      an[u] = ok ? __ldcs(sv + e) : 0.f;
    }
#pragma unroll
    for(int u = 0; u < UNR; ++u)
      if(c[u] >= 0) acc = fma((double)a[u], x[c[u]], acc);
#pragma unroll
    for(int u = 0; u < UNR; ++u) {
      c[u] = cn[u];
      a[u] = an[u];
    }
  }
  y[row] = b[row] - acc;
}

// x split into two floats, x ~ hi + lo (the operand of k_resid_sell_df)
__global__ void k_split_x(int64_t n, const double *__restrict__ x, float2 *__restrict__ xs)
{
  FE_PDL_ENTRY();
  for(int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const dfl d = df_from(x[i]);
    xs[i] = make_float2(d.hi, d.lo);
  }
}

// r = b - A x as k_resid_sell, the products a (x_hi + x_lo) and their sum in
// double-float on the FP32 pipes (a x_hi exact by a fused multiply-add), the
// result subtracted from b in FP64: ~2^-44 relative to sum |a x| against
// FP64's 2^-53, far below the refinement's stops, and the FP64 pipe of the
// GB300 (one FP64 product per entry would take ~27 us at 588 k rows) left
// out.
template <int UNR>
__global__ void __launch_bounds__(256) k_resid_sell_df(int64_t n, const int32_t *__restrict__ sp,
                                                       const int32_t *__restrict__ sc, const float *__restrict__ sv,
                                                       const float2 *__restrict__ xs, const double *__restrict__ b,
                                                       double *__restrict__ y)
{
  FE_PDL_ENTRY();
  const int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if(row >= n) return;
  const int64_t sl = row >> 5;
  const int lane = (int)(row & 31);
  const int32_t base = sp[sl], len = (sp[sl + 1] - base) >> 5;
  dfl acc = df_zero();
  int32_t c[UNR];
  float a[UNR];
#pragma unroll
  for(int u = 0; u < UNR; ++u) {
    const bool ok = u < len;
    const int32_t e = base + (u << 5) + lane;
    c[u] = ok ? __ldcs(sc + e) : -1;
    a[u] = ok ? __ldcs(sv + e) : 0.f;
  }
  for(int32_t k = 0; k < len; k += UNR) {
    int32_t cn[UNR];
    float an[UNR];
#pragma unroll
    for(int u = 0; u < UNR; ++u) {
      const bool ok = k + UNR + u < len;
      const int32_t e = base + ((k + UNR + u) << 5) + lane;
      cn[u] = ok ? __ldcs(sc + e) : -1;
      an[u] = ok ? __ldcs(sv + e) : 0.f;
    }
#pragma unroll
    for(int u = 0; u < UNR; ++u)
      if(c[u] >= 0) {
        const float2 xv = xs[c[u]];
        const float p = __fmul_rn(a[u], xv.x);
        float e = __fmaf_rn(a[u], xv.x, -p);
        e = __fmaf_rn(a[u], xv.y, e);
        acc = df_add(acc, df_fast2(p, e));
      }
#pragma unroll
    for(int u = 0; u < UNR; ++u) {
      c[u] = cn[u];
      a[u] = an[u];
    }
  }
  y[row] = b[row] - df_to(acc);
}

// sliced-ELL values from the CSR values (padding: 0)
__global__ void k_sell_gather(int64_t m, const int32_t *__restrict__ src, const float *__restrict__ a,
                              float *__restrict__ out)
{
  FE_PDL_ENTRY();
  for(int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < m; e += (int64_t)gridDim.x * blockDim.x) {
    const int32_t k = src[e];
    out[e] = k >= 0 ? a[k] : 0.f;
  }
}
}  // namespace

int Krylov::build_sell()
{
  std::vector<int32_t> ia(n_ + 1), ja(A_.nnz);
  CK(cudaMemcpy(ia.data(), A_.ia, sizeof(int32_t) * (n_ + 1), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(ja.data(), A_.ja, sizeof(int32_t) * A_.nnz, cudaMemcpyDeviceToHost));
  const int64_t ns = (n_ + 31) / 32;
  std::vector<int32_t> ptr(ns + 1, 0);
  for(int64_t sl = 0; sl < ns; ++sl) {
    int64_t len = 0;
    for(int64_t r = sl * 32; r < std::min<int64_t>(n_, sl * 32 + 32); ++r) len = std::max<int64_t>(len, ia[r + 1] - ia[r]);
    if(ptr[sl] + 32 * len >= (int64_t)INT32_MAX) return FE_OK;  // CSR only
    ptr[sl + 1] = (int32_t)(ptr[sl] + 32 * len);
  }
  sellN_ = ptr[ns];
  std::vector<int32_t> col(std::max<int64_t>(sellN_, 1)), src(col.size(), -1);
  for(int64_t sl = 0; sl < ns; ++sl) {
    const int32_t len = (ptr[sl + 1] - ptr[sl]) / 32;
    for(int lane = 0; lane < 32; ++lane) {
      const int64_t r = sl * 32 + lane;
      for(int32_t k = 0; k < len; ++k) {
        const int64_t e = ptr[sl] + (int64_t)k * 32 + lane;
        if(r < n_ && ia[r] + k < ia[r + 1]) {
          col[e] = ja[ia[r] + k];
          src[e] = ia[r] + k;
        } else {
          col[e] = (int32_t)std::min<int64_t>(r, n_ - 1);  // padding: value 0 on an existing column
        }
      }
    }
  }
  CK(cudaMalloc(&sellPtr_, sizeof(int32_t) * ptr.size()));
  CK(cudaMalloc(&sellCol_, sizeof(int32_t) * col.size()));
  CK(cudaMalloc(&sellSrc_, sizeof(int32_t) * src.size()));
  CK(cudaMalloc(&sellVal_, sizeof(float) * col.size()));
  CK(cudaMemcpy(sellPtr_, ptr.data(), sizeof(int32_t) * ptr.size(), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(sellCol_, col.data(), sizeof(int32_t) * col.size(), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(sellSrc_, src.data(), sizeof(int32_t) * src.size(), cudaMemcpyHostToDevice));
  CK(cudaMemset(sellVal_, 0, sizeof(float) * col.size()));
  return FE_OK;
}

int Krylov::factor(const double *values64, const float *values32)
{
  factoredOk_ = false;
  cur64_ = values64;
  cur32_ = values32;
  if(opt.mixed && sellVal_ && values32)
    ::feng::launch_k(k_sell_gather, grid_for(sellN_, 256, 4096), 256, 0, s_, sellN_, sellSrc_, values32, sellVal_);
  if(opt.precond == 0) { factoredOk_ = true; return FE_OK; }
  if(opt.precond == 3 || opt.precond == 4) {
    FE_TRY(factor_mg(values64, values32));
    factoredOk_ = true;
    return FE_OK;
  }
  CK(cudaMemsetAsync(ilu_.status, 0, sizeof(int), s_));
  if(opt.precond == 2) {
    const int g = grid_for(n_, 256, 4096);
    if(opt.mixed) ::feng::launch_k(k_inv_diag<float, float>, g, 256, 0, s_, n_, A_.diag, values32, diag32_, ilu_.status);
    else ::feng::launch_k(k_inv_diag<double, double>, g, 256, 0, s_, n_, A_.diag, values64, diag_, ilu_.status);
  } else {
    if(opt.mixed) ilu_factor_levels<float>(nullptr, values32);
    else ilu_factor_levels<double>(values64, nullptr);
  }
  CK(cudaGetLastError());
  int hs = 0;
  CK(cudaMemcpyAsync(&hs, ilu_.status, sizeof(int), cudaMemcpyDeviceToHost, s_));
  CK(cudaStreamSynchronize(s_));
  if(hs != 0) {
    set_error(hs == 1 ? "preconditioner build hit a zero pivot" : "preconditioner build produced a non-finite pivot");
    return FE_PC_FAILED;
  }
  factoredOk_ = true;
  return FE_OK;
}

void Krylov::precond64(const double *r, double *z, const int *done)
{
  if(opt.precond == 0) {
    cudaMemcpyAsync(z, r, sizeof(double) * n_, cudaMemcpyDeviceToDevice, s_);
  } else if(opt.precond >= 3) {
    apply_mg<double>(cur64_, r, z, done);
  } else if(opt.precond == 2) {
    ::feng::launch_k(k_jacobi<double, double>, grid_for(n_, 256, 4096), 256, 0, s_, n_, diag_, r, z, done);
  } else {
    ilu_solve_levels<double, double>(r, z, done);
  }
}

void Krylov::precond32(const float *r, float *z, const int *done)
{
  if(opt.precond == 0) {
    cudaMemcpyAsync(z, r, sizeof(float) * n_, cudaMemcpyDeviceToDevice, s_);
  } else if(opt.precond >= 3) {
    apply_mg<float>(cur32_, r, z, done);
  } else if(opt.precond == 2) {
    ::feng::launch_k(k_jacobi<float, float>, grid_for(n_, 256, 4096), 256, 0, s_, n_, diag32_, r, z, done);
  } else {
    ilu_solve_levels<float, float>(r, z, done);
  }
}


template <typename VA, typename VX, typename VY, typename ACC, bool RESID>
static void spmv_launch(int lanes, int64_t n, const DeviceCSR &A, const VA *a, const VX *x,
                        const double *b, VY *y, const int *done, cudaStream_t s)
{
  const int64_t threads = n * lanes;
  const int grid = (int)((threads + 255) / 256);
  if(lanes == 16)
    ::feng::launch_k(k_spmv<VA, VX, VY, ACC, 16, RESID>, grid, 256, 0, s, n, A.ia, A.ja, a, x, b, y, done);
  else if(lanes == 8)
    ::feng::launch_k(k_spmv<VA, VX, VY, ACC, 8, RESID>, grid, 256, 0, s, n, A.ia, A.ja, a, x, b, y, done);
  else
    ::feng::launch_k(k_spmv<VA, VX, VY, ACC, 4, RESID>, grid, 256, 0, s, n, A.ia, A.ja, a, x, b, y, done);
}

void Krylov::spmv64(const double *values, const double *x, double *y)
{
  spmv_launch<double, double, double, double, false>(lanes_, n_, A_, values, x, nullptr, y,
                                                     nullptr, s_);
}

void Krylov::spmv32(const float *values, const double *x, double *y)
{
  const int gv = grid_for(n_, 256, 2048);
  ::feng::launch_k(k_to_f32, gv, 256, 0, s_, n_, x, v32_, nullptr);
  spmv_launch<float, float, double, float, false>(lanes_, n_, A_, values, v32_, nullptr, y, nullptr, s_);
}

int Krylov::spmvHot()
{
  if(!opt.mixed || !Z32_) {
    set_error("no mixed-precision FGMRES");
    return FE_INVALID_ARG;
  }
  if(sellVal_) spmv_sell(Z32_, w32_, nullptr);
  else if(cur32_) spmv_launch<float, float, float, float, false>(lanes_, n_, A_, cur32_, Z32_, nullptr, w32_, nullptr, s_);
  return FE_OK;
}

int Krylov::precondGraph(int reps, double *avgMs)
{
  if(!factoredOk_ || reps < 1 || !avgMs) {
    set_error("preconditioner not built, or an invalid benchmark request");
    return FE_INVALID_ARG;
  }
  if(opt.mixed && (!V32_ || !Z32_)) {
    set_error("no mixed FP32 basis");
    return FE_INVALID_ARG;
  }
  cudaGraph_t graph;
  cudaGraphExec_t exec;
  CK(cudaStreamBeginCapture(s_, cudaStreamCaptureModeThreadLocal));
  ++g_capturing;
  for(int r = 0; r < reps; ++r) {
    if(opt.mixed) precond32(vc32_, Z32_, nullptr);
    else precond64(V_, Z_, nullptr);
  }
  --g_capturing;
  CK(cudaStreamEndCapture(s_, &graph));
  CK(cudaGraphInstantiate(&exec, graph, 0));
  cudaEvent_t a, b;
  CK(cudaEventCreate(&a));
  CK(cudaEventCreate(&b));
  CK(cudaGraphLaunch(exec, s_));  // warm replay
  CK(cudaEventRecord(a, s_));
  CK(cudaGraphLaunch(exec, s_));
  CK(cudaEventRecord(b, s_));
  CK(cudaEventSynchronize(b));
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, a, b));
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaGraphExecDestroy(exec);
  cudaGraphDestroy(graph);
  CK(cudaGetLastError());
  *avgMs = ms / reps;
  return FE_OK;
}

int Krylov::cycleGraph(bool mixed, const void *vals, const double *b, double *x, int reps, double *msPerStep)
{
  if(reps < 1 || !msPerStep || !useGraphs_ || opt.method != 1) {
    set_error("an invalid benchmark request (FGMRES with CUDA graphs)");
    return FE_INVALID_ARG;
  }
  const double saved = *htol_;
  *htol_ = 0.;  // never converged: every kernel of the m steps runs
  const int m = opt.restart;
  cudaEvent_t a, e;
  CK(cudaEventCreate(&a));
  CK(cudaEventCreate(&e));
  int st = run_cycle(mixed, vals, b, x, m);  // capture + warm replay
  float ms = 0.f;
  if(st == FE_OK) {
    CK(cudaEventRecord(a, s_));
    for(int r = 0; r < reps && st == FE_OK; ++r) st = run_cycle(mixed, vals, b, x, m);
    CK(cudaEventRecord(e, s_));
    CK(cudaEventSynchronize(e));
    CK(cudaEventElapsedTime(&ms, a, e));
  }
  cudaEventDestroy(a);
  cudaEventDestroy(e);
  *htol_ = saved;
  *msPerStep = ms / ((double)reps * m);
  return st;
}

// r = b - A x for the FP32 matrix with FP64 x and accumulation: the sliced
// copy when it is built (it holds the same values), else the CSR kernel.
void Krylov::resid32(const float *vals, const double *x, const double *b, double *r)
{
  if(sellVal_ && xs2_ && dfResid_) {
    ::feng::launch_k(k_split_x, grid_for(n_, 256, 4096), 256, 0, s_, n_, x, (float2 *)xs2_);
    ::feng::launch_k(k_resid_sell_df<8>, grid_for(n_, 256, 1 << 20), 256, 0, s_, n_, sellPtr_, sellCol_, sellVal_,
                     (const float2 *)xs2_, b, r);
  } else if(sellVal_)
    ::feng::launch_k(k_resid_sell<8>, grid_for(n_, 256, 1 << 20), 256, 0, s_, n_, sellPtr_, sellCol_, sellVal_, x, b,
                     r);
  else
    spmv_launch<float, double, double, double, true>(lanes_, n_, A_, vals, x, b, r, nullptr, s_);
}

void Krylov::spmv_sell(const float *x, float *y, const int *done)
{
  ::feng::launch_k(k_spmv_sell<8>, grid_for(n_, 256, 1 << 20), 256, 0, s_, n_, sellPtr_, sellCol_, sellVal_, x, y,
                   done);
}

__global__ void k_f32_to_f64(int64_t n, const float *__restrict__ x, double *__restrict__ y)
{
  FE_PDL_ENTRY();
  for(int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = (double)x[i];
}

int Krylov::applyPrecond(const double *r, double *z)
{
  if(!factoredOk_) {
    set_error("preconditioner not built");
    return FE_PC_FAILED;
  }
  if(opt.mixed) {
    const int gv = grid_for(n_, 256, 2048);
    float *zf = Z32_ ? Z32_ : w32_;
    ::feng::launch_k(k_to_f32, gv, 256, 0, s_, n_, r, v32_, nullptr);
    precond32(v32_, zf, nullptr);
    if(z) ::feng::launch_k(k_f32_to_f64, gv, 256, 0, s_, n_, zf, z);
  } else {
    precond64(r, z, nullptr);
  }
  return FE_OK;
}

double Krylov::dot(const double *x, const double *y)
{
  Ws w = Ws_INIT(this);
  ::feng::launch_k(k_dot, nParts_, RB, 0, s_, n_, x, y, red_, w.st, dsum_);
  cudaMemcpyAsync(hred_, dsum_, sizeof(double), cudaMemcpyDeviceToHost, s_);
  cudaStreamSynchronize(s_);
  return hred_[0];
}

double Krylov::norm2(const double *x) { return sqrt(dot(x, x)); }

double Krylov::norminf(const double *x)
{
  Ws w = Ws_INIT(this);
  ::feng::launch_k(k_absmax, nParts_, RB, 0, s_, n_, x, red_, w.st, dsum_);
  cudaMemcpyAsync(hred_, dsum_, sizeof(double), cudaMemcpyDeviceToHost, s_);
  cudaStreamSynchronize(s_);
  return hred_[0];
}

int Krylov::gsStep(int mode, int ncols, int64_t *bytes)
{
  if(!V32_ || (mode != 0 && mode != 4 && mode != 6) || ncols < 1 || ncols > opt.restart) {
    set_error("no mixed FP32 basis, or an invalid Gram-Schmidt request");
    return FE_INVALID_ARG;
  }
  if(!zeroFlag_) {
    CK(cudaMalloc(&zeroFlag_, sizeof(int)));
    CK(cudaMemsetAsync(zeroFlag_, 0, sizeof(int), s_));
  }
  Ws w = Ws_INIT(this);
  if(mode == 4) gs32(4, ncols, w.gs->hcur, nullptr, w.gs->H + ncols, zeroFlag_, 0);
  else gs32(mode, ncols, nullptr, w.gs->hcur, w.gs->H, zeroFlag_, 0);
  // dots: ncols columns and w read; update: ncols columns and w read, w
  // written
  if(bytes) *bytes = (int64_t)(ncols + (mode == 4 ? 2 : 1)) * ld32_ * (int64_t)sizeof(float);
  return FE_OK;
}

int Krylov::gsStepStream(int mode, int ncols, int reps, double *avgMs)
{
  if(!V32_ || (mode != 0 && mode != 4) || ncols < 1 || ncols > opt.restart || reps < 1 ||
     !avgMs) {
    set_error("no mixed FP32 basis, or an invalid Gram-Schmidt request");
    return FE_INVALID_ARG;
  }
  if(!zeroFlag_) {
    CK(cudaMalloc(&zeroFlag_, sizeof(int)));
    CK(cudaMemsetAsync(zeroFlag_, 0, sizeof(int), s_));
  }
  int dev = 0, l2 = 0;
  CK(cudaGetDevice(&dev));
  CK(cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, dev));
  // one copy: the row-blocked basis (the pass reads ncols columns of every
  // row block) and w
  const size_t colBytes = sizeof(float) * (size_t)ld32_;
  const size_t basisBytes = (size_t)(opt.restart + 1) * colBytes;
  const size_t per = basisBytes + colBytes;
  const int copies = (int)std::max<size_t>(2, (3 * (size_t)l2) / per + 1);
  char *buf = nullptr;
  CK(cudaMalloc(&buf, per * copies));
  for(int c = 0; c < copies; ++c) {
    CK(cudaMemcpyAsync(buf + per * c, V32_, basisBytes, cudaMemcpyDeviceToDevice, s_));
    CK(cudaMemcpyAsync(buf + per * c + basisBytes, w32_, colBytes, cudaMemcpyDeviceToDevice, s_));
  }
  float *V0 = V32_, *w0 = w32_;
  Ws w = Ws_INIT(this);
  cudaEvent_t a, b;
  CK(cudaEventCreate(&a));
  CK(cudaEventCreate(&b));
  auto pass = [&](int c) {
    V32_ = (float *)(buf + per * c);
    w32_ = (float *)(buf + per * c + basisBytes);
    if(mode == 0) gs32(0, ncols, nullptr, w.gs->hcur, w.gs->H, zeroFlag_, 0);
    else gs32(4, ncols, w.gs->hcur, nullptr, w.gs->H + ncols, zeroFlag_, 0);
  };
  for(int c = 0; c < copies; ++c) pass(c);  // warm-up round
  CK(cudaEventRecord(a, s_));
  for(int r = 0; r < reps; ++r) pass(r % copies);
  CK(cudaEventRecord(b, s_));
  V32_ = V0;
  w32_ = w0;
  CK(cudaEventSynchronize(b));
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, a, b));
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(buf);
  *avgMs = ms / reps;
  return FE_OK;
}

// One FP32 Gram-Schmidt pass over the first ncols basis vectors: mode 0 the
// dot pass (k_gs_dots), 5 the dot pass with the Pythagoras norm, 1 update +
// dots, 2 update + norm (k_gs32), 3 the update that writes the next basis
// vector, 4 update + norm (k_gs_upd), 6 the dot pass by column groups
// (k_gs_dots; mode 0 runs k_gs_dots_all unless FENG_GS_DOTS=groups).
void Krylov::gs32(int mode, int ncols, const double *hprev, double *hcur, double *Hcol, const int *done, int pass)
{
  RedState *st = (RedState *)red_state_;
  const int g = gsParts_;
  const int64_t n4 = ld32_ / 4;
  const int m1 = opt.restart + 1;  // columns per row block of the basis
  const int gu = (int)std::max<int64_t>(1, std::min<int64_t>((n4 + RB - 1) / RB, 4 * nSM_));
#define FE_GS_LAUNCH(C)                                                                                         \
  do {                                                                                                          \
    if(mode == 0)                                                                                               \
      ::feng::launch_k(k_gs32<C, 0>, g, RB, 0, s_, n4, m1, V32_, ncols, hprev, w32_, red_, st, hcur, Hcol, done, pass); \
    else if(mode == 1)                                                                                          \
      ::feng::launch_k(k_gs32<C, 1>, g, RB, 0, s_, n4, m1, V32_, ncols, hprev, w32_, red_, st, hcur, Hcol, done, pass); \
    else if(mode == 2)                                                                                          \
      ::feng::launch_k(k_gs32<C, 2>, g, RB, 0, s_, n4, m1, V32_, ncols, hprev, w32_, red_, st, hcur, Hcol, done, pass); \
    else if(mode == 3)                                                                                          \
      ::feng::launch_k(k_gs_upd<C, false>, gu, RB, 0, s_, n4, m1, V32_, ncols, hprev, w32_, vc32_, st, red_, nullptr, done, 0); \
    else                                                                                                        \
      ::feng::launch_k(k_gs_upd<C, true>, gu, RB, 0, s_, n4, m1, V32_, ncols, hprev, w32_, nullptr, st, red_, Hcol, done, pass); \
  } while(0)
  if(mode == 0 && allDots_) {
    // one pass over w and every column (k_gs_dots_all), one wave of four
    // blocks per SM over the slices of 16 columns
    const int gy = (ncols + 15) / 16;
    const int gd = (int)std::max<int64_t>(
        1, std::min<int64_t>({(n4 + RB - 1) / RB, (int64_t)(4 * nSM_ + gy - 1) / gy, (int64_t)MAXRED}));
#define FE_GSA_LAUNCH(C)                                                                                    \
  ::feng::launch_k(k_gs_dots_all<C>, dim3(gd, gy), RB, 0, s_, n4, m1, V32_, ncols, w32_, red_, st, hcur, Hcol, done, pass)
    if(ncols <= 8) FE_GSA_LAUNCH(8);
    else FE_GSA_LAUNCH(16);
#undef FE_GSA_LAUNCH
    return;
  }
  if(mode == 0 || mode == 5 || mode == 6) {
    // mode 5: the dot pass that also takes the norm of the update by Pythagoras
    // about four blocks per SM in all: each block loops over several row
    // groups (fewer partials, one counter increment per block)
    const int gy = (ncols + 7) / 8;
    const int64_t gx = std::max<int64_t>(
        1, std::min<int64_t>({(n4 + RB - 1) / RB, (int64_t)MAXRED, (int64_t)(4 * nSM_ + gy - 1) / gy}));
    const dim3 gb((unsigned)gx, (unsigned)gy);
    ::feng::launch_k(k_gs_dots, gb, RB, 0, s_, n4, m1, V32_, ncols, w32_, red_, st, hcur, Hcol, done, pass, mode == 5 ? 1 : 0);
    return;
  }
  if(ncols <= 8) FE_GS_LAUNCH(8);
  else if(ncols <= 16) FE_GS_LAUNCH(16);
  else if(ncols <= 32) FE_GS_LAUNCH(32);
  else FE_GS_LAUNCH(64);
#undef FE_GS_LAUNCH
}

// FGMRES(m), right preconditioned, FP64 throughout (Saad Alg. 9.6).
// One FGMRES(m) restart cycle (Saad Alg. 9.6): r = b - A x, V_0 = r/||r||,
// then up to jmax Arnoldi steps with right preconditioning z_j = M^-1 v_j,
// classical Gram-Schmidt applied twice, Givens rotations on the device.
// Every kernel after convergence is skipped through the device done flag,
// so the same launch sequence can be replayed from a CUDA graph.
void Krylov::launch_cycle(bool mixed, const void *vals, const double *b, double *x, int jmax, bool poll)
{
  Ws w = Ws_INIT(this);
  const int gv = grid_for(n_, 256, 2048);
  if(mixed) {
    launch_cycle_mixed((const float *)vals, b, x, jmax, poll);
    return;
  }
  spmv_launch<double, double, double, double, true>(lanes_, n_, A_, (const double *)vals, x, b, w_, nullptr, s_);
  cudaMemsetAsync(&w.gs->done, 0, sizeof(int), s_);
  cudaMemcpyAsync(&w.gs->tol, htol_, sizeof(double), cudaMemcpyHostToDevice, s_);
  ::feng::launch_k(k_norm_to, nParts_, RB, 0, s_, n_, w_, red_, w.st, &w.gs->done);
  ::feng::launch_k(k_gmres_init, 1, 1, 0, s_, w.gs, w.st);
  ::feng::launch_k(k_scale_from, gv, 256, 0, s_, n_, w_, V_, w.st, &w.gs->beta, &w.gs->done);
  for(int j = 0; j < jmax; ++j) {
    double *vj = V_ + (int64_t)j * n_;
    {
      double *zj = Z_ + (int64_t)j * n_;
      precond64(vj, zj, &w.gs->done);
      spmv_launch<double, double, double, double, false>(lanes_, n_, A_, (const double *)vals, zj, nullptr,
                                                         w_, &w.gs->done, s_);
    }
    double *Hcol = w.gs->H + (int64_t)j * (MAXM + 1);
    for(int pass = 0; pass < 2; ++pass) {
      ::feng::launch_k(k_mdot_partial, dim3(nParts_, j + 1), RB, 0, s_, n_, V_, j + 1, w_, red_, &w.gs->done);
      ::feng::launch_k(k_mdot_final, j + 1, RB, 0, s_, nParts_, red_, w.gs->hcur, Hcol, pass, &w.gs->done);
      ::feng::launch_k(k_mupdate, gv, 256, 0, s_, n_, V_, j + 1, w.gs->hcur, w_, &w.gs->done);
    }
    ::feng::launch_k(k_norm_to, nParts_, RB, 0, s_, n_, w_, red_, w.st, &w.gs->done);
    ::feng::launch_k(k_scale_from, gv, 256, 0, s_, n_, w_, V_ + (int64_t)(j + 1) * n_, w.st, Hcol + j + 1, &w.gs->done);
    ::feng::launch_k(k_givens, 1, 32, 0, s_, w.gs, j);
    if(poll && poll_done(&w.gs->done, j)) break;
  }
  ::feng::launch_k(k_backsolve, 1, 256, backsolveSmem(opt.restart), s_, w.gs);
  ::feng::launch_k(k_xupdate<double>, gv, 256, 0, s_, n_, n_, Z_, w.gs, x);
  cudaMemcpyAsync(h_gmres_, w.gs, sizeof(GmresHead), cudaMemcpyDeviceToHost, s_);
}

// One mixed-precision restart cycle: the residual b - A x with FP64
// accumulation (iterative refinement), then Arnoldi on an FP32 basis: FP32
// preconditioner and SpMV, classical Gram-Schmidt in FP32 with FP64 partial
// sums (a dot pass, then a fused update + norm pass; gsPasses = 2 adds the
// fused update + dot pass of the second orthogonalisation), FP64 Hessenberg
// and Givens rotations, FP64 solution update.
void Krylov::launch_cycle_mixed(const float *vals, const double *b, double *x, int jmax, bool poll)
{
  mixed_part(vals, b, x, 0, jmax, poll, true, true);
}

// Part of a mixed restart cycle: the prologue (restart residual, its norm,
// v_0) when `pro`, the Arnoldi steps j0 <= j < j1, the epilogue
// (back-substitution, x update, head copy) when `epi`.
void Krylov::mixed_part(const float *vals, const double *b, double *x, int j0, int j1, bool poll, bool pro, bool epi)
{
  Ws w = Ws_INIT(this);
  const int gv = grid_for(n_, 256, 2048);
  const int m1 = opt.restart + 1;
  if(pro) {
  resid32(vals, x, b, w_);
  cudaMemsetAsync(&w.gs->done, 0, sizeof(int), s_);
  cudaMemcpyAsync(&w.gs->tol, htol_, sizeof(double), cudaMemcpyHostToDevice, s_);
  ::feng::launch_k(k_norm_to, nParts_, RB, 0, s_, n_, w_, red_, w.st, &w.gs->done);
  ::feng::launch_k(k_gmres_init, 1, 1, 0, s_, w.gs, w.st);
  ::feng::launch_k(k_scale_r32, gv, 256, 0, s_, n_, w_, V32_, m1, vc32_, w.st, &w.gs->beta, &w.gs->done);
  }
  const int g4 = grid_for(ld32_ / 4, 256, 4 * 152);
  for(int j = j0; j < j1; ++j) {
    // v_j: the contiguous copy written with basis column j
    const float *vj = vc32_;
    float *zj = Z32_ + (int64_t)j * ld32_;
    precond32(vj, zj, &w.gs->done);
    double *Hcol = w.gs->H + (int64_t)j * (MAXM + 1);
    if(sellVal_)
      spmv_sell(zj, w32_, &w.gs->done);
    else
      spmv_launch<float, float, float, float, false>(lanes_, n_, A_, vals, zj, nullptr, w32_, &w.gs->done, s_);
    if(opt.gsPasses == 2) {
      // always twice: dots, fused update + dots, update + norm
      gs32(0, j + 1, nullptr, w.gs->hcur, Hcol, &w.gs->done, 0);
      gs32(1, j + 1, w.gs->hcur, w.gs->hcur, Hcol, &w.gs->done, 0);
      gs32(2, j + 1, w.gs->hcur, nullptr, Hcol + j + 1, &w.gs->done, 2);
    } else if(opt.gsPasses == 3) {
      // once, the norm of the update by Pythagoras from the dot pass and the
      // next basis vector written by the update pass; a second time only
      // when the update kept less than a tenth of ||w|| (decided on the
      // device, so the replayed graph is fixed): the update goes back to w,
      // the second dot pass, update + norm pass and scale pass run.
      gs32(5, j + 1, nullptr, w.gs->hcur, Hcol, &w.gs->done, 0);
      gs32(3, j + 1, w.gs->hcur, nullptr, nullptr, &w.gs->done, 0);
      gs32(0, j + 1, nullptr, w.gs->hcur, Hcol, &w.gs->done, 1);
      gs32(4, j + 1, w.gs->hcur, nullptr, Hcol + j + 1, &w.gs->done, 1);
    } else {
      // once (dot pass, update + norm pass), and a second time only when
      // the update kept less than a tenth of ||w|| (decided on the device,
      // so the replayed graph is fixed)
      gs32(0, j + 1, nullptr, w.gs->hcur, Hcol, &w.gs->done, 0);
      gs32(4, j + 1, w.gs->hcur, nullptr, Hcol + j + 1, &w.gs->done, 0);
      gs32(0, j + 1, nullptr, w.gs->hcur, Hcol, &w.gs->done, 1);
      gs32(4, j + 1, w.gs->hcur, nullptr, Hcol + j + 1, &w.gs->done, 1);
    }
    if(opt.gsPasses == 3) {
      // gated scale (only after a second pass), then the rotations
      ::feng::launch_k(k_scale32, g4, 256, 0, s_, ld32_ / 4, w32_, V32_, m1, j + 1, vc32_, w.st, &w.gs->done, 1,
                       (GmresState *)nullptr, 0);
      ::feng::launch_k(k_givens, 1, 32, 0, s_, w.gs, j);
    } else {
      ::feng::launch_k(k_scale32, g4 + 1, 256, 0, s_, ld32_ / 4, w32_, V32_, m1, j + 1, vc32_, w.st, &w.gs->done, 0,
                       w.gs, j);
    }
    if(poll && poll_done(&w.gs->done, j)) break;
  }
  if(!epi) return;
  ::feng::launch_k(k_backsolve, 1, 256, backsolveSmem(opt.restart), s_, w.gs);
  ::feng::launch_k(k_xupdate<float>, gv, 256, 0, s_, n_, ld32_, Z32_, w.gs, x);
  cudaMemcpyAsync(h_gmres_, w.gs, sizeof(GmresHead), cudaMemcpyDeviceToHost, s_);
}

// Runs one full restart cycle, from a CUDA graph when the cycle has its full
// length (the graph is captured once per operand set and replayed).
// A graph per part of the mixed cycle (part c: steps [cK, cK + K), the
// prologue with part 0, then a copy of the done flag to pinned memory;
// part P: the epilogue), looked up or captured.
int Krylov::part_graph(const GraphKey &key, int part, int P, int K, const float *vals, const double *b, double *x,
                       cudaGraphExec_t *out, size_t *nKernels)
{
  for(size_t i = 0; i < graphs_.size(); ++i) {
    const GraphKey &g = graphs_[i].first;
    if(g.mixed == key.mixed && g.vals == key.vals && g.b == key.b && g.x == key.x && g.dfResid == key.dfResid &&
       g.part == part) {
      *nKernels = graphKernels_[i];
      *out = graphs_[i].second;
      return FE_OK;
    }
  }
  const int m = opt.restart;
  cudaGraph_t graph;
  cudaGraphExec_t exec = nullptr;
  CK(cudaStreamBeginCapture(s_, cudaStreamCaptureModeThreadLocal));
  ++g_capturing;
  if(part == P) {
    mixed_part(vals, b, x, 0, 0, false, false, true);
  } else {
    mixed_part(vals, b, x, part * K, std::min(m, part * K + K), false, part == 0, false);
    Ws w = Ws_INIT(this);
    cudaMemcpyAsync(hdone_ + part, &w.gs->done, sizeof(int), cudaMemcpyDeviceToHost, s_);
  }
  --g_capturing;
  CK(cudaStreamEndCapture(s_, &graph));
  CK(cudaGraphInstantiate(&exec, graph, 0));
  size_t nn = 0, nk = 0;
  CK(cudaGraphGetNodes(graph, nullptr, &nn));
  std::vector<cudaGraphNode_t> nodes(nn);
  CK(cudaGraphGetNodes(graph, nodes.data(), &nn));
  for(auto nd : nodes) {
    cudaGraphNodeType t;
    CK(cudaGraphNodeGetType(nd, &t));
    if(t == cudaGraphNodeTypeKernel) ++nk;
  }
  cudaGraphDestroy(graph);
  GraphKey k2 = key;
  k2.part = part;
  graphs_.push_back({k2, exec});
  graphKernels_.push_back(nk);
  *nKernels = nk;
  *out = exec;
  return FE_OK;
}

// One full mixed restart cycle from part graphs of chunk_ Arnoldi steps:
// part c + 1 is queued before the done flag of part c is read, so the GPU
// always has work and a converged cycle stops within one part (instead of
// replaying every remaining step's kernels, which return at once).
int Krylov::run_cycle_chunked(const float *vals, const double *b, double *x)
{
  const int m = opt.restart, K = chunk_, P = (m + K - 1) / K;
  GraphKey key{true, vals, b, x, dfResid_, -1};
  if(evs_.size() < (size_t)P) {
    for(size_t i = evs_.size(); i < (size_t)P; ++i) {
      cudaEvent_t e;
      CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
      evs_.push_back(e);
    }
  }
  size_t nk = 0;
  for(int c = 0; c < P; ++c) {
    cudaGraphExec_t ex = nullptr;
    FE_TRY(part_graph(key, c, P, K, vals, b, x, &ex, &nk));
    CK(cudaGraphLaunch(ex, s_));
    g_launches.fetch_add((long long)nk, std::memory_order_relaxed);
    CK(cudaEventRecord(evs_[c], s_));
    if(c > 0) {
      CK(cudaEventSynchronize(evs_[c - 1]));
      if(hdone_[c - 1]) break;
    }
  }
  cudaGraphExec_t ex = nullptr;
  FE_TRY(part_graph(key, P, P, K, vals, b, x, &ex, &nk));
  CK(cudaGraphLaunch(ex, s_));
  g_launches.fetch_add((long long)nk, std::memory_order_relaxed);
  CK(cudaStreamSynchronize(s_));
  CK(cudaGetLastError());
  return FE_OK;
}

int Krylov::run_cycle(bool mixed, const void *vals, const double *b, double *x, int jmax)
{
  const int m = opt.restart;
  if(useGraphs_ && jmax == m && mixed && chunk_ > 0 && chunk_ < m) return run_cycle_chunked((const float *)vals, b, x);
  if(useGraphs_ && jmax == m) {
    GraphKey key{mixed, vals, b, x, mixed && dfResid_, -1};
    cudaGraphExec_t exec = nullptr;
    for(auto &g : graphs_)
      if(g.first.mixed == key.mixed && g.first.vals == key.vals && g.first.b == key.b && g.first.x == key.x &&
         g.first.dfResid == key.dfResid && g.first.part == -1)
        exec = g.second;
    size_t nKernels = 0;
    if(!exec) {
      cudaGraph_t graph;
      CK(cudaStreamBeginCapture(s_, cudaStreamCaptureModeThreadLocal));
      ++g_capturing;
      launch_cycle(mixed, vals, b, x, m, false);
      --g_capturing;
      CK(cudaStreamEndCapture(s_, &graph));
      CK(cudaGraphInstantiate(&exec, graph, 0));
      size_t nn = 0;
      CK(cudaGraphGetNodes(graph, nullptr, &nn));
      std::vector<cudaGraphNode_t> nodes(nn);
      CK(cudaGraphGetNodes(graph, nodes.data(), &nn));
      for(auto nd : nodes) {
        cudaGraphNodeType t;
        CK(cudaGraphNodeGetType(nd, &t));
        if(t == cudaGraphNodeTypeKernel) ++nKernels;
      }
      cudaGraphDestroy(graph);
      graphs_.push_back({key, exec});
      graphKernels_.push_back(nKernels);
    } else {
      for(size_t i = 0; i < graphs_.size(); ++i)
        if(graphs_[i].second == exec) nKernels = graphKernels_[i];
    }
    CK(cudaGraphLaunch(exec, s_));
    g_launches.fetch_add((long long)nKernels, std::memory_order_relaxed);
  } else {
    launch_cycle(mixed, vals, b, x, jmax, true);
  }
  CK(cudaStreamSynchronize(s_));
  CK(cudaGetLastError());
  return FE_OK;
}

int Krylov::solve_fgmres64(const double *vals, const double *b, double *x, double tolAbs, int maxIt,
                           KrylovStats &st)
{
  const GmresHead *hd = (const GmresHead *)h_gmres_;
  int total = 0;
  *htol_ = tolAbs;
  while(true) {
    FE_TRY(run_cycle(false, vals, b, x, std::min(opt.restart, maxIt - total)));
    total += hd->k;
    st.iterations = total;
    st.rnorm = hd->est;
    if(!std::isfinite(hd->est)) { set_error("non-finite residual in FGMRES"); return FE_NONFINITE; }
    if(hd->est <= tolAbs) break;
    if(total >= maxIt || hd->k == 0) break;
    if(hd->est > opt.dtol * std::max(st.rnorm0, 1e-300)) { set_error("FGMRES diverged"); return FE_NOT_CONVERGED; }
  }
  // Converged on the Arnoldi estimate (as PETSc's default test); report the
  // true residual alongside.
  const bool conv = hd->est <= tolAbs;
  spmv_launch<double, double, double, double, true>(lanes_, n_, A_, vals, x, b, w_, nullptr, s_);
  st.rnorm = norm2(w_);
  return conv ? FE_OK : FE_NOT_CONVERGED;
}

// FGMRES with FP32 matrix, SpMV and preconditioner, FP64 Krylov basis and
// Gram-Schmidt; every restart recomputes the true residual b - A x with FP64
// accumulation (iterative refinement).
int Krylov::solve_fgmres_mixed(const float *vals32, const double *b, double *x, double tolAbs,
                               int maxIt, KrylovStats &st)
{
  const GmresHead *hd = (const GmresHead *)h_gmres_;
  int total = 0;
  *htol_ = tolAbs;
  dfResid_ = tolAbs >= 1e-9 * st.rnorm0;
  while(true) {
    FE_TRY(run_cycle(true, vals32, b, x, std::min(opt.restart, maxIt - total)));
    st.refinements++;
    total += hd->k;
    st.iterations = total;
    if(!std::isfinite(hd->est)) { set_error("non-finite residual in mixed FGMRES"); return FE_NONFINITE; }
    // Refinement check on the true residual.
    resid32(vals32, x, b, w_);
    st.rnorm = norm2(w_);
    if(st.rnorm <= tolAbs) break;
    if(total >= maxIt || hd->k == 0) break;
    if(st.rnorm > opt.dtol * std::max(st.rnorm0, 1e-300)) { set_error("mixed FGMRES diverged"); return FE_NOT_CONVERGED; }
  }
  return st.rnorm <= tolAbs * 1.0000001 + 1e-300 ? FE_OK : FE_NOT_CONVERGED;
}

// Preconditioned CG (Saad Alg. 9.1) with device-resident scalars; the host
// polls convergence every 8 iterations.
int Krylov::solve_cg64(const double *vals, const double *b, double *x, double tolAbs, int maxIt,
                       KrylovStats &st)
{
  Ws w = Ws_INIT(this);
  const int gv = grid_for(n_, 256, 2048);
  // x = 0, r = b
  ::feng::launch_k(k_zero, gv, 256, 0, s_, n_, x);
  ::feng::launch_k(k_copy, gv, 256, 0, s_, n_, b, r_);
  CGState init{};
  init.tol = tolAbs;
  init.done = 0;
  cudaMemcpyAsync(w.cg, &init, sizeof(CGState), cudaMemcpyHostToDevice, s_);
  // z = M r ; rz = r.z ; p = z
  precond64(r_, t_, &w.cg->done);
  ::feng::launch_k(k_dot_if, nParts_, RB, 0, s_, n_, r_, t_, red_, w.st, w.cg);
  ::feng::launch_k(k_cg_p, gv, 256, 0, s_, n_, w.cg, w.st, t_, p_, 1);
  ::feng::launch_k(k_cg_rz, 1, 1, 0, s_, w.cg, w.st);
  int it = 0;
  while(it < maxIt) {
    const int batch = std::min(8, maxIt - it);
    for(int k = 0; k < batch; ++k) {
      spmv_launch<double, double, double, double, false>(lanes_, n_, A_, vals, p_, nullptr, q_,
                                                         &w.cg->done, s_);
      ::feng::launch_k(k_dot_if, nParts_, RB, 0, s_, n_, p_, q_, red_, w.st, w.cg);
      ::feng::launch_k(k_cg_pq, 1, 1, 0, s_, w.cg, w.st);
      ::feng::launch_k(k_cg_xr, nParts_, RB, 0, s_, n_, w.cg, p_, q_, x, r_, red_, w.st);
      ::feng::launch_k(k_cg_check, 1, 1, 0, s_, w.cg, w.st);
      precond64(r_, t_, &w.cg->done);
      ::feng::launch_k(k_dot_if, nParts_, RB, 0, s_, n_, r_, t_, red_, w.st, w.cg);
      ::feng::launch_k(k_cg_p, gv, 256, 0, s_, n_, w.cg, w.st, t_, p_, 0);
      ::feng::launch_k(k_cg_rz, 1, 1, 0, s_, w.cg, w.st);
    }
    it += batch;
    cudaMemcpyAsync(w.hcg, w.cg, sizeof(CGState), cudaMemcpyDeviceToHost, s_);
    CK(cudaStreamSynchronize(s_));
    CK(cudaGetLastError());
    if(w.hcg->done) break;
  }
  st.iterations = w.hcg->it;
  st.rnorm = sqrt(w.hcg->rr);
  if(!std::isfinite(st.rnorm)) { set_error("non-finite residual in CG"); return FE_NONFINITE; }
  return st.rnorm <= tolAbs * 1.0000001 ? FE_OK : FE_NOT_CONVERGED;
}

int Krylov::solve(const double *values64, const float *values32, const double *b, double *x,
                  KrylovStats &st)
{
  st = KrylovStats();
  if(!factoredOk_) {
    set_error("preconditioner not built");
    return FE_PC_FAILED;
  }
  const double bn = norm2(b);
  st.rnorm0 = bn;
  if(!std::isfinite(bn)) { set_error("non-finite right-hand side"); return FE_NONFINITE; }
  const int gv = grid_for(n_, 256, 2048);
  ::feng::launch_k(k_zero, gv, 256, 0, s_, n_, x);
  const double tolAbs = std::max(opt.rtol * bn, opt.atol);
  if(bn <= opt.atol) { st.rnorm = bn; return FE_OK; }
  if(opt.method == 0) {
    if(opt.mixed) { set_error("CG runs in FP64 only"); return FE_INVALID_ARG; }
    return solve_cg64(values64, b, x, tolAbs, opt.maxIter, st);
  }
  if(opt.mixed) return solve_fgmres_mixed(values32, b, x, tolAbs, opt.maxIter, st);
  return solve_fgmres64(values64, b, x, tolAbs, opt.maxIter, st);
}

}  // namespace feng
