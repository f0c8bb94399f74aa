// Multigrid-based preconditioners of the Krylov solver (kinds 3 and 4 in
// fe_krylov.h): AMG V-cycles on the scalar P2 stiffness matrix, used directly
// for a scalar field or per velocity component inside the block
// upper-triangular saddle-point preconditioner
//     P = [ A  G ]      z_p = S^-1 r_p,   S^-1 ~ (mu / c_div) M_p^-1 (lumped)
//         [ 0  S ]      z_u = A^-1 (r_u - G z_p),  A^-1 ~ (s K)^-1 per component
// (Elman, Silvester, Wathen, "Finite Elements and Fast Iterative Solvers",
// 2nd ed., ch. 9: block preconditioning of the Oseen problem).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <memory>

#include "fe_amg.h"
#include "fe_common.h"
#include "fe_launch.h"
#include "fe_krylov.h"

namespace feng {

#define CKM(x)                                                                         \
  do {                                                                                 \
    cudaError_t _e = (x);                                                              \
    if(_e != cudaSuccess) {                                                            \
      set_error("CUDA error %s at %s:%d", cudaGetErrorString(_e), __FILE__, __LINE__); \
      return FE_CUDA_FAIL;                                                             \
    }                                                                                  \
  } while(0)

struct Krylov::MG {
  std::unique_ptr<AMGDevice> amg = std::make_unique<AMGDevice>();
  // Time-dependent problems: the stiffness and mass kept for re-set-ups,
  // the pressure Laplacian multigrid and the Cahouet-Chabard coefficient.
  HostCSR lapH, massH, lapPH;
  std::unique_ptr<AMGDevice> amgP;
  AMGParams params;
  double cc = 0.;
  void *pr = nullptr, *pz = nullptr;
  int kind = 0;
  int64_t nNodes = 0, nP = 0;
  int32_t *dofX = nullptr, *dofY = nullptr, *pRows = nullptr;
  // Tetrahedral Taylor-Hood: three components, slot q = 3 k + c of node k
  // is row dofC[q]; vectors bxy / zxy then hold the three components
  // interleaved.  nc = 2 on triangles (the paired kernels above).
  int nc = 2;
  int32_t *dofC = nullptr;
  double vfac = 1.5;  // diag(A_xx) / (mu diag(K)) of the symmetric-gradient operator: 1 + 1/dim
  int32_t *upIa = nullptr, *upPos = nullptr, *upCol = nullptr;  // G block, rows = velocity slot 2k+c
  void *gVals = nullptr;  // the G block's values, gathered contiguous at each factor()
  int64_t nG = 0;
  int32_t *dnIa = nullptr, *dnPos = nullptr, *dnCol = nullptr;  // D block, rows = pressure rows
  int32_t *slotOf = nullptr;                                     // velocity DOF -> slot 2k+c (-1 otherwise)
  double cMc = 0, cSc = 0;  // constant pressure mode: c^T M c and c^T S c (deflation)
  double *pMassDev = nullptr, *tP = nullptr;
  double *consts = nullptr;   // device: 1/s, c^T S c, c^T M c
  double hconst[4] = {1, 0, 0, 0};
  int32_t *diagX = nullptr;                                        // CSR position of diag of x rows
  double *pScale64 = nullptr;
  float *pScale32 = nullptr;
  void *bx = nullptr, *by = nullptr, *zx = nullptr, *zy = nullptr;
  void *bxy = nullptr, *zxy = nullptr;  // both components interleaved (paired V-cycle)
  double *dsum = nullptr;
  double lapDiagSum = 0, s = 1, sigma = 1, divu = 1;
  std::vector<double> pMass;
  int fp32 = 0;
  // Inner preconditioned CG on K (AMG V-cycle preconditioner), `inner`
  // iterations per component; 0 = a single V-cycle.
  int inner = 0;
  void *ir = nullptr, *iz = nullptr, *ip = nullptr, *iq = nullptr;
  double *part = nullptr;  // [2][1024] partial sums
  double *scal = nullptr;  // rz, pq
  unsigned *count = nullptr;  // blocks done of the fused pressure sum (k_psum)
  // Pressure fold (steady, two components, one V-cycle): G with its columns
  // scaled by the pressure scale (gScaled), the pressure index of each G
  // entry (upColP), u_k = 1/cSc - sc_k m_k / cMc (uP) and bgu = V(G u) (the
  // V-cycle of G u), so that z_u = (V(r_u - G (sc r_p)) - c bgu) / s without
  // z_p; see apply_mg.
  int32_t *upColP = nullptr;
  void *gScaled = nullptr, *bgu = nullptr;
  double *uP = nullptr;
  bool fold = false;
  ~MG()
  {
    cudaFree(dofX); cudaFree(dofY); cudaFree(pRows); cudaFree(upIa); cudaFree(upPos); cudaFree(upCol);
    cudaFree(diagX); cudaFree(pScale64); cudaFree(pScale32); cudaFree(bx); cudaFree(by); cudaFree(zx);
    cudaFree(zy); cudaFree(dsum); cudaFree(ir); cudaFree(iz); cudaFree(ip); cudaFree(iq);
    cudaFree(part); cudaFree(scal); cudaFree(dnIa); cudaFree(dnPos); cudaFree(dnCol); cudaFree(slotOf);
    cudaFree(pMassDev); cudaFree(tP); cudaFree(consts); cudaFree(bxy); cudaFree(zxy); cudaFree(gVals);
    cudaFree(pr); cudaFree(pz); cudaFree(count); cudaFree(dofC);
    cudaFree(upColP); cudaFree(gScaled); cudaFree(bgu); cudaFree(uP);
  }
  template <typename V> void solveK(const V *b, V *x, cudaStream_t st);
};

namespace {

constexpr int NPART = 512;

// The Schur complement approximation S^-1 ~ -SCHUR_FACTOR (s / (vfac sigma
// c_div)) M_p^-1: the viscous estimate (the velocity block ~ s K, so
// mu ~ -s / (vfac sigma)) scaled up for what convection and the Newton terms
// add to the velocity block.  Measured (FGMRES iterations; factor 1 / 3 / 6
// / 10): Kovasznay 256^2 555 / 364 / 331 / 327 per solve, 512^2 884 (1) /
// 489 (6) / 502 (8); cavity 384^2 64.0 / 50.6 / 49.3 per step (8: 52.6);
// 48^3 cube 66.8 / 47.5 / 40.3 per step (8: 39.5).
constexpr double SCHUR_FACTOR = 6.0;

template <typename V>
__global__ void k_dot_part(int64_t n, const V *__restrict__ a, const V *__restrict__ b, double *part)
{
  FE_PDL_ENTRY();
  __shared__ double sh[256];
  double s = 0.;
  for(int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    s += (double)a[i] * (double)b[i];
  sh[threadIdx.x] = s;
  __syncthreads();
  for(int o = 128; o > 0; o >>= 1) {
    if(threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if(threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

__global__ void k_dot_fin(int nparts, const double *__restrict__ part, double *out)
{
  FE_PDL_ENTRY();
  __shared__ double sh[256];
  double s = 0.;
  for(int i = threadIdx.x; i < nparts; i += blockDim.x) s += part[i];
  sh[threadIdx.x] = s;
  __syncthreads();
  for(int o = 128; o > 0; o >>= 1) {
    if(threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if(threadIdx.x == 0) *out = sh[0];
}

// x += alpha p, r -= alpha q with alpha = rz / pq (device scalars); a zero
// or non-finite pq leaves x, r unchanged.
template <typename V>
__global__ void k_pcg_xr(int64_t n, const double *__restrict__ scal, const V *__restrict__ p,
                         const V *__restrict__ q, V *__restrict__ x, V *__restrict__ r)
{
  FE_PDL_ENTRY();
  const double pq = scal[1];
  const double alpha = (pq != 0. && isfinite(pq)) ? scal[0] / pq : 0.;
  for(int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    x[i] += (V)alpha * p[i];
    r[i] -= (V)alpha * q[i];
  }
}

// p = z + beta p with beta = rz_new / rz (scal[2] / scal[0]); then rz = rz_new.
template <typename V>
__global__ void k_pcg_p(int64_t n, const double *__restrict__ scal, const V *__restrict__ z, V *__restrict__ p,
                        int first)
{
  FE_PDL_ENTRY();
  const double beta = (first || scal[0] == 0.) ? 0. : scal[2] / scal[0];
  for(int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    p[i] = z[i] + (V)beta * p[i];
}

__global__ void k_pcg_shift(double *scal) {
  FE_PDL_ENTRY(); scal[0] = scal[2]; }

template <typename V>
__global__ void k_copy_v(int64_t n, const V *__restrict__ a, V *__restrict__ b)
{
  FE_PDL_ENTRY();
  for(int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    b[i] = a[i];
}

__global__ void k_zero_d(int64_t n, double *x)
{
  FE_PDL_ENTRY();
  for(int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) x[i] = 0.;
}

}  // namespace

// x = K^-1 b approximately: one V-cycle, or `inner` steps of CG preconditioned
// by the V-cycle (Saad Alg. 9.1), all scalars kept on the device.
template <typename V>
void Krylov::MG::solveK(const V *b, V *x, cudaStream_t st)
{
  const int64_t n = nNodes;
  auto vc = [&](const V *in, V *out) {
    if constexpr(sizeof(V) == 8) amg->vcycle64(in, out);
    else amg->vcycle32(in, out);
  };
  auto spmv = [&](const V *in, V *out) {
    if constexpr(sizeof(V) == 8) amg->spmv64(in, out);
    else amg->spmv32(in, out);
  };
  if(inner <= 0) {
    vc(b, x);
    return;
  }
  const int g = (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 4096));
  const int gp = (int)std::min<int64_t>(NPART, std::max<int64_t>(1, (n + 255) / 256));
  V *r = (V *)ir, *z = (V *)iz, *p = (V *)ip, *q = (V *)iq;
  ::feng::launch_k(k_copy_v<V>, g, 256, 0, st, n, b, r);
  // x = 0 (written through r's type)
  if constexpr(sizeof(V) == 8) ::feng::launch_k(k_zero_d, g, 256, 0, st, n, (double *)x);
  else cudaMemsetAsync(x, 0, sizeof(float) * n, st);
  vc(r, z);
  ::feng::launch_k(k_dot_part<V>, gp, 256, 0, st, n, r, z, part);
  ::feng::launch_k(k_dot_fin, 1, 256, 0, st, gp, part, scal + 0);
  ::feng::launch_k(k_pcg_p<V>, g, 256, 0, st, n, scal, z, p, 1);
  for(int it = 0; it < inner; ++it) {
    spmv(p, q);
    ::feng::launch_k(k_dot_part<V>, gp, 256, 0, st, n, p, q, part);
    ::feng::launch_k(k_dot_fin, 1, 256, 0, st, gp, part, scal + 1);
    ::feng::launch_k(k_pcg_xr<V>, g, 256, 0, st, n, scal, p, q, x, r);
    if(it + 1 == inner) break;
    vc(r, z);
    ::feng::launch_k(k_dot_part<V>, gp, 256, 0, st, n, r, z, part);
    ::feng::launch_k(k_dot_fin, 1, 256, 0, st, gp, part, scal + 2);
    ::feng::launch_k(k_pcg_p<V>, g, 256, 0, st, n, scal, z, p, 0);
    ::feng::launch_k(k_pcg_shift, 1, 1, 0, st, scal);
  }
}

namespace {

int grid(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 1 << 16)); }

// partial sums of the entries a[pos[i]] (the finest velocity diagonal),
// one per block; k_dot_fin adds them in block order
template <typename VA>
__global__ void k_diag_part(int64_t n, const int32_t *__restrict__ pos, const VA *__restrict__ a, double *part)
{
  FE_PDL_ENTRY();
  __shared__ double sh[256];
  double s = 0.;
  for(int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    s += (double)a[pos[i]];
  sh[threadIdx.x] = s;
  __syncthreads();
  for(int o = 128; o > 0; o >>= 1) {
    if(threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if(threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

template <typename V>
__global__ void k_scale_copy(int64_t n, const V *__restrict__ r, V *__restrict__ z, V f,
                             const int *__restrict__ skip)
{
  FE_PDL_ENTRY();
  if(skip && *skip) return;
  for(int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    z[i] = r[i] * f;
}

// Pressure block with the constant mode deflated:
//   z_p = pscale_p (r_p - (c^T r) m_p / c^T M c) + (c^T r) / c^T S c,
// c = 1 on the pressure unknowns, (c^T r) read from *cr.
template <typename V, typename S>
__global__ void k_pressure(int64_t nP, const int32_t *__restrict__ rows, const S *__restrict__ sc,
                           const double *__restrict__ mass, const double *__restrict__ cr,
                           const double *__restrict__ consts, const V *__restrict__ r, V *__restrict__ z,
                           const int *__restrict__ skip)
{
  FE_PDL_ENTRY();
  if(skip && *skip) return;
  const double c = *cr, cSc = consts[1], cMc = consts[2];
  const double shift = cMc > 0 ? c / cMc : 0., lift = cSc != 0. ? c / cSc : 0.;
  for(int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nP; k += (int64_t)gridDim.x * blockDim.x) {
    const int32_t i = rows[k];
    const double rp = (double)r[i] - shift * mass[k];
    z[i] = (V)((double)sc[k] * rp + lift);
  }
}

// *out = sum of r over the pressure rows in one launch: one partial sum per
// block, then the last block to finish sums them in block order as
// k_dot_fin does (deterministic).  psum_blocks: the body, run by vg blocks with
// block index vb (the whole grid of k_psum, or a trailing range of blocks
// of k_vel_rhs_fold).
template <typename V>
__device__ __forceinline__ void psum_blocks(int vb, int vg, int64_t nP, const int32_t *__restrict__ rows,
                                            const V *__restrict__ r, double *part, unsigned *count, double *out)
{
  __shared__ double sh[256];
  __shared__ bool last;
  double s = 0.;
  for(int64_t k = (int64_t)vb * blockDim.x + threadIdx.x; k < nP; k += (int64_t)vg * blockDim.x)
    s += (double)r[rows[k]];
  sh[threadIdx.x] = s;
  __syncthreads();
  for(int o = 128; o > 0; o >>= 1) {
    if(threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if(threadIdx.x == 0) {
    part[vb] = sh[0];
    __threadfence();
    last = atomicAdd(count, 1u) == (unsigned)vg - 1;
  }
  __syncthreads();
  if(!last) return;
  __threadfence();
  double t = 0.;
  for(int i = threadIdx.x; i < vg; i += blockDim.x) t += __ldcg(part + i);
  sh[threadIdx.x] = t;
  __syncthreads();
  for(int o = 128; o > 0; o >>= 1) {
    if(threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if(threadIdx.x == 0) {
    *out = sh[0];
    *count = 0;
  }
}

template <typename V>
__global__ void k_psum(int64_t nP, const int32_t *__restrict__ rows, const V *__restrict__ r, double *part,
                       unsigned *count, double *out)
{
  FE_PDL_ENTRY();
  psum_blocks<V>(blockIdx.x, gridDim.x, nP, rows, r, part, count, out);
}

// partial sums of a double array
__global__ void k_tsum(int64_t n, const double *__restrict__ t, double *part)
{
  FE_PDL_ENTRY();
  __shared__ double sh[256];
  double s = 0.;
  for(int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
    s += t[k];
  sh[threadIdx.x] = s;
  __syncthreads();
  for(int o = 128; o > 0; o >>= 1) {
    if(threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if(threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

// g = G c: row sums of the G block per velocity slot.
template <typename V>
__global__ void k_gsum(int64_t nN, const int32_t *__restrict__ upIa, const int32_t *__restrict__ upPos,
                       const V *__restrict__ a, V *__restrict__ bx, V *__restrict__ by)
{
  FE_PDL_ENTRY();
  for(int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nN; k += (int64_t)gridDim.x * blockDim.x)
    for(int c = 0; c < 2; ++c) {
      double s = 0.;
      for(int32_t e = upIa[2 * k + c]; e < upIa[2 * k + c + 1]; ++e) s += (double)a[upPos[e]];
      if(c == 0) bx[k] = (V)s;
      else by[k] = (V)s;
    }
}

// t_p = (D w)_p with w given per slot by (wx, wy).
template <typename V>
__global__ void k_dw(int64_t nP, const int32_t *__restrict__ dnIa, const int32_t *__restrict__ dnPos,
                     const int32_t *__restrict__ dnCol, const int32_t *__restrict__ slotOf,
                     const V *__restrict__ a, const V *__restrict__ wx, const V *__restrict__ wy,
                     double *__restrict__ t)
{
  FE_PDL_ENTRY();
  for(int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nP; k += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.;
    for(int32_t e = dnIa[k]; e < dnIa[k + 1]; ++e) {
      const int32_t sl = slotOf[dnCol[e]];
      const double w = (sl & 1) ? (double)wy[sl >> 1] : (double)wx[sl >> 1];
      s += (double)a[dnPos[e]] * w;
    }
    t[k] = s;
  }
}

// b_c[k] = r_u - G z_p on velocity component c of node k.
template <typename V>
__global__ void k_vel_rhs(int64_t nN, const int32_t *__restrict__ dofX, const int32_t *__restrict__ dofY,
                          const int32_t *__restrict__ upIa, const int32_t *__restrict__ upPos,
                          const int32_t *__restrict__ upCol, const V *__restrict__ a,
                          const V *__restrict__ r, const V *__restrict__ z, V *__restrict__ bx,
                          V *__restrict__ by, const int *__restrict__ skip)
{
  FE_PDL_ENTRY();
  if(skip && *skip) return;
  for(int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nN; k += (int64_t)gridDim.x * blockDim.x) {
    for(int c = 0; c < 2; ++c) {
      const int32_t d = c == 0 ? dofX[k] : dofY[k];
      V t = r[d];
      const int64_t slot = 2 * k + c;
      if(upIa)
        for(int32_t e = upIa[slot]; e < upIa[slot + 1]; ++e) t -= a[upPos[e]] * z[upCol[e]];
      if(c == 0) bx[k] = t;
      else by[k] = t;
    }
  }
}

template <typename V>
__global__ void k_gather_vals(int64_t n, const int32_t *__restrict__ pos, const V *__restrict__ a, V *__restrict__ out)
{
  FE_PDL_ENTRY();
  for(int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
    out[e] = a[pos[e]];
}

// Cahouet-Chabard term: pr = r_p - (c^T r / c^T M c) m_p (the same deflated
// pressure residual as k_pressure) in the P1 Laplacian's row order, and
// z_p += cc * pz afterwards.
template <typename V>
__global__ void k_p_gather(int64_t nP, const int32_t *__restrict__ rows, const double *__restrict__ mass,
                           const double *__restrict__ cr, const double *__restrict__ consts, const V *__restrict__ r,
                           V *__restrict__ pr, const int *__restrict__ skip)
{
  FE_PDL_ENTRY();
  if(skip && *skip) return;
  const double cMc = consts[2];
  const double shift = cMc > 0 ? *cr / cMc : 0.;
  for(int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nP; k += (int64_t)gridDim.x * blockDim.x)
    pr[k] = (V)((double)r[rows[k]] - shift * mass[k]);
}

template <typename V>
__global__ void k_p_add(int64_t nP, const int32_t *__restrict__ rows, const V *__restrict__ pz,
                        const double *__restrict__ consts, V *__restrict__ z, const int *__restrict__ skip)
{
  FE_PDL_ENTRY();
  if(skip && *skip) return;
  const V cc = (V)consts[3];
  for(int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nP; k += (int64_t)gridDim.x * blockDim.x)
    z[rows[k]] += cc * pz[k];
}

// The same right-hand side, both components interleaved: bxy[2 k + c].
template <typename V>
__global__ void k_vel_rhs_pair(int64_t nN, const int32_t *__restrict__ dofX, const int32_t *__restrict__ dofY,
                               const int32_t *__restrict__ upIa, const int32_t *__restrict__ upPos,
                               const int32_t *__restrict__ upCol, const V *__restrict__ a,
                               const V *__restrict__ r, const V *__restrict__ z, V *__restrict__ bxy,
                               const int *__restrict__ skip)
{
  FE_PDL_ENTRY();
  if(skip && *skip) return;
  for(int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < 2 * nN; q += (int64_t)gridDim.x * blockDim.x) {
    const int64_t k = q >> 1;
    const int c = (int)(q & 1);
    V t = r[c == 0 ? dofX[k] : dofY[k]];
    for(int32_t e = upIa[q]; e < upIa[q + 1]; ++e) t -= (upPos ? a[upPos[e]] : a[e]) * z[upCol[e]];
    bxy[q] = t;
  }
}

// Folded velocity right-hand side b0 = r_u - (G sc) r_p on the slots
// (both components interleaved, one thread per slot), and in the leading
// gp blocks (scheduled first, so that the sum's last-block reduction
// overlaps the slots) the pressure sum c = sum of r over the pressure rows
// (k_psum's partials and order) into *cr.
template <typename V>
__global__ void k_vel_rhs_fold(int64_t nN, const int32_t *__restrict__ dofX, const int32_t *__restrict__ dofY,
                               const int32_t *__restrict__ upIa, const int32_t *__restrict__ upCol,
                               const V *__restrict__ gs, const V *__restrict__ r, V *__restrict__ bxy,
                               int slotBlocks, int64_t nP, const int32_t *__restrict__ pRows, double *part,
                               unsigned *count, double *cr, const int *__restrict__ skip)
{
  FE_PDL_ENTRY();
  if(skip && *skip) return;
  const int gp = (int)gridDim.x - slotBlocks;
  if((int)blockIdx.x < gp) {
    psum_blocks<V>((int)blockIdx.x, gp, nP, pRows, r, part, count, cr);
    return;
  }
  const int64_t q = (int64_t)((int)blockIdx.x - gp) * blockDim.x + threadIdx.x;
  if(q >= 2 * nN) return;
  const int64_t k = q >> 1;
  V t = r[(q & 1) == 0 ? dofX[k] : dofY[k]];
  for(int32_t e = upIa[q]; e < upIa[q + 1]; ++e) t -= gs[e] * r[upCol[e]];
  bxy[q] = t;
}

// Per Jacobian: the pressure scale sc_k = coef / (den m_k) in FP64 and
// FP32 and, for the pressure fold (u non-null), u_k = iS - sc_k m_k iM with
// sc_k as the apply kernels read it (FP32-rounded when fp32).
__global__ void k_pressure_scale(int64_t nP, double coef, double den, const double *__restrict__ mass,
                                 double *__restrict__ sc64, float *__restrict__ sc32, double *__restrict__ u,
                                 double iS, double iM, int fp32)
{
  FE_PDL_ENTRY();
  for(int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nP; k += (int64_t)gridDim.x * blockDim.x) {
    const double m = mass[k];
    const double sc = coef / (den * m);
    const float s32 = (float)sc;
    sc64[k] = sc;
    sc32[k] = s32;
    if(u) u[k] = iS - (fp32 ? (double)s32 : sc) * m * iM;
  }
}

// Per Jacobian, for the pressure fold: gScaled[e] = G_e sc_k(e) and
// gu[q] = sum_e G_e u_k(e) on slot q (FP64 sums).
template <typename V, typename S>
__global__ void k_fold_prep(int64_t nq, const int32_t *__restrict__ upIa, const int32_t *__restrict__ upColP,
                            const V *__restrict__ g, const S *__restrict__ sc, const double *__restrict__ u,
                            V *__restrict__ gScaled, V *__restrict__ gu)
{
  FE_PDL_ENTRY();
  for(int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < nq; q += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.;
    for(int32_t e = upIa[q]; e < upIa[q + 1]; ++e) {
      const int32_t kp = upColP[e];
      gScaled[e] = (V)(g[e] * (V)sc[kp]);
      s += (double)g[e] * u[kp];
    }
    gu[q] = (V)s;
  }
}

template <typename V>
__global__ void k_vel_out_pair(int64_t nN, const int32_t *__restrict__ dofX, const int32_t *__restrict__ dofY,
                               const V *__restrict__ zxy, const double *__restrict__ consts, V *__restrict__ z,
                               const int *__restrict__ skip)
{
  FE_PDL_ENTRY();
  if(skip && *skip) return;
  const V f = (V)consts[0];
  for(int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < 2 * nN; q += (int64_t)gridDim.x * blockDim.x) {
    const int64_t k = q >> 1;
    z[(q & 1) == 0 ? dofX[k] : dofY[k]] = zxy[q] * f;
  }
}

template <typename V>
__global__ void k_vel_out(int64_t nN, const int32_t *__restrict__ dofX, const int32_t *__restrict__ dofY,
                          const V *__restrict__ zx, const V *__restrict__ zy, const double *__restrict__ consts,
                          V *__restrict__ z, const int *__restrict__ skip)
{
  FE_PDL_ENTRY();
  if(skip && *skip) return;
  const V f = (V)consts[0];
  for(int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nN; k += (int64_t)gridDim.x * blockDim.x) {
    z[dofX[k]] = zx[k] * f;
    if(dofY) z[dofY[k]] = zy[k] * f;
  }
}

// Three-component variants (tetrahedra): slot q = nc k + c.
// b[q] = r_u - G z_p on slot q.
template <typename V>
__global__ void k_vel_rhs_nc(int64_t nq, const int32_t *__restrict__ dofC, const int32_t *__restrict__ upIa,
                             const int32_t *__restrict__ upCol, const V *__restrict__ g, const V *__restrict__ r,
                             const V *__restrict__ z, V *__restrict__ b, const int *__restrict__ skip)
{
  FE_PDL_ENTRY();
  if(skip && *skip) return;
  for(int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < nq; q += (int64_t)gridDim.x * blockDim.x) {
    V t = r[dofC[q]];
    for(int32_t e = upIa[q]; e < upIa[q + 1]; ++e) t -= g[e] * z[upCol[e]];
    b[q] = t;
  }
}

template <typename V>
__global__ void k_vel_out_nc(int64_t nq, const int32_t *__restrict__ dofC, const V *__restrict__ zc,
                             const double *__restrict__ consts, V *__restrict__ z, const int *__restrict__ skip)
{
  FE_PDL_ENTRY();
  if(skip && *skip) return;
  const V f = (V)consts[0];
  for(int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < nq; q += (int64_t)gridDim.x * blockDim.x)
    z[dofC[q]] = zc[q] * f;
}

// g = G c per slot (row sums of the G block).
template <typename V>
__global__ void k_gsum_nc(int64_t nq, const int32_t *__restrict__ upIa, const int32_t *__restrict__ upPos,
                          const V *__restrict__ a, V *__restrict__ b)
{
  FE_PDL_ENTRY();
  for(int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < nq; q += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.;
    for(int32_t e = upIa[q]; e < upIa[q + 1]; ++e) s += (double)a[upPos[e]];
    b[q] = (V)s;
  }
}

// t_p = (D w)_p with w given per slot.
template <typename V>
__global__ void k_dw_nc(int64_t nP, const int32_t *__restrict__ dnIa, const int32_t *__restrict__ dnPos,
                        const int32_t *__restrict__ dnCol, const int32_t *__restrict__ slotOf,
                        const V *__restrict__ a, const V *__restrict__ w, double *__restrict__ t)
{
  FE_PDL_ENTRY();
  for(int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nP; k += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.;
    for(int32_t e = dnIa[k]; e < dnIa[k + 1]; ++e) s += (double)a[dnPos[e]] * (double)w[slotOf[dnCol[e]]];
    t[k] = s;
  }
}

template <typename T>
int up(T **dst, const std::vector<T> &v)
{
  CKM(cudaMalloc(dst, sizeof(T) * std::max<size_t>(1, v.size())));
  CKM(cudaMemcpy(*dst, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice));
  return FE_OK;
}

}  // namespace

int Krylov::setup_mg(const PrecondInfo &pi)
{
  if(!pi.lap || pi.lap->n <= 0) {
    set_error("multigrid preconditioner needs the scalar stiffness matrix");
    return FE_INVALID_ARG;
  }
  mg_ = new MG();
  MG &M = *mg_;
  M.kind = opt.precond;
  M.fp32 = opt.mixed;
  M.sigma = pi.sigma;
  M.divu = pi.divu;
  M.nNodes = pi.lap->n;
  if((int64_t)pi.nodeDofX.size() != M.nNodes ||
     (M.kind == 4 && (int64_t)pi.nodeDofY.size() != M.nNodes)) {
    set_error("node maps do not match the stiffness matrix");
    return FE_INVALID_ARG;
  }
  AMGParams ap;
  ap.chebyDegree = pi.chebyDegree;
  M.params = ap;
  M.inner = pi.innerIterations;
  M.nc = pi.nodeDofZ.empty() ? 2 : 3;
  M.vfac = M.nc == 3 ? 4.0 / 3.0 : 1.5;
  if(M.nc == 3 && (M.kind != 4 || M.inner > 0 || (int64_t)pi.nodeDofZ.size() != M.nNodes)) {
    set_error("three-component multigrid: Taylor-Hood, one V-cycle per application, a DOF per node");
    return FE_INVALID_ARG;
  }
  if(M.kind == 4) {
    M.lapH = *pi.lap;
    if(pi.massV) M.massH = *pi.massV;
    if(pi.lapP) M.lapPH = *pi.lapP;
  }
  AMGHierarchy H;
  FE_TRY(amg_build(*pi.lap, ap, H));
  FE_TRY(M.amg->upload(H, ap, M.fp32, s_));
  M.lapDiagSum = M.amg->finestDiagSum();
  FE_TRY(up(&M.dofX, pi.nodeDofX));
  if(M.kind == 4) FE_TRY(up(&M.dofY, pi.nodeDofY));
  const size_t vs = M.fp32 ? sizeof(float) : sizeof(double);
  for(void **v : {&M.bx, &M.by, &M.zx, &M.zy, &M.ir, &M.iz, &M.ip, &M.iq})
    CKM(cudaMalloc(v, vs * M.nNodes));
  for(void **v : {&M.bxy, &M.zxy, &M.bgu}) CKM(cudaMalloc(v, 3 * vs * M.nNodes));
  CKM(cudaMalloc(&M.dsum, 2 * sizeof(double)));
  CKM(cudaMalloc(&M.part, sizeof(double) * NPART));
  CKM(cudaMalloc(&M.scal, sizeof(double) * 4));
  CKM(cudaMalloc(&M.consts, sizeof(double) * 4));
  CKM(cudaMemset(M.scal, 0, sizeof(double) * 4));
  CKM(cudaMalloc(&M.count, sizeof(unsigned)));
  CKM(cudaMemset(M.count, 0, sizeof(unsigned)));
  // Host pattern for the diagonal positions and the G block.
  std::vector<int32_t> hia(n_ + 1), hja(A_.nnz);
  CKM(cudaMemcpy(hia.data(), A_.ia, sizeof(int32_t) * (n_ + 1), cudaMemcpyDeviceToHost));
  CKM(cudaMemcpy(hja.data(), A_.ja, sizeof(int32_t) * A_.nnz, cudaMemcpyDeviceToHost));
  std::vector<int32_t> diagX(M.nNodes, -1);
  for(int64_t k = 0; k < M.nNodes; ++k) {
    const int32_t d = pi.nodeDofX[k];
    if(d < 0 || d >= n_) { set_error("node DOF out of range"); return FE_INVALID_ARG; }
    for(int32_t e = hia[d]; e < hia[d + 1]; ++e)
      if(hja[e] == d) diagX[k] = e;
    if(diagX[k] < 0) { set_error("missing diagonal"); return FE_INVALID_ARG; }
  }
  FE_TRY(up(&M.diagX, diagX));
  if(M.kind == 4) {
    M.nP = (int64_t)pi.pRows.size();
    M.pMass = pi.pMass;
    std::vector<uint8_t> isP(n_, 0);
    for(int32_t p : pi.pRows) {
      if(p < 0 || p >= n_) { set_error("pressure row out of range"); return FE_INVALID_ARG; }
      isP[p] = 1;
    }
    const int nc = M.nc;
    auto dofOf = [&](int64_t k, int c) {
      return c == 0 ? pi.nodeDofX[k] : c == 1 ? pi.nodeDofY[k] : pi.nodeDofZ[k];
    };
    std::vector<int32_t> ia2(nc * M.nNodes + 1, 0), pos, col, dofC(nc * M.nNodes);
    for(int64_t k = 0; k < M.nNodes; ++k)
      for(int c = 0; c < nc; ++c) {
        const int32_t d = dofOf(k, c);
        if(d < 0 || d >= n_) { set_error("node DOF out of range"); return FE_INVALID_ARG; }
        dofC[nc * k + c] = d;
        for(int32_t e = hia[d]; e < hia[d + 1]; ++e)
          if(isP[hja[e]]) { pos.push_back(e); col.push_back(hja[e]); }
        ia2[nc * k + c + 1] = (int32_t)pos.size();
      }
    if(nc == 3) FE_TRY(up(&M.dofC, dofC));
    FE_TRY(up(&M.upIa, ia2));
    FE_TRY(up(&M.upPos, pos));
    M.nG = (int64_t)pos.size();
    CKM(cudaMalloc(&M.gVals, sizeof(double) * std::max<int64_t>(1, M.nG)));
    FE_TRY(up(&M.upCol, col));
    FE_TRY(up(&M.pRows, pi.pRows));
    {
      // pressure index of each G entry's column (the pressure fold)
      std::vector<int32_t> pIndex(n_, -1), colP(col.size());
      for(int64_t k = 0; k < M.nP; ++k) pIndex[pi.pRows[k]] = (int32_t)k;
      for(size_t e = 0; e < col.size(); ++e) colP[e] = pIndex[col[e]];
      FE_TRY(up(&M.upColP, colP));
      CKM(cudaMalloc(&M.gScaled, sizeof(double) * std::max<int64_t>(1, M.nG)));
      CKM(cudaMalloc(&M.uP, sizeof(double) * std::max<int64_t>(1, M.nP)));
    }
    // D block (pressure rows -> velocity columns) and the slot of each velocity DOF.
    std::vector<int32_t> slot(n_, -1);
    for(int64_t k = 0; k < M.nNodes; ++k)
      for(int c = 0; c < nc; ++c) slot[dofOf(k, c)] = (int32_t)(nc * k + c);
    std::vector<int32_t> dia(M.nP + 1, 0), dpos, dcol;
    for(int64_t k = 0; k < M.nP; ++k) {
      const int32_t p = pi.pRows[k];
      for(int32_t e = hia[p]; e < hia[p + 1]; ++e)
        if(slot[hja[e]] >= 0) { dpos.push_back(e); dcol.push_back(hja[e]); }
      dia[k + 1] = (int32_t)dpos.size();
    }
    FE_TRY(up(&M.dnIa, dia));
    FE_TRY(up(&M.dnPos, dpos));
    FE_TRY(up(&M.dnCol, dcol));
    FE_TRY(up(&M.slotOf, slot));
    FE_TRY(up(&M.pMassDev, pi.pMass));
    CKM(cudaMalloc(&M.tP, sizeof(double) * std::max<int64_t>(1, M.nP)));
    M.cMc = 0.;
    for(double m : pi.pMass) M.cMc += m;
    CKM(cudaMalloc(&M.pScale64, sizeof(double) * std::max<int64_t>(1, M.nP)));
    CKM(cudaMalloc(&M.pScale32, sizeof(float) * std::max<int64_t>(1, M.nP)));
  }
  return FE_OK;
}

int Krylov::factor_mg(const double *values64, const float *values32)
{
  MG &M = *mg_;
  M.amg->setSkip(nullptr);
  // Everything the scalars need is launched first and read back with one
  // synchronisation: the diagonal sum (dsum[0]) and, for the saddle-point
  // preconditioner, c^T S c's estimate (dsum[1]).
  const int gd = (int)std::min<int64_t>(NPART, std::max<int64_t>(1, (M.nNodes + 255) / 256));
  if(values64) ::feng::launch_k(k_diag_part<double>, gd, 256, 0, s_, M.nNodes, M.diagX, values64, M.part);
  else ::feng::launch_k(k_diag_part<float>, gd, 256, 0, s_, M.nNodes, M.diagX, values32, M.part);
  ::feng::launch_k(k_dot_fin, 1, 256, 0, s_, gd, M.part, M.dsum);
  double sums[2] = {0., 0.};
  if(M.kind == 4) {
    // Contiguous copy of the G block's values for the apply kernels.
    if(values64)
      ::feng::launch_k(k_gather_vals<double>, grid(M.nG), 256, 0, s_, M.nG, M.upPos, values64, (double *)M.gVals);
    else
      ::feng::launch_k(k_gather_vals<float>, grid(M.nG), 256, 0, s_, M.nG, M.upPos, values32, (float *)M.gVals);
    // Constant pressure mode c: with the pressure fixed at a single point the
    // true Schur complement is nearly singular along c, far below the mass
    // estimate.  c^T S c = -(D^T c) . A^-1 (G c) is estimated once per
    // Jacobian with the velocity solve A^-1 ~ (s K)^-1 (the factor 1/s is
    // applied on the host below): here t = D K^-1 G c.
    if(M.nc == 3 || M.inner <= 0) {
      // the components interleaved (slot nc k + c) through one V-cycle
      const int64_t nq = (int64_t)M.nc * M.nNodes;
      if(values64) {
        ::feng::launch_k(k_gsum_nc<double>, grid(nq), 256, 0, s_, nq, M.upIa, M.upPos, values64, (double *)M.bxy);
        if(M.nc == 3) M.amg->vcycle3_64((const double *)M.bxy, (double *)M.zxy);
        else M.amg->vcycle2_64((const double *)M.bxy, (double *)M.zxy, nullptr);
        ::feng::launch_k(k_dw_nc<double>, grid(M.nP), 256, 0, s_, M.nP, M.dnIa, M.dnPos, M.dnCol, M.slotOf, values64,
                         (const double *)M.zxy, M.tP);
      } else {
        ::feng::launch_k(k_gsum_nc<float>, grid(nq), 256, 0, s_, nq, M.upIa, M.upPos, values32, (float *)M.bxy);
        if(M.nc == 3) M.amg->vcycle3_32((const float *)M.bxy, (float *)M.zxy);
        else M.amg->vcycle2_32((const float *)M.bxy, (float *)M.zxy, nullptr);
        ::feng::launch_k(k_dw_nc<float>, grid(M.nP), 256, 0, s_, M.nP, M.dnIa, M.dnPos, M.dnCol, M.slotOf, values32,
                         (const float *)M.zxy, M.tP);
      }
    } else {
      const int g = grid(M.nNodes);
      if(values64) {
        ::feng::launch_k(k_gsum<double>, g, 256, 0, s_, M.nNodes, M.upIa, M.upPos, values64, (double *)M.bx, (double *)M.by);
        M.solveK<double>((const double *)M.bx, (double *)M.zx, s_);
        M.solveK<double>((const double *)M.by, (double *)M.zy, s_);
        ::feng::launch_k(k_dw<double>, grid(M.nP), 256, 0, s_, M.nP, M.dnIa, M.dnPos, M.dnCol, M.slotOf, values64,
                         (const double *)M.zx, (const double *)M.zy, M.tP);
      } else {
        ::feng::launch_k(k_gsum<float>, g, 256, 0, s_, M.nNodes, M.upIa, M.upPos, values32, (float *)M.bx, (float *)M.by);
        M.solveK<float>((const float *)M.bx, (float *)M.zx, s_);
        M.solveK<float>((const float *)M.by, (float *)M.zy, s_);
        ::feng::launch_k(k_dw<float>, grid(M.nP), 256, 0, s_, M.nP, M.dnIa, M.dnPos, M.dnCol, M.slotOf, values32,
                         (const float *)M.zx, (const float *)M.zy, M.tP);
      }
    }
    const int gp = (int)std::min<int64_t>(NPART, std::max<int64_t>(1, (M.nP + 255) / 256));
    ::feng::launch_k(k_tsum, gp, 256, 0, s_, M.nP, M.tP, M.part);
    ::feng::launch_k(k_dot_fin, 1, 256, 0, s_, gp, M.part, M.dsum + 1);
    CKM(cudaMemcpyAsync(sums, M.dsum, 2 * sizeof(double), cudaMemcpyDeviceToHost, s_));
  } else {
    CKM(cudaMemcpyAsync(sums, M.dsum, sizeof(double), cudaMemcpyDeviceToHost, s_));
  }
  CKM(cudaStreamSynchronize(s_));
  const double sum = sums[0];
  if(!(std::isfinite(sum)) || sum == 0.) {
    set_error("preconditioner scale: zero or non-finite diagonal");
    return FE_PC_FAILED;
  }
  // A_xx ~ s K; for the symmetric-gradient viscous operator the diagonal of
  // one component block is about 1.5 times the Laplacian's, so
  // mu ~ -s / (1.5 sigma) and S^-1 ~ (mu / c_div) M_p^-1.
  M.s = sum / M.lapDiagSum;
  if(M.kind == 4) {
    M.cSc = -sums[1] / M.s;
    // Against the lumped-mass estimate c^T S c ~ -vfac sigma c_div c^T M c / s:
    // a negligible value means the pressure is determined only up to a
    // constant (no pressure DOF fixed); then the constant mode is only
    // projected out of z_p (no lift).
    const double massEst = std::fabs(M.vfac * M.sigma * M.divu * M.cMc / M.s);
    if(!std::isfinite(M.cSc) || std::fabs(M.cSc) <= 1e-8 * massEst) M.cSc = 0.;  // no deflation
  }
  // Scalars read by the (graph-replayed) apply kernels; the solve that
  // follows runs on the same stream.
  M.hconst[0] = 1.0 / M.s;
  M.hconst[1] = M.cSc;
  M.hconst[2] = M.cMc;
  M.hconst[3] = M.cc;
  CKM(cudaMemcpyAsync(M.consts, M.hconst, sizeof(double) * 4, cudaMemcpyHostToDevice, s_));
  // The pressure fold: the steady two-component preconditioner with one
  // V-cycle on a sliced-ELL finest level (the fold's output goes through
  // that level's post-smoothing pass).
  static const bool foldOn = [] {
    const char *e = std::getenv("FENG_PFOLD");
    return !(e && std::strcmp(e, "0") == 0);
  }();
  M.fold = foldOn && M.kind == 4 && M.nc == 2 && M.inner <= 0 && !M.amgP && M.amg->fineSell();
  if(M.kind == 4) {
    // the pressure scale (FP64 and FP32) and, for the fold, u on the device
    const double coef = -SCHUR_FACTOR * M.s, den = M.vfac * M.sigma * M.divu;
    const double iS = M.cSc != 0. ? 1.0 / M.cSc : 0., iM = M.cMc > 0 ? 1.0 / M.cMc : 0.;
    ::feng::launch_k(k_pressure_scale, grid(M.nP), 256, 0, s_, M.nP, coef, den, M.pMassDev, M.pScale64, M.pScale32,
                     M.fold ? M.uP : (double *)nullptr, iS, iM, values64 ? 0 : 1);
  }
  if(M.fold) {
    const int64_t nq = 2 * M.nNodes;
    if(values64) {
      ::feng::launch_k(k_fold_prep<double, double>, grid(nq), 256, 0, s_, nq, M.upIa, M.upColP, (const double *)M.gVals,
                       M.pScale64, M.uP, (double *)M.gScaled, (double *)M.bxy);
      M.amg->vcycle2_64((const double *)M.bxy, (double *)M.bgu, nullptr);
    } else {
      ::feng::launch_k(k_fold_prep<float, float>, grid(nq), 256, 0, s_, nq, M.upIa, M.upColP, (const float *)M.gVals,
                       M.pScale32, M.uP, (float *)M.gScaled, (float *)M.bxy);
      M.amg->vcycle2_32((const float *)M.bxy, (float *)M.bgu, nullptr);
    }
  }
  return FE_OK;
}

int Krylov::setTransientShift(double c0, double mu)
{
  if(!mg_ || mg_->kind != 4) return FE_OK;
  MG &M = *mg_;
  if(!(c0 >= 0.) || !(mu > 0.)) {
    set_error("transient shift needs c0 >= 0 and a positive viscosity");
    return FE_INVALID_ARG;
  }
  if(M.massH.a.size() != M.lapH.a.size() || M.lapPH.n != M.nP) {
    set_error("transient shift: preconditioner operators missing");
    return FE_INVALID_ARG;
  }
  // Velocity multigrid on K + (c0 / mu) M (same pattern), the prolongators
  // smoothed with the filtered operator when shifted.
  HostCSR L = M.lapH;
  const double alpha = c0 / mu;
  for(size_t k = 0; k < L.a.size(); ++k) L.a[k] += alpha * M.massH.a[k];
  AMGParams vp = M.params;
  vp.filterSmoothing = c0 > 0.;
  AMGHierarchy H;
  FE_TRY(amg_build(L, vp, H));
  auto amg = std::make_unique<AMGDevice>();
  FE_TRY(amg->upload(H, vp, M.fp32, s_));
  M.amg = std::move(amg);
  M.lapDiagSum = M.amg->finestDiagSum();
  // Pressure Laplacian multigrid (built once) and the Cahouet-Chabard weight.
  if(c0 > 0. && !M.amgP) {
    // With no pressure DOF fixed (velocity prescribed on the whole boundary,
    // the pressure determined up to a constant) the P1 Laplacian is the pure
    // Neumann one: constants span its null space and the coarsest direct
    // solve would divide by a rounding-level pivot.  A diagonal shift of
    // 1e-6 keeps it regular; k_p_gather projects the input to zero sum, so
    // the shift only bounds the constant part of the output (a null vector
    // of the saddle-point operator).
    HostCSR Lp = M.lapPH;
    double dmax = 0., rmax = 0.;
    for(int64_t i = 0; i < Lp.n; ++i) {
      double rs = 0.;
      for(int64_t k = Lp.ia[i]; k < Lp.ia[i + 1]; ++k) {
        rs += Lp.a[k];
        if(Lp.ja[k] == i) dmax = std::max(dmax, std::fabs(Lp.a[k]));
      }
      rmax = std::max(rmax, std::fabs(rs));
    }
    if(rmax <= 1e-10 * dmax)
      for(int64_t i = 0; i < Lp.n; ++i)
        for(int64_t k = Lp.ia[i]; k < Lp.ia[i + 1]; ++k)
          if(Lp.ja[k] == i) Lp.a[k] *= 1. + 1e-6;
    AMGHierarchy HP;
    FE_TRY(amg_build(Lp, M.params, HP));
    auto ap = std::make_unique<AMGDevice>();
    FE_TRY(ap->upload(HP, M.params, M.fp32, s_));
    M.amgP = std::move(ap);
    const size_t vs = M.fp32 ? sizeof(float) : sizeof(double);
    CKM(cudaMalloc(&M.pr, vs * std::max<int64_t>(1, M.nP)));
    CKM(cudaMalloc(&M.pz, vs * std::max<int64_t>(1, M.nP)));
  }
  M.cc = c0;
  if(c0 == 0.) M.amgP.reset();
  // The replayed cycles hold pointers into the old hierarchy.
  for(auto &g : graphs_) cudaGraphExecDestroy(g.second);
  graphs_.clear();
  graphKernels_.clear();
  factoredOk_ = false;  // rebuilt (scale, deflation) at the next factor
  return FE_OK;
}

int Krylov::smootherStep(int64_t *bytes)
{
  if(!mg_) {
    if(bytes) *bytes = 0;
    set_error("no multigrid preconditioner");
    return FE_INVALID_ARG;
  }
  mg_->amg->setSkip(nullptr);
  mg_->amg->fineStep2();
  if(bytes) *bytes = mg_->amg->fineStep2Bytes();
  return FE_OK;
}

template <typename V>
void Krylov::apply_mg(const V *vals, const V *r, V *z, const int *skip)
{
  MG &M = *mg_;
  M.amg->setSkip(skip);
  if(M.kind == 3) {
    // z = (s K)^-1 r on the unknown rows (the nodes are the unknowns)
    ::feng::launch_k(k_vel_rhs<V>, grid(M.nNodes), 256, 0, s_, M.nNodes, M.dofX, M.dofX, nullptr, nullptr, nullptr,
                                                  vals, r, z, (V *)M.bx, (V *)M.by, skip);
  } else if(M.fold) {
    // z_p = sc r_p + c u and b = r_u - G z_p = b0 - c G u with
    // b0 = r_u - (G sc) r_p, c = the pressure sum: the V-cycle is linear, so
    // z_u = (V(b0) - c V(G u)) / s with V(G u) = bgu from the set-up.  One
    // kernel forms b0 and c, the V-cycle's last pass writes z_u and z_p.
    const int gp = (int)std::min<int64_t>(NPART, std::max<int64_t>(1, (M.nP + 255) / 256));
    const int slotBlocks = (int)((2 * M.nNodes + 255) / 256);
    double *cr = M.scal + 3;
    ::feng::launch_k(k_vel_rhs_fold<V>, slotBlocks + gp, 256, 0, s_, M.nNodes, M.dofX, M.dofY, M.upIa, M.upCol,
                     (const V *)M.gScaled, r, (V *)M.bxy, slotBlocks, M.nP, M.pRows, M.part, M.count, cr, skip);
    AMGDevice::OutMap om;
    om.dofX = M.dofX;
    om.dofY = M.dofY;
    om.scale = M.consts;
    om.z = z;
    om.cr = cr;
    om.bgu = M.bgu;
    om.nP = M.nP;
    om.pRows = M.pRows;
    if constexpr(sizeof(V) == 8) om.pScale = M.pScale64;
    else om.pScale = M.pScale32;
    om.pMass = M.pMassDev;
    om.consts = M.consts;
    om.r = r;
    bool written;
    if constexpr(sizeof(V) == 8) written = M.amg->vcycle2_64((const double *)M.bxy, (double *)M.zxy, &om);
    else written = M.amg->vcycle2_32((const float *)M.bxy, (float *)M.zxy, &om);
    if(!written) set_error("pressure fold: the finest post-smoothing pass did not write the result");
    return;
  } else {
    const int gp = (int)std::min<int64_t>(NPART, std::max<int64_t>(1, (M.nP + 255) / 256));
    ::feng::launch_k(k_psum<V>, gp, 256, 0, s_, M.nP, M.pRows, r, M.part, M.count, M.scal + 3);
    const double *cr = M.scal + 3;
    if constexpr(sizeof(V) == 8)
      ::feng::launch_k(k_pressure<V, double>, grid(M.nP), 256, 0, s_, M.nP, M.pRows, M.pScale64, M.pMassDev, cr, M.consts,
                                                        r, z, skip);
    else
      ::feng::launch_k(k_pressure<V, float>, grid(M.nP), 256, 0, s_, M.nP, M.pRows, M.pScale32, M.pMassDev, cr, M.consts,
                                                       r, z, skip);
    if(M.amgP) {
      // + c0 L_p^-1 r_p (Cahouet-Chabard); its V-cycle skips with the cycle
      M.amgP->setSkip(skip);
      ::feng::launch_k(k_p_gather<V>, grid(M.nP), 256, 0, s_, M.nP, M.pRows, M.pMassDev, cr, M.consts, r, (V *)M.pr, skip);
      if constexpr(sizeof(V) == 8) M.amgP->vcycle64((const double *)M.pr, (double *)M.pz);
      else M.amgP->vcycle32((const float *)M.pr, (float *)M.pz);
      ::feng::launch_k(k_p_add<V>, grid(M.nP), 256, 0, s_, M.nP, M.pRows, (const V *)M.pz, M.consts, z, skip);
    }
    if(M.nc == 3) {
      // The three velocity components through one V-cycle on interleaved
      // right-hand sides, then z_u = (1/s) x.
      const int64_t nq = 3 * M.nNodes;
      ::feng::launch_k(k_vel_rhs_nc<V>, grid(nq), 256, 0, s_, nq, M.dofC, M.upIa, M.upCol, (const V *)M.gVals, r, z, (V *)M.bxy,
                                                 skip);
      if constexpr(sizeof(V) == 8) M.amg->vcycle3_64((const double *)M.bxy, (double *)M.zxy);
      else M.amg->vcycle3_32((const float *)M.bxy, (float *)M.zxy);
      ::feng::launch_k(k_vel_out_nc<V>, grid(nq), 256, 0, s_, nq, M.dofC, (const V *)M.zxy, M.consts, z, skip);
      return;
    }
    if(M.inner <= 0) {
      // Both velocity components through one paired V-cycle (one pass over
      // each level operator for the two right-hand sides).
      ::feng::launch_k(k_vel_rhs_pair<V>, grid(2 * M.nNodes), 256, 0, s_, M.nNodes, M.dofX, M.dofY, M.upIa, nullptr, M.upCol,
                                                               (const V *)M.gVals, r, z, (V *)M.bxy, skip);
      // the finest post-smoothing pass writes z_u (times 1/s) itself when
      // it can; otherwise the interleaved result is scattered here
      AMGDevice::OutMap om;
      om.dofX = M.dofX;
      om.dofY = M.dofY;
      om.scale = M.consts;
      om.z = z;
      bool written;
      if constexpr(sizeof(V) == 8) written = M.amg->vcycle2_64((const double *)M.bxy, (double *)M.zxy, &om);
      else written = M.amg->vcycle2_32((const float *)M.bxy, (float *)M.zxy, &om);
      if(!written)
        ::feng::launch_k(k_vel_out_pair<V>, grid(2 * M.nNodes), 256, 0, s_, M.nNodes, M.dofX, M.dofY, (const V *)M.zxy, M.consts,
                                                                z, skip);
      return;
    }
    ::feng::launch_k(k_vel_rhs<V>, grid(M.nNodes), 256, 0, s_, M.nNodes, M.dofX, M.dofY, M.upIa, M.upPos, M.upCol,
                                                  vals, r, z, (V *)M.bx, (V *)M.by, skip);
  }
  // The component solves run unconditionally; when `skip` is set their
  // output is discarded by the skipped scatter below.
  M.solveK<V>((const V *)M.bx, (V *)M.zx, s_);
  if(M.kind == 4) M.solveK<V>((const V *)M.by, (V *)M.zy, s_);
  ::feng::launch_k(k_vel_out<V>, grid(M.nNodes), 256, 0, s_, M.nNodes, M.dofX, M.kind == 4 ? M.dofY : nullptr,
                                                (const V *)M.zx, (const V *)M.zy, M.consts, z, skip);
}

template void Krylov::apply_mg<double>(const double *, const double *, double *, const int *);
template void Krylov::apply_mg<float>(const float *, const float *, float *, const int *);

}  // namespace feng
