// Element assembly kernels: residual (FP64) and Jacobian (FP64 or FP32) of
// the fused weak forms.
//
// Colored kernels (residuals; scalar P2 Jacobian): one launch per element
// color, entries scattered into CSR through the element-to-nonzero map as
// L2 reductions; no two elements of a color share a DOF, so every entry
// receives one contribution per color and the sums are the colored
// read-modify-write's, in color order.
//
// Row-owned kernel (Taylor-Hood Jacobian, k_matrix_th_rows): one thread per
// CSR row sums the element-matrix rows of the elements holding that DOF, in
// color order, in shared memory; each block writes its contiguous range of
// CSR values once (no atomics, no map, no separate zeroing pass).
//
// Mapping: a block holds 32 elements (lane = element) x 6 warps (warp = P2
// function a of the element).  Thread (e, a) produces the element-matrix rows
// of the DOFs attached to function a -- one row for a scalar field, the two
// component rows (a,x) (a,y) for the Taylor-Hood velocity -- plus, for a < 3,
// the pressure row of P1 function a.  All lanes of a warp read the same
// reference tensor entries (shared-memory broadcast) and their own element's
// data (shared-memory columns), so the contraction has no divergence.
//
// Arithmetic: for affine (P1) geometry the physical gradients are
// grad phi = G^T dphi/dr with G[r][k] = d r_r / d x_k constant per element,
// so every quadrature sum of the reference weak forms factors into constant
// reference tensors contracted with G, |J| and the element DOF values:
//   int dphi_a/dx_k dphi_b/dx_l     = |J| sum_rs G[r][k] G[s][l] K[r][s][a][b]
//   int phi_a phi_c dphi_b/dx_k     = |J| sum_r  G[r][k] T[r][a][c][b]
//   int psi_j dphi_a/dx_k           = |J| sum_r  G[r][k] D[r][j][a]
//   int phi_a phi_b                 = |J| M[a][b]
// The tensors are sums over the same quadrature nodes and weights the
// reference loops over (feSysElm.cpp:530-583, feVectorSysElm.cpp:112-130,
// 390-427, 685-747, 1171-1240, 1454-1530), so the results are the same sums
// regrouped: they agree to rounding.
#include <cuda_runtime.h>

#include <algorithm>

#include "fe_common.h"
#include "fe_device.h"
#include "fe_df.h"

namespace feng {

namespace {

constexpr int EPB = 32;  // elements per block (one per lane)
constexpr double PI = 3.14159265358979323846;

__device__ __forceinline__ void source_value(int kind, const double *p, double x, double y,
                                             double f[2])
{
  switch(kind) {
    case SRC_SIN_SIN:
      f[0] = p[0] * sin(PI * x) * sin(PI * y);
      f[1] = 0.;
      break;
    case SRC_NS_MMS_POLY: {
      // f = -( -u.grad u - grad p + lap u ) for u=(x^4 y^4, -4/5 x^3 y^5), p = x^2 y^2
      const double mdpdx0 = -2. * x * y * y, mdpdx1 = -2. * x * x * y;
      const double lap0 = 12. * (x * x * y * y * y * y + x * x * x * x * y * y);
      const double lap1 = -4. / 5. * (6. * x * y * y * y * y * y + 20. * x * x * x * y * y * y);
      const double u0 = x * x * x * x * y * y * y * y, u1 = -4. / 5. * x * x * x * y * y * y * y * y;
      const double g00 = 4. * x * x * x * y * y * y * y, g01 = -12. * x * x * y * y * y * y * y / 5.;
      const double g10 = 4. * x * x * x * x * y * y * y, g11 = -4. * x * x * x * y * y * y * y;
      const double c0 = u0 * g00 + u1 * g10, c1 = u0 * g01 + u1 * g11;
      f[0] = -(-c0 + mdpdx0 + lap0);
      f[1] = -(-c1 + mdpdx1 + lap1);
      break;
    }
    case SRC_CONST_VEC:
      f[0] = p[0];
      f[1] = p[1];
      break;
    case SRC_SIN_BODY:
      f[0] = p[0] * sin(PI * x) * sin(PI * y);
      f[1] = 0.;
      break;
    default:
      f[0] = f[1] = 0.;
  }
}

template <typename V>
struct SharedTensors {
  V K[2][2][6][6];
  V T[2][6][6][6];
  V D[2][3][6];
  V M[6][6];
};

template <typename V>
__device__ void load_tensors(SharedTensors<V> &s, const RefTensors *g)
{
  const int tid = threadIdx.y * blockDim.x + threadIdx.x, nt = blockDim.x * blockDim.y;
  const double *K = &g->K[0][0][0][0], *T = &g->T[0][0][0][0], *D = &g->D[0][0][0], *M = &g->M[0][0];
  V *sK = &s.K[0][0][0][0], *sT = &s.T[0][0][0][0], *sD = &s.D[0][0][0], *sM = &s.M[0][0];
  for(int i = tid; i < 144; i += nt) sK[i] = (V)K[i];
  for(int i = tid; i < 432; i += nt) sT[i] = (V)T[i];
  for(int i = tid; i < 36; i += nt) sD[i] = (V)D[i];
  for(int i = tid; i < 36; i += nt) sM[i] = (V)M[i];
}

// ---------------------------------------------------------------------------
// Residual, scalar P2 (DIFFUSION + SOURCE).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(EPB * 6) k_residual_p2(DeviceMesh dm, FormCoeffs fc,
                                                        const RefTensors *__restrict__ gT,
                                                        const double *__restrict__ u, double t,
                                                        int64_t nInc, double *__restrict__ rhs,
                                                        int64_t begin, int64_t end)
{
  __shared__ SharedTensors<double> sT;
  __shared__ double sU[6][EPB];
  __shared__ double sG[5][EPB];
  __shared__ double sF[16][EPB];
  __shared__ int32_t sA[6][EPB];
  const int lane = threadIdx.x, a = threadIdx.y;
  const int64_t p = begin + (int64_t)blockIdx.x * EPB + lane;
  const bool live = p < end;
  const int64_t nE = dm.nElm;
  load_tensors(sT, gT);
  if(live) {
    int32_t d = dm.adr[(int64_t)a * nE + p];
    sA[a][lane] = d;
    sU[a][lane] = u[d];
    if(a < 5) sG[a][lane] = dm.geo[(int64_t)a * nE + p];
  }
  const int nq = gT->nq;
  if(fc.srcKind != SRC_NONE && live) {
    const double x0 = dm.xy[0 * nE + p], y0 = dm.xy[1 * nE + p], x1 = dm.xy[2 * nE + p],
                 y1 = dm.xy[3 * nE + p], x2 = dm.xy[4 * nE + p], y2 = dm.xy[5 * nE + p];
    for(int q = a; q < nq; q += 6) {
      const double r = gT->qr[q], s = gT->qs[q];
      const double x = x0 * (1. - r - s) + x1 * r + x2 * s;
      const double y = y0 * (1. - r - s) + y1 * r + y2 * s;
      double f[2];
      source_value(fc.srcKind, fc.srcParam, x, y, f);
      sF[q][lane] = f[0];
    }
  }
  __syncthreads();
  if(!live) return;
  const double G[2][2] = {{sG[0][lane], sG[1][lane]}, {sG[2][lane], sG[3][lane]}};
  const double J = sG[4][lane];
  double be = 0.;
  if(fc.hasDiff) {
    // Be_a -= k grad phi_a . grad u  (feSysElm.cpp:560-583)
    double GG[2][2];
    for(int r = 0; r < 2; ++r)
      for(int s2 = 0; s2 < 2; ++s2) GG[r][s2] = G[r][0] * G[s2][0] + G[r][1] * G[s2][1];
    double acc = 0.;
    for(int b = 0; b < 6; ++b) {
      double L = 0.;
      for(int r = 0; r < 2; ++r)
        for(int s2 = 0; s2 < 2; ++s2) L += GG[r][s2] * sT.K[r][s2][a][b];
      acc += L * sU[b][lane];
    }
    be -= fc.diff * acc * J;
  }
  if(fc.srcKind != SRC_NONE) {
    // Be_a -= phi_a S jac w  (feSysElm.cpp:16-27)
    double acc = 0.;
    for(int q = 0; q < nq; ++q) acc += gT->phi[q][a] * sF[q][lane] * gT->qw[q];
    be -= fc.srcCoeff * acc * J;
  }
  const int32_t d = sA[a][lane];
  if(d < nInc) atomicAdd(rhs + d, be);  // one contribution per DOF and color
}

// ---------------------------------------------------------------------------
// Jacobian, scalar P2 (DIFFUSION).
// ---------------------------------------------------------------------------
template <typename V>
__global__ void __launch_bounds__(EPB * 6) k_matrix_p2(DeviceMesh dm, FormCoeffs fc,
                                                      const RefTensors *__restrict__ gT,
                                                      V *__restrict__ values, int64_t begin,
                                                      int64_t end)
{
  __shared__ SharedTensors<V> sT;
  __shared__ V sG[5][EPB];
  const int lane = threadIdx.x, a = threadIdx.y;
  const int64_t p = begin + (int64_t)blockIdx.x * EPB + lane;
  const bool live = p < end;
  const int64_t nE = dm.nElm;
  load_tensors(sT, gT);
  if(live && a < 5) sG[a][lane] = (V)dm.geo[(int64_t)a * nE + p];
  __syncthreads();
  if(!live || !fc.hasDiff) return;
  const V G[2][2] = {{sG[0][lane], sG[1][lane]}, {sG[2][lane], sG[3][lane]}};
  const V cJ = (V)fc.diff * sG[4][lane];
  V GG[2][2];
  for(int r = 0; r < 2; ++r)
    for(int s2 = 0; s2 < 2; ++s2) GG[r][s2] = G[r][0] * G[s2][0] + G[r][1] * G[s2][1];
  for(int b = 0; b < 6; ++b) {
    V L = 0;
    for(int r = 0; r < 2; ++r)
      for(int s2 = 0; s2 < 2; ++s2) L += GG[r][s2] * sT.K[r][s2][a][b];
    const int32_t pos = dm.map[(int64_t)(a * 6 + b) * nE + p];
    if(pos >= 0) atomicAdd(values + pos, cJ * L);  // one contribution per entry and color
  }
}

// ---------------------------------------------------------------------------
// Residual, Taylor-Hood P2-P1 (VECTOR_CONVECTIVE_ACCELERATION,
// DIV_NEWTONIAN_STRESS, MIXED_DIVERGENCE, TRANSIENT_VECTOR_MASS,
// VECTOR_SOURCE).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(EPB * 6) k_residual_th(DeviceMesh dm, FormCoeffs fc,
                                                        const RefTensors *__restrict__ gT,
                                                        const double *__restrict__ u,
                                                        const double *__restrict__ udot, double t,
                                                        int64_t nInc, double *__restrict__ rhs,
                                                        int64_t begin, int64_t end)
{
  __shared__ SharedTensors<double> sT;
  __shared__ double sU[12][EPB];
  __shared__ double sUd[12][EPB];
  __shared__ double sP[3][EPB];
  __shared__ double sG[5][EPB];
  __shared__ double sF[2][16][EPB];
  __shared__ int32_t sA[15][EPB];
  const int lane = threadIdx.x, a = threadIdx.y;
  const int64_t p = begin + (int64_t)blockIdx.x * EPB + lane;
  const bool live = p < end;
  const int64_t nE = dm.nElm;
  load_tensors(sT, gT);
  const bool hasSrc = fc.srcKind != SRC_NONE;
  if(live) {
    for(int i = a; i < 15; i += 6) {
      int32_t d = dm.adr[(int64_t)i * nE + p];
      sA[i][lane] = d;
      if(i < 12) {
        sU[i][lane] = u[d];
        if(fc.hasMass) sUd[i][lane] = udot[d];
      } else {
        sP[i - 12][lane] = u[d];
      }
    }
    if(a < 5) sG[a][lane] = dm.geo[(int64_t)a * nE + p];
  }
  const int nq = gT->nq;
  if(hasSrc && live) {
    const double x0 = dm.xy[0 * nE + p], y0 = dm.xy[1 * nE + p], x1 = dm.xy[2 * nE + p],
                 y1 = dm.xy[3 * nE + p], x2 = dm.xy[4 * nE + p], y2 = dm.xy[5 * nE + p];
    for(int q = a; q < nq; q += 6) {
      const double r = gT->qr[q], s = gT->qs[q];
      const double x = x0 * (1. - r - s) + x1 * r + x2 * s;
      const double y = y0 * (1. - r - s) + y1 * r + y2 * s;
      double f[2];
      source_value(fc.srcKind, fc.srcParam, x, y, f);
      sF[0][q][lane] = f[0];
      sF[1][q][lane] = f[1];
    }
  }
  __syncthreads();
  if(!live) return;
  const double G[2][2] = {{sG[0][lane], sG[1][lane]}, {sG[2][lane], sG[3][lane]}};
  const double J = sG[4][lane];
  double be[2] = {0., 0.};

  if(fc.hasConv) {
    // Be_(a,m) -= c (u . grad u)_m phi_a jac w   (feVectorSysElm.cpp:1206-1240)
    double V0[2][6];
    for(int c = 0; c < 6; ++c)
      for(int r = 0; r < 2; ++r) V0[r][c] = sU[2 * c][lane] * G[r][0] + sU[2 * c + 1][lane] * G[r][1];
    double R[2] = {0., 0.};
    for(int b = 0; b < 6; ++b) {
      double W = 0.;
      for(int c = 0; c < 6; ++c) W += V0[0][c] * sT.T[0][a][c][b] + V0[1][c] * sT.T[1][a][c][b];
      R[0] += W * sU[2 * b][lane];
      R[1] += W * sU[2 * b + 1][lane];
    }
    be[0] -= fc.conv * R[0] * J;
    be[1] -= fc.conv * R[1] * J;
  }
  if(fc.hasSigma) {
    // Be_(a,m) -= c (p div phi - mu (grad u + grad u^T) : grad phi) jac w
    // (feVectorSysElm.cpp:1494-1530)
    double GG[2][2][2][2];  // [k][l][r][s] = G[r][k] G[s][l]
    for(int k = 0; k < 2; ++k)
      for(int l = 0; l < 2; ++l)
        for(int r = 0; r < 2; ++r)
          for(int s2 = 0; s2 < 2; ++s2) GG[k][l][r][s2] = G[r][k] * G[s2][l];
    double visc[2] = {0., 0.};
    for(int b = 0; b < 6; ++b) {
      double S[2][2];
      for(int k = 0; k < 2; ++k)
        for(int l = 0; l < 2; ++l) {
          double v = 0.;
          for(int r = 0; r < 2; ++r)
            for(int s2 = 0; s2 < 2; ++s2) v += GG[k][l][r][s2] * sT.K[r][s2][a][b];
          S[k][l] = v;
        }
      const double tr = S[0][0] + S[1][1];
      const double ub0 = sU[2 * b][lane], ub1 = sU[2 * b + 1][lane];
      // m-th component: U_bm (S_xx+S_yy) + sum_k U_bk S_km
      visc[0] += ub0 * tr + ub0 * S[0][0] + ub1 * S[1][0];
      visc[1] += ub1 * tr + ub0 * S[0][1] + ub1 * S[1][1];
    }
    double pdiv[2] = {0., 0.};
    for(int j = 0; j < 3; ++j) {
      const double pj = sP[j][lane];
      for(int m = 0; m < 2; ++m) pdiv[m] += pj * (G[0][m] * sT.D[0][j][a] + G[1][m] * sT.D[1][j][a]);
    }
    for(int m = 0; m < 2; ++m) be[m] -= fc.sigma * (pdiv[m] - fc.mu * visc[m]) * J;
  }
  if(fc.hasMass) {
    // Be_(a,m) -= c udot . phi jac w   (feVectorSysElm.cpp:410-427)
    double acc[2] = {0., 0.};
    for(int b = 0; b < 6; ++b) {
      acc[0] += sT.M[a][b] * sUd[2 * b][lane];
      acc[1] += sT.M[a][b] * sUd[2 * b + 1][lane];
    }
    be[0] -= fc.mass * acc[0] * J;
    be[1] -= fc.mass * acc[1] * J;
  }
  if(hasSrc) {
    // Be_(a,m) -= f . phi jac w   (feVectorSysElm.cpp:112-130)
    double acc[2] = {0., 0.};
    for(int q = 0; q < nq; ++q) {
      const double pw = gT->phi[q][a] * gT->qw[q];
      acc[0] += sF[0][q][lane] * pw;
      acc[1] += sF[1][q][lane] * pw;
    }
    be[0] -= fc.srcCoeff * acc[0] * J;
    be[1] -= fc.srcCoeff * acc[1] * J;
  }
  for(int m = 0; m < 2; ++m) {
    const int32_t d = sA[2 * a + m][lane];
    if(d < nInc) atomicAdd(rhs + d, be[m]);  // one contribution per DOF and color
  }
  if(fc.hasDivu && a < 3) {
    // Be_pj -= c div u psi_j jac w   (feVectorSysElm.cpp:722-747), j = a
    double acc = 0.;
    for(int b = 0; b < 6; ++b)
      for(int n = 0; n < 2; ++n)
        acc += sU[2 * b + n][lane] * (G[0][n] * sT.D[0][a][b] + G[1][n] * sT.D[1][a][b]);
    const int32_t d = sA[12 + a][lane];
    if(d < nInc) atomicAdd(rhs + d, -fc.divu * acc * J);
  }
}

// ---------------------------------------------------------------------------
// Residual, Taylor-Hood, by quadrature with a 7-node rule exact to degree 5
// (used when the form's own rule is also exact to degree 5, so that both
// compute the exact integrals of these polynomial integrands and agree to
// rounding).  The quadrature-node fluxes are computed once per element
// (threads of the element split the nodes) and projected onto each test
// function: about a quarter of the FP64 work of the tensor contraction.
// Sources keep the form's own rule (their integrands are not polynomial).
//   Be_(a,m) = sum_q [ Fphi_m phi_a + sum_r H_rm dphi_a/dr ]
//   Fphi_m   = w |J| ( -c_conv (u . grad) u_m - c_mass udot_m )
//   H_rm     = sum_k G[r][k] w |J| ( -sigma ( p delta_km - mu (d_k u_m + d_m u_k) ) )
//   Be_pj    = sum_q w |J| ( -c_div div u ) psi_j
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(EPB * 6) k_residual_th_q(DeviceMesh dm, FormCoeffs fc,
                                                          const RefTensors *__restrict__ gT,
                                                          const double *__restrict__ u,
                                                          const double *__restrict__ udot, double t,
                                                          int64_t nInc, double *__restrict__ rhs,
                                                          int64_t begin, int64_t end)
{
  __shared__ double sU[12][EPB];
  __shared__ double sUd[12][EPB];
  __shared__ double sP[3][EPB];
  __shared__ double sG[5][EPB];
  __shared__ double sQ[7][7][EPB];
  __shared__ double sF[2][16][EPB];
  __shared__ int32_t sA[15][EPB];
  const int lane = threadIdx.x, a = threadIdx.y;
  const int64_t p = begin + (int64_t)blockIdx.x * EPB + lane;
  const bool live = p < end;
  const int64_t nE = dm.nElm;
  const bool hasSrc = fc.srcKind != SRC_NONE;
  if(live) {
    for(int i = a; i < 15; i += 6) {
      int32_t d = dm.adr[(int64_t)i * nE + p];
      sA[i][lane] = d;
      if(i < 12) {
        sU[i][lane] = u[d];
        sUd[i][lane] = fc.hasMass ? udot[d] : 0.;
      } else {
        sP[i - 12][lane] = u[d];
      }
    }
    if(a < 5) sG[a][lane] = dm.geo[(int64_t)a * nE + p];
  }
  const int nq = gT->nq;
  if(hasSrc && live) {
    const double x0 = dm.xy[0 * nE + p], y0 = dm.xy[1 * nE + p], x1 = dm.xy[2 * nE + p],
                 y1 = dm.xy[3 * nE + p], x2 = dm.xy[4 * nE + p], y2 = dm.xy[5 * nE + p];
    for(int q = a; q < nq; q += 6) {
      const double r = gT->qr[q], s = gT->qs[q];
      const double x = x0 * (1. - r - s) + x1 * r + x2 * s;
      const double y = y0 * (1. - r - s) + y1 * r + y2 * s;
      double f[2];
      source_value(fc.srcKind, fc.srcParam, x, y, f);
      sF[0][q][lane] = f[0];
      sF[1][q][lane] = f[1];
    }
  }
  __syncthreads();
  if(live) {
    const double G[2][2] = {{sG[0][lane], sG[1][lane]}, {sG[2][lane], sG[3][lane]}};
    const double J = sG[4][lane];
    for(int q = a; q < 7; q += 6) {
      double uq[2] = {0., 0.}, ur[2] = {0., 0.}, us[2] = {0., 0.}, udq[2] = {0., 0.};
      for(int b = 0; b < 6; ++b) {
        const double ph = gT->phi5[q][b], dr = gT->dr5[q][b], ds = gT->ds5[q][b];
        for(int m = 0; m < 2; ++m) {
          const double v = sU[2 * b + m][lane];
          uq[m] += ph * v;
          ur[m] += dr * v;
          us[m] += ds * v;
          udq[m] += ph * sUd[2 * b + m][lane];
        }
      }
      double gu[2][2];  // gu[k][m] = d_k u_m
      for(int k = 0; k < 2; ++k)
        for(int m = 0; m < 2; ++m) gu[k][m] = G[0][k] * ur[m] + G[1][k] * us[m];
      const double pq = gT->psi5[q][0] * sP[0][lane] + gT->psi5[q][1] * sP[1][lane] + gT->psi5[q][2] * sP[2][lane];
      const double wJ = gT->w5[q] * J;
      for(int m = 0; m < 2; ++m) {
        double f = 0.;
        if(fc.hasConv) f -= fc.conv * (uq[0] * gu[0][m] + uq[1] * gu[1][m]);
        if(fc.hasMass) f -= fc.mass * udq[m];
        sQ[q][m][lane] = wJ * f;
      }
      double Fg[2][2] = {{0., 0.}, {0., 0.}};  // coefficient of d_k phi_a, component m
      if(fc.hasSigma)
        for(int k = 0; k < 2; ++k)
          for(int m = 0; m < 2; ++m)
            Fg[k][m] = -fc.sigma * wJ * ((k == m ? pq : 0.) - fc.mu * (gu[k][m] + gu[m][k]));
      for(int r = 0; r < 2; ++r)
        for(int m = 0; m < 2; ++m) sQ[q][2 + 2 * r + m][lane] = G[r][0] * Fg[0][m] + G[r][1] * Fg[1][m];
      sQ[q][6][lane] = fc.hasDivu ? -fc.divu * wJ * (gu[0][0] + gu[1][1]) : 0.;
    }
  }
  __syncthreads();
  if(!live) return;
  const double J = sG[4][lane];
  double be[2] = {0., 0.};
  for(int q = 0; q < 7; ++q) {
    const double ph = gT->phi5[q][a], dr = gT->dr5[q][a], ds = gT->ds5[q][a];
    for(int m = 0; m < 2; ++m) be[m] += sQ[q][m][lane] * ph + sQ[q][2 + m][lane] * dr + sQ[q][4 + m][lane] * ds;
  }
  if(hasSrc) {
    // Be_(a,m) -= f . phi jac w   (feVectorSysElm.cpp:112-130), the form's own rule
    double acc[2] = {0., 0.};
    for(int q = 0; q < nq; ++q) {
      const double pw = gT->phi[q][a] * gT->qw[q];
      acc[0] += sF[0][q][lane] * pw;
      acc[1] += sF[1][q][lane] * pw;
    }
    be[0] -= fc.srcCoeff * acc[0] * J;
    be[1] -= fc.srcCoeff * acc[1] * J;
  }
  for(int m = 0; m < 2; ++m) {
    const int32_t d = sA[2 * a + m][lane];
    if(d < nInc) atomicAdd(rhs + d, be[m]);  // one contribution per DOF and color
  }
  if(fc.hasDivu && a < 3) {
    double acc = 0.;
    for(int q = 0; q < 7; ++q) acc += sQ[q][6][lane] * gT->psi5[q][a];
    const int32_t d = sA[12 + a][lane];
    if(d < nInc) atomicAdd(rhs + d, acc);
  }
}

// k_residual_th_q in double-float: the same 7-node quadrature, the same
// sums in the same order; sources (non-polynomial) and the scatter in FP64.
// Block: 32 elements x 7 warps.  Quadrature node q is warp q; then warps
// 0-5 form the two velocity rows of P2 function a = warp, warp 6 the three
// pressure rows.  Inputs are already float pairs (no FP64 arithmetic but
// the source and the final scatter).
__global__ void __launch_bounds__(EPB * 7) k_residual_th_df(DeviceMesh dm, FormCoeffs fc,
                                                           const RefTensors *__restrict__ gT,
                                                           const float2 *__restrict__ up,
                                                           const float2 *__restrict__ udp, double t,
                                                           int64_t nInc, double *__restrict__ rhs,
                                                           int64_t begin, int64_t end)
{
  __shared__ dfl sU[12][EPB];
  __shared__ dfl sUd[12][EPB];
  __shared__ dfl sP[3][EPB];
  __shared__ dfl sG[5][EPB];
  __shared__ dfl sQ[7][7][EPB];
  __shared__ double sF[2][16][EPB];
  __shared__ int32_t sA[15][EPB];
  const int lane = threadIdx.x, a = threadIdx.y;
  const int64_t p = begin + (int64_t)blockIdx.x * EPB + lane;
  const bool live = p < end;
  const int64_t nE = dm.nElm;
  const bool hasSrc = fc.srcKind != SRC_NONE;
  if(live) {
    for(int i = a; i < 15; i += 7) {
      int32_t d = dm.adr[(int64_t)i * nE + p];
      sA[i][lane] = d;
      const float2 v = up[d];
      if(i < 12) {
        sU[i][lane] = {v.x, v.y};
        if(fc.hasMass) {
          const float2 w = udp[d];
          sUd[i][lane] = {w.x, w.y};
        } else {
          sUd[i][lane] = df_zero();
        }
      } else {
        sP[i - 12][lane] = {v.x, v.y};
      }
    }
    if(a < 5) {
      const float2 g = dm.geoPair[(int64_t)a * nE + p];
      sG[a][lane] = {g.x, g.y};
    }
  }
  const int nq = gT->nq;
  if(hasSrc && live) {
    const double x0 = dm.xy[0 * nE + p], y0 = dm.xy[1 * nE + p], x1 = dm.xy[2 * nE + p],
                 y1 = dm.xy[3 * nE + p], x2 = dm.xy[4 * nE + p], y2 = dm.xy[5 * nE + p];
    for(int q = a; q < nq; q += 7) {
      const double r = gT->qr[q], s = gT->qs[q];
      const double x = x0 * (1. - r - s) + x1 * r + x2 * s;
      const double y = y0 * (1. - r - s) + y1 * r + y2 * s;
      double f[2];
      source_value(fc.srcKind, fc.srcParam, x, y, f);
      sF[0][q][lane] = f[0];
      sF[1][q][lane] = f[1];
    }
  }
  __syncthreads();
  if(live) {
    const dfl G[2][2] = {{sG[0][lane], sG[1][lane]}, {sG[2][lane], sG[3][lane]}};
    const dfl J = sG[4][lane];
    const dfl conv = {fc.pair[0][0], fc.pair[0][1]}, mass = {fc.pair[1][0], fc.pair[1][1]},
              sig = {fc.pair[2][0], fc.pair[2][1]}, mu = {fc.pair[3][0], fc.pair[3][1]},
              divu = {fc.pair[4][0], fc.pair[4][1]};
    const int q = a;  // one quadrature node per warp
    dfl uq[2] = {df_zero(), df_zero()}, ur[2] = {df_zero(), df_zero()}, us[2] = {df_zero(), df_zero()},
        udq[2] = {df_zero(), df_zero()};
    for(int b = 0; b < 6; ++b) {
      const dfl ph = {gT->phi5h[q][b], gT->phi5l[q][b]}, dr = {gT->dr5h[q][b], gT->dr5l[q][b]},
                ds = {gT->ds5h[q][b], gT->ds5l[q][b]};
      for(int m = 0; m < 2; ++m) {
        const dfl v = sU[2 * b + m][lane];
        uq[m] = df_fma(ph, v, uq[m]);
        ur[m] = df_fma(dr, v, ur[m]);
        us[m] = df_fma(ds, v, us[m]);
        if(fc.hasMass) udq[m] = df_fma(ph, sUd[2 * b + m][lane], udq[m]);
      }
    }
    dfl gu[2][2];  // gu[k][m] = d_k u_m
    for(int k = 0; k < 2; ++k)
      for(int m = 0; m < 2; ++m) gu[k][m] = df_add(df_mul(G[0][k], ur[m]), df_mul(G[1][k], us[m]));
    dfl pq = df_zero();
    for(int j = 0; j < 3; ++j) pq = df_fma({gT->psi5h[q][j], gT->psi5l[q][j]}, sP[j][lane], pq);
    const dfl wJ = df_mul({gT->w5h[q], gT->w5l[q]}, J);
    for(int m = 0; m < 2; ++m) {
      dfl f = df_zero();
      if(fc.hasConv) f = df_sub(f, df_mul(conv, df_add(df_mul(uq[0], gu[0][m]), df_mul(uq[1], gu[1][m]))));
      if(fc.hasMass) f = df_sub(f, df_mul(mass, udq[m]));
      sQ[q][m][lane] = df_mul(wJ, f);
    }
    dfl Fg[2][2] = {{df_zero(), df_zero()}, {df_zero(), df_zero()}};  // coefficient of d_k phi_a, component m
    if(fc.hasSigma) {
      const dfl sw = df_neg(df_mul(sig, wJ));
      for(int k = 0; k < 2; ++k)
        for(int m = 0; m < 2; ++m) {
          const dfl in = df_sub(k == m ? pq : df_zero(), df_mul(mu, df_add(gu[k][m], gu[m][k])));
          Fg[k][m] = df_mul(sw, in);
        }
    }
    for(int r = 0; r < 2; ++r)
      for(int m = 0; m < 2; ++m)
        sQ[q][2 + 2 * r + m][lane] = df_add(df_mul(G[r][0], Fg[0][m]), df_mul(G[r][1], Fg[1][m]));
    sQ[q][6][lane] = fc.hasDivu ? df_neg(df_mul(df_mul(divu, wJ), df_add(gu[0][0], gu[1][1]))) : df_zero();
  }
  __syncthreads();
  if(!live) return;
  if(a == 6) {
    // the three pressure rows
    if(!fc.hasDivu) return;
    for(int j = 0; j < 3; ++j) {
      dfl acc = df_zero();
      for(int q = 0; q < 7; ++q) acc = df_fma(sQ[q][6][lane], {gT->psi5h[q][j], gT->psi5l[q][j]}, acc);
      const int32_t d = sA[12 + j][lane];
      if(d < nInc) atomicAdd(rhs + d, df_to(acc));
    }
    return;
  }
  dfl be[2] = {df_zero(), df_zero()};
  for(int q = 0; q < 7; ++q) {
    const dfl ph = {gT->phi5h[q][a], gT->phi5l[q][a]}, dr = {gT->dr5h[q][a], gT->dr5l[q][a]},
              ds = {gT->ds5h[q][a], gT->ds5l[q][a]};
    for(int m = 0; m < 2; ++m)
      be[m] = df_add(be[m], df_add(df_add(df_mul(sQ[q][m][lane], ph), df_mul(sQ[q][2 + m][lane], dr)),
                                   df_mul(sQ[q][4 + m][lane], ds)));
  }
  double bd[2] = {df_to(be[0]), df_to(be[1])};
  if(hasSrc) {
    // Be_(a,m) -= f . phi jac w   (feVectorSysElm.cpp:112-130), the form's own rule, in FP64
    const double J = dm.geo[(int64_t)4 * nE + p];
    double acc[2] = {0., 0.};
    for(int q = 0; q < nq; ++q) {
      const double pw = gT->phi[q][a] * gT->qw[q];
      acc[0] += sF[0][q][lane] * pw;
      acc[1] += sF[1][q][lane] * pw;
    }
    bd[0] -= fc.srcCoeff * acc[0] * J;
    bd[1] -= fc.srcCoeff * acc[1] * J;
  }
  for(int m = 0; m < 2; ++m) {
    const int32_t d = sA[2 * a + m][lane];
    if(d < nInc) atomicAdd(rhs + d, bd[m]);  // one contribution per DOF and color
  }
}

__global__ void k_split_pairs(int64_t n, const double *__restrict__ x, float2 *__restrict__ out)
{
  for(int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double v = x[i];
    const float h = __double2float_rn(v);
    out[i] = make_float2(h, __double2float_rn(v - (double)h));
  }
}

// Local entry k = a*18 + j of the staged rows (2a+m) of a Taylor-Hood
// element matrix -> index of the element-to-nonzero map (i = 2a+m; j < 12
// velocity column j, 12 <= j < 15 pressure column j-12, 15 <= j < 18 the
// entry of pressure row j-15 in column i).
__device__ __forceinline__ int th_map_index(int k, int m)
{
  const int a = k / 18, j = k % 18, i = 2 * a + m;
  return j < 15 ? i * 15 + j : (12 + j - 15) * 15 + i;
}

template <typename V>
__device__ __forceinline__ void scatter_staged(const int32_t *__restrict__ map, int64_t nE, int64_t p0, int64_t end,
                                               int hasSigma, int hasDivu, int m, const V (*sAdd)[EPB],
                                               V *__restrict__ values)
{
  const int tid = threadIdx.y * EPB + threadIdx.x;
  constexpr int NT = EPB * 6, TOTAL = 108 * EPB, BATCH = 6;
  for(int base = tid; base < TOTAL; base += NT * BATCH) {
    int32_t pos[BATCH];
    V add[BATCH];
#pragma unroll
    for(int q = 0; q < BATCH; ++q) {
      const int idx = base + q * NT;
      pos[q] = -1;
      add[q] = 0;
      if(idx < TOTAL) {
        const int e = idx % EPB, k = idx / EPB, j = k % 18;
        const bool on = (j < 12) || (j < 15 ? hasSigma : hasDivu);
        if(on && p0 + e < end) {
          pos[q] = __ldg(map + (int64_t)th_map_index(k, m) * nE + p0 + e);
          add[q] = sAdd[k][e];
        }
      }
    }
    // Within one color every CSR entry receives at most one contribution, so
    // the reduction in L2 (no round trip to the SM) gives the same bits as
    // a read-modify-write.
#pragma unroll
    for(int q = 0; q < BATCH; ++q)
      if(pos[q] >= 0) atomicAdd(values + pos[q], add[q]);
  }
}

// ---------------------------------------------------------------------------
// Jacobian, Taylor-Hood P2-P1.
// ---------------------------------------------------------------------------
template <typename V>
__global__ void __launch_bounds__(EPB * 6) k_matrix_th(DeviceMesh dm, FormCoeffs fc,
                                                      const RefTensors *__restrict__ gT,
                                                      const double *__restrict__ u, double c0,
                                                      V *__restrict__ values, int64_t begin,
                                                      int64_t end)
{
  __shared__ SharedTensors<V> sT;
  __shared__ V sU[12][EPB];
  __shared__ V sG[5][EPB];
  __shared__ V sAdd[108][EPB];
  const int lane = threadIdx.x, a = threadIdx.y;
  const int64_t p = begin + (int64_t)blockIdx.x * EPB + lane;
  const bool live = p < end;
  const int64_t nE = dm.nElm;
  load_tensors(sT, gT);
  if(live) {
    if(fc.hasConv)
      for(int i = a; i < 12; i += 6) sU[i][lane] = (V)u[dm.adr[(int64_t)i * nE + p]];
    if(a < 5) sG[a][lane] = (V)dm.geo[(int64_t)a * nE + p];
  } else {
    // Past the end of the color: zero data, entries never scattered.
    for(int i = a; i < 12; i += 6) sU[i][lane] = 0;
    if(a < 5) sG[a][lane] = 0;
  }
  __syncthreads();
  const V G[2][2] = {{sG[0][lane], sG[1][lane]}, {sG[2][lane], sG[3][lane]}};
  const V J = sG[4][lane];

  // Element rows (a,0) and (a,1): 12 velocity columns + 3 pressure columns.
  V A[2][12];
#pragma unroll
  for(int m = 0; m < 2; ++m)
#pragma unroll
    for(int j = 0; j < 12; ++j) A[m][j] = 0;

  if(fc.hasConv) {
    // A_(a,m),(b,n) += c [ delta_mn phi_a (u0 . grad phi_b) + phi_a phi_b d_n u0_m ]
    // (vectorDotGradShapeDotShape + shapeDotTensorDotShape, feVectorSpace.cpp:202-290)
    V V0[2][6];
    for(int c = 0; c < 6; ++c)
      for(int r = 0; r < 2; ++r) V0[r][c] = sU[2 * c][lane] * G[r][0] + sU[2 * c + 1][lane] * G[r][1];
    const V cc = (V)fc.conv * J;
    for(int b = 0; b < 6; ++b) {
      V W = 0, Z[2][2] = {{0, 0}, {0, 0}};  // Z[r][m] = sum_c U_cm T[r][a][b][c]
      for(int c = 0; c < 6; ++c) {
        W += V0[0][c] * sT.T[0][a][c][b] + V0[1][c] * sT.T[1][a][c][b];
        const V t0 = sT.T[0][a][b][c], t1 = sT.T[1][a][b][c];
        const V uc0 = sU[2 * c][lane], uc1 = sU[2 * c + 1][lane];
        Z[0][0] += uc0 * t0; Z[0][1] += uc1 * t0;
        Z[1][0] += uc0 * t1; Z[1][1] += uc1 * t1;
      }
      for(int m = 0; m < 2; ++m)
        for(int n = 0; n < 2; ++n) {
          V v = G[0][n] * Z[0][m] + G[1][n] * Z[1][m];
          if(m == n) v += W;
          A[m][2 * b + n] += cc * v;
        }
    }
  }
  if(fc.hasSigma) {
    // A_(a,m),(b,n) += -c mu [ delta_mn grad phi_a . grad phi_b + d_n phi_a d_m phi_b ]
    // (feVectorSysElm.cpp:1454-1492)
    const V cs = -(V)fc.sigma * (V)fc.mu * J;
    V GG[2][2][2][2];
    for(int k = 0; k < 2; ++k)
      for(int l = 0; l < 2; ++l)
        for(int r = 0; r < 2; ++r)
          for(int s2 = 0; s2 < 2; ++s2) GG[k][l][r][s2] = G[r][k] * G[s2][l];
    for(int b = 0; b < 6; ++b) {
      V S[2][2];
      for(int k = 0; k < 2; ++k)
        for(int l = 0; l < 2; ++l) {
          V v = 0;
          for(int r = 0; r < 2; ++r)
            for(int s2 = 0; s2 < 2; ++s2) v += GG[k][l][r][s2] * sT.K[r][s2][a][b];
          S[k][l] = v;
        }
      const V tr = S[0][0] + S[1][1];
      for(int m = 0; m < 2; ++m)
        for(int n = 0; n < 2; ++n) A[m][2 * b + n] += cs * ((m == n ? tr : (V)0) + S[n][m]);
    }
  }
  if(fc.hasMass) {
    // A_(a,m),(b,n) += c c0 delta_mn phi_a phi_b   (feVectorSysElm.cpp:390-408)
    const V cm = (V)fc.mass * (V)c0 * J;
    for(int b = 0; b < 6; ++b) {
      A[0][2 * b] += cm * sT.M[a][b];
      A[1][2 * b + 1] += cm * sT.M[a][b];
    }
  }
  // Pressure columns of rows (a,m) and the column (a,m) of the pressure rows:
  // both are int psi_j d_m phi_a.
  V Bp[2][3];
  for(int m = 0; m < 2; ++m)
    for(int j = 0; j < 3; ++j) Bp[m][j] = (G[0][m] * sT.D[0][j][a] + G[1][m] * sT.D[1][j][a]) * J;

  // Stage the element's 216 structurally nonzero entries in shared memory
  // (thread (e, a): rows 2a+m, velocity + pressure columns, and the
  // pressure-row entries in columns 2a+m), then scatter them block-wide: consecutive
  // threads take consecutive elements of one entry, so the map reads are
  // coalesced and every thread keeps several read-modify-writes in flight.
  // (two passes, one row component m at a time, to bound shared memory)
#pragma unroll
  for(int m = 0; m < 2; ++m) {
    if(m) __syncthreads();
#pragma unroll
    for(int j = 0; j < 12; ++j) sAdd[a * 18 + j][lane] = A[m][j];
#pragma unroll
    for(int j = 0; j < 3; ++j) {
      sAdd[a * 18 + 12 + j][lane] = fc.hasSigma ? (V)fc.sigma * Bp[m][j] : (V)0;
      sAdd[a * 18 + 15 + j][lane] = fc.hasDivu ? (V)fc.divu * Bp[m][j] : (V)0;
    }
    __syncthreads();
    scatter_staged<V>(dm.map, nE, begin + (int64_t)blockIdx.x * EPB, end, fc.hasSigma, fc.hasDivu, m, sAdd,
                      values);
  }
}

int64_t nblocks(int64_t begin, int64_t end) { return (end - begin + EPB - 1) / EPB; }

// ---------------------------------------------------------------------------
// Row-owned Jacobian, Taylor-Hood.
// ---------------------------------------------------------------------------
template <typename V>
__global__ void k_pack_th(DeviceMesh dm, int hasConv, const double *__restrict__ u, V *__restrict__ pack)
{
  const int64_t nE = dm.nElm;
  for(int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < nE; p += (int64_t)gridDim.x * blockDim.x) {
    V *o = pack + p * ROWASM_PACK;
#pragma unroll
    for(int i = 0; i < 12; ++i) o[i] = hasConv ? (V)u[dm.adr[(int64_t)i * nE + p]] : (V)0;
#pragma unroll
    for(int k = 0; k < 5; ++k) o[12 + k] = (V)dm.geo[(int64_t)k * nE + p];
  }
}

// Both component rows (a, 0) and (a, 1) of velocity function a of an
// element, from its packed data e (u, G, J): A[m][12] velocity columns and
// the pressure-column factors Bp[m][3] -- k_matrix_th's arithmetic for one
// (element, a).
template <typename V>
__device__ __forceinline__ void th_rows_pair(const SharedTensors<V> &sT, const FormCoeffs &fc, double c0,
                                             const V *e, int a, V (&A)[2][12], V (&Bp)[2][3])
{
  const V G[2][2] = {{e[12], e[13]}, {e[14], e[15]}};
  const V J = e[16];
#pragma unroll
  for(int m = 0; m < 2; ++m)
#pragma unroll
    for(int j = 0; j < 12; ++j) A[m][j] = 0;
  if(fc.hasConv) {
    V U[12];
#pragma unroll
    for(int i = 0; i < 12; ++i) U[i] = e[i];
    V V0[2][6];
#pragma unroll
    for(int c = 0; c < 6; ++c)
#pragma unroll
      for(int q = 0; q < 2; ++q) V0[q][c] = U[2 * c] * G[q][0] + U[2 * c + 1] * G[q][1];
    const V cc = (V)fc.conv * J;
#pragma unroll
    for(int b = 0; b < 6; ++b) {
      V W = 0, Z[2][2] = {{0, 0}, {0, 0}};
#pragma unroll
      for(int c = 0; c < 6; ++c) {
        W += V0[0][c] * sT.T[0][a][c][b] + V0[1][c] * sT.T[1][a][c][b];
        const V t0 = sT.T[0][a][b][c], t1 = sT.T[1][a][b][c];
        const V uc0 = U[2 * c], uc1 = U[2 * c + 1];
        Z[0][0] += uc0 * t0; Z[0][1] += uc1 * t0;
        Z[1][0] += uc0 * t1; Z[1][1] += uc1 * t1;
      }
#pragma unroll
      for(int m = 0; m < 2; ++m)
#pragma unroll
        for(int n = 0; n < 2; ++n) {
          V v = G[0][n] * Z[0][m] + G[1][n] * Z[1][m];
          if(m == n) v += W;
          A[m][2 * b + n] += cc * v;
        }
    }
  }
  if(fc.hasSigma) {
    const V cs = -(V)fc.sigma * (V)fc.mu * J;
    V GG[2][2][2][2];
#pragma unroll
    for(int k = 0; k < 2; ++k)
#pragma unroll
      for(int l = 0; l < 2; ++l)
#pragma unroll
        for(int q = 0; q < 2; ++q)
#pragma unroll
          for(int s2 = 0; s2 < 2; ++s2) GG[k][l][q][s2] = G[q][k] * G[s2][l];
#pragma unroll
    for(int b = 0; b < 6; ++b) {
      V S[2][2];
#pragma unroll
      for(int k = 0; k < 2; ++k)
#pragma unroll
        for(int l = 0; l < 2; ++l) {
          V v = 0;
#pragma unroll
          for(int q = 0; q < 2; ++q)
#pragma unroll
            for(int s2 = 0; s2 < 2; ++s2) v += GG[k][l][q][s2] * sT.K[q][s2][a][b];
          S[k][l] = v;
        }
      const V tr = S[0][0] + S[1][1];
#pragma unroll
      for(int m = 0; m < 2; ++m)
#pragma unroll
        for(int n = 0; n < 2; ++n) A[m][2 * b + n] += cs * ((m == n ? tr : (V)0) + S[n][m]);
    }
  }
  if(fc.hasMass) {
    const V cm = (V)fc.mass * (V)c0 * J;
#pragma unroll
    for(int b = 0; b < 6; ++b) {
      A[0][2 * b] += cm * sT.M[a][b];
      A[1][2 * b + 1] += cm * sT.M[a][b];
    }
  }
#pragma unroll
  for(int m = 0; m < 2; ++m)
#pragma unroll
    for(int j = 0; j < 3; ++j) Bp[m][j] = (G[0][m] * sT.D[0][j][a] + G[1][m] * sT.D[1][j][a]) * J;
}

// Thread = unit (RowAsm): a pair of component rows of one velocity node, or
// one row.  Entry (p, li): li < 12 is velocity row (a = li / 2, component
// m = li % 2) of element p, whose 12 velocity and 3 pressure columns are the
// element-matrix row of k_matrix_th; li >= 12 is pressure row j = li - 12,
// whose 12 velocity columns are divu * int psi_j d_m phi_a.  A pair takes
// the entries of its component-0 row and builds both rows (same columns,
// same offsets); the arithmetic is k_matrix_th's.
template <typename V>
__global__ void __launch_bounds__(256) k_matrix_th_rows(RowAsm ra, FormCoeffs fc, const RefTensors *__restrict__ gT,
                                                        double c0, V *__restrict__ values, int accumulate)
{
  extern __shared__ __align__(16) unsigned char rowsmem[];
  V *sv = reinterpret_cast<V *>(rowsmem);
  __shared__ SharedTensors<V> sT;
  load_tensors(sT, gT);
  const int32_t uA = ra.blockUnits[blockIdx.x], uB = ra.blockUnits[blockIdx.x + 1];
  const int32_t base = ra.ia[ra.unitRow[uA]], L = ra.ia[ra.unitRow[uB]] - base;
  for(int i = threadIdx.x; i < L; i += blockDim.x) sv[i] = accumulate ? values[base + i] : (V)0;
  __syncthreads();
  const int32_t u = uA + (int32_t)threadIdx.x;
  if(u < uB && ra.unitTwo[u]) {
    const int32_t r = ra.unitRow[u];
    V *row0 = sv + (ra.ia[r] - base), *row1 = sv + (ra.ia[r + 1] - base);
    const V *pk = reinterpret_cast<const V *>(ra.pack);
    for(int32_t k = ra.rowPtr[r]; k < ra.rowPtr[r + 1]; ++k) {
      const int32_t ent = ra.rowEnt[k];
      const int64_t p = ent >> 4;
      const int a = (ent & 15) >> 1;
      uint8_t off[16];
      *reinterpret_cast<uint4 *>(off) = reinterpret_cast<const uint4 *>(ra.offs)[k];
      V A[2][12], Bp[2][3];
      th_rows_pair<V>(sT, fc, c0, pk + p * ROWASM_PACK, a, A, Bp);
#pragma unroll
      for(int j = 0; j < 12; ++j)
        if(off[j] != 255) {
          row0[off[j]] += A[0][j];
          row1[off[j]] += A[1][j];
        }
#pragma unroll
      for(int j = 0; j < 3; ++j)
        if(off[12 + j] != 255) {
          row0[off[12 + j]] += fc.hasSigma ? (V)fc.sigma * Bp[0][j] : (V)0;
          row1[off[12 + j]] += fc.hasSigma ? (V)fc.sigma * Bp[1][j] : (V)0;
        }
    }
  } else if(u < uB) {
    const int32_t r = ra.unitRow[u];
    V *row = sv + (ra.ia[r] - base);
    const V *pk = reinterpret_cast<const V *>(ra.pack);
    for(int32_t k = ra.rowPtr[r]; k < ra.rowPtr[r + 1]; ++k) {
      const int32_t ent = ra.rowEnt[k];
      const int64_t p = ent >> 4;
      const int li = ent & 15;
      uint8_t off[16];
      *reinterpret_cast<uint4 *>(off) = reinterpret_cast<const uint4 *>(ra.offs)[k];
      const V *e = pk + p * ROWASM_PACK;
      const V G[2][2] = {{e[12], e[13]}, {e[14], e[15]}};
      const V J = e[16];
      if(li < 12) {
        const int a = li >> 1, m = li & 1;
        V A[12];
#pragma unroll
        for(int j = 0; j < 12; ++j) A[j] = 0;
        if(fc.hasConv) {
          V U[12];
#pragma unroll
          for(int i = 0; i < 12; ++i) U[i] = e[i];
          V V0[2][6];
#pragma unroll
          for(int c = 0; c < 6; ++c)
#pragma unroll
            for(int q = 0; q < 2; ++q) V0[q][c] = U[2 * c] * G[q][0] + U[2 * c + 1] * G[q][1];
          const V cc = (V)fc.conv * J;
#pragma unroll
          for(int b = 0; b < 6; ++b) {
            V W = 0, Z0 = 0, Z1 = 0;  // Z_q = sum_c U_cm T[q][a][b][c]
#pragma unroll
            for(int c = 0; c < 6; ++c) {
              W += V0[0][c] * sT.T[0][a][c][b] + V0[1][c] * sT.T[1][a][c][b];
              const V t0 = sT.T[0][a][b][c], t1 = sT.T[1][a][b][c];
              const V ucm = U[2 * c + m];
              Z0 += ucm * t0;
              Z1 += ucm * t1;
            }
#pragma unroll
            for(int n = 0; n < 2; ++n) {
              V v = G[0][n] * Z0 + G[1][n] * Z1;
              if(m == n) v += W;
              A[2 * b + n] += cc * v;
            }
          }
        }
        if(fc.hasSigma) {
          const V cs = -(V)fc.sigma * (V)fc.mu * J;
          V GG[2][2][2][2];
#pragma unroll
          for(int kk = 0; kk < 2; ++kk)
#pragma unroll
            for(int l = 0; l < 2; ++l)
#pragma unroll
              for(int q = 0; q < 2; ++q)
#pragma unroll
                for(int s2 = 0; s2 < 2; ++s2) GG[kk][l][q][s2] = G[q][kk] * G[s2][l];
#pragma unroll
          for(int b = 0; b < 6; ++b) {
            V S[2][2];
#pragma unroll
            for(int kk = 0; kk < 2; ++kk)
#pragma unroll
              for(int l = 0; l < 2; ++l) {
                V v = 0;
#pragma unroll
                for(int q = 0; q < 2; ++q)
#pragma unroll
                  for(int s2 = 0; s2 < 2; ++s2) v += GG[kk][l][q][s2] * sT.K[q][s2][a][b];
                S[kk][l] = v;
              }
            const V tr = S[0][0] + S[1][1];
#pragma unroll
            for(int n = 0; n < 2; ++n) A[2 * b + n] += cs * ((m == n ? tr : (V)0) + S[n][m]);
          }
        }
        if(fc.hasMass) {
          const V cm = (V)fc.mass * (V)c0 * J;
#pragma unroll
          for(int b = 0; b < 6; ++b) A[2 * b + m] += cm * sT.M[a][b];
        }
#pragma unroll
        for(int j = 0; j < 12; ++j)
          if(off[j] != 255) row[off[j]] += A[j];
#pragma unroll
        for(int j = 0; j < 3; ++j) {
          const V bp = (G[0][m] * sT.D[0][j][a] + G[1][m] * sT.D[1][j][a]) * J;
          if(off[12 + j] != 255) row[off[12 + j]] += fc.hasSigma ? (V)fc.sigma * bp : (V)0;
        }
      } else {
        const int j = li - 12;
#pragma unroll
        for(int a = 0; a < 6; ++a)
#pragma unroll
          for(int m = 0; m < 2; ++m) {
            const V bp = (G[0][m] * sT.D[0][j][a] + G[1][m] * sT.D[1][j][a]) * J;
            if(off[2 * a + m] != 255) row[off[2 * a + m]] += fc.hasDivu ? (V)fc.divu * bp : (V)0;
          }
      }
    }
  }
  __syncthreads();
  for(int i = threadIdx.x; i < L; i += blockDim.x) values[base + i] = sv[i];
}

int pack_grid(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 8192)); }

}  // namespace

void launch_pack_th_f32(const DeviceMesh &dm, const FormCoeffs &fc, const double *u, float *pack, cudaStream_t s)
{
  (k_pack_th<float><<<pack_grid(dm.nElm), 256, 0, s>>>(dm, fc.hasConv, u, pack), ::feng::count_launch());
}

void launch_pack_th_f64(const DeviceMesh &dm, const FormCoeffs &fc, const double *u, double *pack, cudaStream_t s)
{
  (k_pack_th<double><<<pack_grid(dm.nElm), 256, 0, s>>>(dm, fc.hasConv, u, pack), ::feng::count_launch());
}

void launch_matrix_th_rows_f32(const RowAsm &ra, const FormCoeffs &fc, const RefTensors *dT, double c0,
                               float *values, int accumulate, cudaStream_t s)
{
  if(ra.nBlocks < 1) return;
  (k_matrix_th_rows<float><<<ra.nBlocks, 256, ra.capBytes, s>>>(ra, fc, dT, c0, values, accumulate),
   ::feng::count_launch());
}

void launch_matrix_th_rows_f64(const RowAsm &ra, const FormCoeffs &fc, const RefTensors *dT, double c0,
                               double *values, int accumulate, cudaStream_t s)
{
  if(ra.nBlocks < 1) return;
  (k_matrix_th_rows<double><<<ra.nBlocks, 256, ra.capBytes, s>>>(ra, fc, dT, c0, values, accumulate),
   ::feng::count_launch());
}

void launch_assemble_residual_df(const DeviceMesh &dm, const FormCoeffs &fc, const RefTensors *dT,
                                 const float2 *uPair, const float2 *udotPair, double t, int64_t nInc,
                                 double *rhs, int64_t begin, int64_t end, cudaStream_t s)
{
  if(end <= begin) return;
  (k_residual_th_df<<<nblocks(begin, end), dim3(EPB, 7), 0, s>>>(dm, fc, dT, uPair, udotPair, t, nInc, rhs, begin,
                                                                 end), ::feng::count_launch());
}

void launch_split_pairs(int64_t n, const double *x, float2 *out, cudaStream_t s)
{
  const int g = (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 4096));
  (k_split_pairs<<<g, 256, 0, s>>>(n, x, out), ::feng::count_launch());
}

void launch_assemble_residual(const DeviceMesh &dm, const FormCoeffs &fc, const RefTensors *dT,
                              const double *u, const double *udot, double t, int64_t nInc,
                              double *rhs, int64_t begin, int64_t end, cudaStream_t s, int exact5)
{
  if(end <= begin) return;
  dim3 block(EPB, 6);
  if(fc.elemType == 1)
    (k_residual_p2<<<nblocks(begin, end), block, 0, s>>>(dm, fc, dT, u, t, nInc, rhs, begin, end), ::feng::count_launch());
  else if(exact5)
    (k_residual_th_q<<<nblocks(begin, end), block, 0, s>>>(dm, fc, dT, u, udot, t, nInc, rhs, begin,
                                                          end), ::feng::count_launch());
  else
    (k_residual_th<<<nblocks(begin, end), block, 0, s>>>(dm, fc, dT, u, udot, t, nInc, rhs, begin,
                                                        end), ::feng::count_launch());
}

void launch_assemble_matrix_f64(const DeviceMesh &dm, const FormCoeffs &fc, const RefTensors *dT,
                                const double *u, double c0, double *values, int64_t begin,
                                int64_t end, cudaStream_t s)
{
  if(end <= begin) return;
  dim3 block(EPB, 6);
  if(fc.elemType == 1)
    (k_matrix_p2<double><<<nblocks(begin, end), block, 0, s>>>(dm, fc, dT, values, begin, end), ::feng::count_launch());
  else
    (k_matrix_th<double><<<nblocks(begin, end), block, 0, s>>>(dm, fc, dT, u, c0, values, begin, end), ::feng::count_launch());
}

void launch_assemble_matrix_f32(const DeviceMesh &dm, const FormCoeffs &fc, const RefTensors *dT,
                                const double *u, double c0, float *values, int64_t begin,
                                int64_t end, cudaStream_t s)
{
  if(end <= begin) return;
  dim3 block(EPB, 6);
  if(fc.elemType == 1)
    (k_matrix_p2<float><<<nblocks(begin, end), block, 0, s>>>(dm, fc, dT, values, begin, end), ::feng::count_launch());
  else
    (k_matrix_th<float><<<nblocks(begin, end), block, 0, s>>>(dm, fc, dT, u, c0, values, begin, end), ::feng::count_launch());
}

}  // namespace feng
