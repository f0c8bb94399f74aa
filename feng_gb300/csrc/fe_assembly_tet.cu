// Element assembly on tetrahedra: scalar P2 (DIFFUSION + SOURCE, the
// reference's feSysElm_Diffusion<3> and feSysElm_Source on feSpaceTetPn(2),
// src/feSysElm.cpp:16-27, 520-589) and Taylor-Hood P2-P1 (the vector forms
// of src/feVectorSysElm.cpp in three dimensions, which the reference
// instantiates only in two).
//
// Colored kernels: one launch per element color; a block holds 32 elements
// (lane = element) x 10 warps (warp = P2 function a).  Thread (e, a) forms
// the element-matrix rows of the DOFs of function a (one scalar row, or the
// three velocity component rows), and threads a < 4 the pressure row of P1
// function a.  Entries go to the CSR values through the element-to-nonzero
// map as L2 reductions (one contribution per entry and color: the sums of a
// colored read-modify-write, in color order).
//
// Arithmetic: affine (P1) geometry, so grad phi = G^T dphi/d(r,s,t) with
// G[r][k] = d r_r / d x_k constant per element and every quadrature sum of
// the weak forms is a reference tensor (RefTensorsTet, built from the same
// rule's nodes and weights) contracted with G, J and the element's DOF values:
//   int dphi_a/dx_k dphi_b/dx_l = J sum_rs G[r][k] G[s][l] K[r][s][a][b]
//   int phi_a phi_c dphi_b/dx_k = J sum_r  G[r][k] T[r][a][c][b]
//   int psi_j dphi_a/dx_k       = J sum_r  G[r][k] D[r][j][a]
//   int phi_a phi_b             = J M[a][b]
// Source terms are summed over the rule's nodes (non-polynomial integrands).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "fe_common.h"
#include "fe_device.h"
#include "fe_df.h"
#include "fe_mesh3d.h"
#include "fe_setup.h"

namespace feng {

namespace {

constexpr int EPB = 32;
constexpr int TPB = 10;  // warps per block: one per P2 function
constexpr double PI = 3.14159265358979323846;
constexpr int NTEN = 900 + 3000 + 120 + 100;  // K, T, D, M

// x-component (or scalar value) of the tetrahedral sources at a point.
__device__ __forceinline__ double source_x(int kind, const double *p, double x, double y, double z)
{
  if(kind == SRC_SIN3 || kind == SRC_SIN3_BODY) return p[0] * sin(PI * x) * sin(PI * y) * sin(PI * z);
  return 0.;
}

template <typename V>
struct TetTensors {
  const V *K, *T, *D, *M;
  __device__ V k(int r, int s, int a, int b) const { return K[((r * 3 + s) * 10 + a) * 10 + b]; }
  __device__ V t(int r, int a, int c, int b) const { return T[((r * 10 + a) * 10 + c) * 10 + b]; }
  __device__ V d(int r, int j, int a) const { return D[(r * 4 + j) * 10 + a]; }
  __device__ V m(int a, int b) const { return M[a * 10 + b]; }
};

template <typename V>
__device__ TetTensors<V> load_tet_tensors(V *sh, const RefTensorsTet *g)
{
  const int tid = threadIdx.y * blockDim.x + threadIdx.x, nt = blockDim.x * blockDim.y;
  const double *src[4] = {&g->K[0][0][0][0], &g->T[0][0][0][0], &g->D[0][0][0], &g->M[0][0]};
  const int len[4] = {900, 3000, 120, 100};
  int off = 0;
  for(int k = 0; k < 4; ++k) {
    for(int i = tid; i < len[k]; i += nt) sh[off + i] = (V)src[k][i];
    off += len[k];
  }
  return TetTensors<V>{sh, sh + 900, sh + 3900, sh + 4020};
}

// ---------------------------------------------------------------------------
// Residual, FP64: scalar P2 and Taylor-Hood.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(EPB *TPB) k_residual_tet(DeviceMesh dm, FormCoeffs fc, const RefTensorsTet *__restrict__ gT,
                                                           const double *__restrict__ u, const double *__restrict__ udot,
                                                           int64_t nInc, double *__restrict__ rhs, int64_t begin,
                                                           int64_t end)
{
  extern __shared__ __align__(16) double smem[];
  const bool th = fc.elemType == 4;
  const int nq = gT->nq;
  double *sTen = smem;
  double *sU = sTen + NTEN;           // [30][EPB] (scalar: [10][EPB])
  double *sUd = sU + 30 * EPB;        // [30][EPB]
  double *sG = sUd + 30 * EPB;        // [10][EPB]
  double *sP = sG + 10 * EPB;         // [4][EPB]
  double *sF = sP + 4 * EPB;          // [nq][EPB]
  const int lane = threadIdx.x, a = threadIdx.y;
  const int64_t p = begin + (int64_t)blockIdx.x * EPB + lane;
  const bool live = p < end;
  const int64_t nE = dm.nElm;
  const TetTensors<double> Tt = load_tet_tensors(sTen, gT);
  if(live) {
    if(th) {
      for(int m = 0; m < 3; ++m) {
        const int32_t d = dm.adr[(int64_t)(3 * a + m) * nE + p];
        sU[(3 * a + m) * EPB + lane] = u[d];
        sUd[(3 * a + m) * EPB + lane] = (fc.hasMass && udot) ? udot[d] : 0.;
      }
      if(a < 4) sP[a * EPB + lane] = u[dm.adr[(int64_t)(30 + a) * nE + p]];
    } else {
      sU[a * EPB + lane] = u[dm.adr[(int64_t)a * nE + p]];
    }
    sG[a * EPB + lane] = dm.geo[(int64_t)a * nE + p];
    if(fc.srcKind == SRC_SIN3 || fc.srcKind == SRC_SIN3_BODY) {
      double X[4][3];
      for(int v = 0; v < 4; ++v)
        for(int k = 0; k < 3; ++k) X[v][k] = dm.xy[(int64_t)(3 * v + k) * nE + p];
      for(int q = a; q < nq; q += TPB) {
        const double r = gT->qr[q], s = gT->qs[q], t = gT->qt[q], l0 = 1. - r - s - t;
        double x[3];
        for(int k = 0; k < 3; ++k) x[k] = l0 * X[0][k] + r * X[1][k] + s * X[2][k] + t * X[3][k];
        sF[q * EPB + lane] = source_x(fc.srcKind, fc.srcParam, x[0], x[1], x[2]);
      }
    }
  }
  __syncthreads();
  if(!live) return;
  double G[3][3];
  for(int r = 0; r < 3; ++r)
    for(int k = 0; k < 3; ++k) G[r][k] = sG[(3 * r + k) * EPB + lane];
  const double J = sG[9 * EPB + lane];
  // source integral of phi_a: sum_q w phi_a(q) f(q)
  double srcA = 0.;
  if(fc.srcKind == SRC_SIN3 || fc.srcKind == SRC_SIN3_BODY)
    for(int q = 0; q < nq; ++q) srcA += gT->phi[q][a] * sF[q * EPB + lane] * gT->qw[q];
  if(!th) {
    // Be_a -= k grad phi_a . grad u   (feSysElm.cpp:558-583),  Be_a -= phi_a f   (feSysElm.cpp:16-27)
    double GG[3][3];
    for(int r = 0; r < 3; ++r)
      for(int s = 0; s < 3; ++s) GG[r][s] = G[r][0] * G[s][0] + G[r][1] * G[s][1] + G[r][2] * G[s][2];
    double acc = 0.;
    for(int b = 0; b < 10; ++b) {
      double L = 0.;
      for(int r = 0; r < 3; ++r)
        for(int s = 0; s < 3; ++s) L += GG[r][s] * Tt.k(r, s, a, b);
      acc += L * sU[b * EPB + lane];
    }
    double be = fc.hasDiff ? -fc.diff * acc * J : 0.;
    if(fc.srcKind == SRC_SIN3) be -= fc.srcCoeff * srcA * J;
    const int32_t d = dm.adr[(int64_t)a * nE + p];
    if(d < nInc) atomicAdd(rhs + d, be);
    return;
  }
  double be[3] = {0., 0., 0.};
  if(fc.hasConv) {
    // Be_(a,m) -= c int phi_a (u . grad u)_m = c J sum_b W_b u_(b,m),
    // W_b = sum_c sum_r (sum_k G[r][k] u_(c,k)) T[r][a][c][b]
    double V0[3][10];
    for(int c = 0; c < 10; ++c)
      for(int r = 0; r < 3; ++r)
        V0[r][c] = G[r][0] * sU[(3 * c) * EPB + lane] + G[r][1] * sU[(3 * c + 1) * EPB + lane] +
                   G[r][2] * sU[(3 * c + 2) * EPB + lane];
    for(int b = 0; b < 10; ++b) {
      double W = 0.;
      for(int c = 0; c < 10; ++c)
        for(int r = 0; r < 3; ++r) W += V0[r][c] * Tt.t(r, a, c, b);
      for(int m = 0; m < 3; ++m) be[m] -= fc.conv * J * W * sU[(3 * b + m) * EPB + lane];
    }
  }
  if(fc.hasSigma) {
    // Be_(a,m) -= sigma (p d_m phi_a - mu sum_n (d_n u_m + d_m u_n) d_n phi_a)
    //   = -sigma sum_j p_j Bp[m][j] + sigma mu J sum_b (tr S_ab u_(b,m) + sum_n S_ab[n][m] u_(b,n))
    for(int b = 0; b < 10; ++b) {
      double P[3][3], S[3][3];
      for(int r = 0; r < 3; ++r)
        for(int l = 0; l < 3; ++l) P[r][l] = Tt.k(r, 0, a, b) * G[0][l] + Tt.k(r, 1, a, b) * G[1][l] + Tt.k(r, 2, a, b) * G[2][l];
      for(int k = 0; k < 3; ++k)
        for(int l = 0; l < 3; ++l) S[k][l] = G[0][k] * P[0][l] + G[1][k] * P[1][l] + G[2][k] * P[2][l];
      const double tr = S[0][0] + S[1][1] + S[2][2];
      const double ub[3] = {sU[(3 * b) * EPB + lane], sU[(3 * b + 1) * EPB + lane], sU[(3 * b + 2) * EPB + lane]};
      for(int m = 0; m < 3; ++m)
        be[m] += fc.sigma * fc.mu * J * (tr * ub[m] + S[0][m] * ub[0] + S[1][m] * ub[1] + S[2][m] * ub[2]);
    }
    for(int m = 0; m < 3; ++m) {
      double acc = 0.;
      for(int j = 0; j < 4; ++j) {
        const double bp = (G[0][m] * Tt.d(0, j, a) + G[1][m] * Tt.d(1, j, a) + G[2][m] * Tt.d(2, j, a)) * J;
        acc += sP[j * EPB + lane] * bp;
      }
      be[m] -= fc.sigma * acc;
    }
  }
  if(fc.hasMass) {
    // Be_(a,m) -= c int udot_m phi_a   (feVectorSysElm.cpp:409-427)
    for(int m = 0; m < 3; ++m) {
      double acc = 0.;
      for(int b = 0; b < 10; ++b) acc += Tt.m(a, b) * sUd[(3 * b + m) * EPB + lane];
      be[m] -= fc.mass * J * acc;
    }
  }
  if(fc.srcKind == SRC_SIN3_BODY) be[0] -= fc.srcCoeff * srcA * J;
  else if(fc.srcKind == SRC_CONST_VEC) {
    double ia = 0.;
    for(int q = 0; q < nq; ++q) ia += gT->phi[q][a] * gT->qw[q];
    for(int m = 0; m < 3; ++m) be[m] -= fc.srcCoeff * fc.srcParam[m] * ia * J;
  }
  for(int m = 0; m < 3; ++m) {
    const int32_t d = dm.adr[(int64_t)(3 * a + m) * nE + p];
    if(d < nInc) atomicAdd(rhs + d, be[m]);
  }
  if(fc.hasDivu && a < 4) {
    // Be_pj -= c int (div u) psi_j = c J sum_b sum_n u_(b,n) sum_r G[r][n] D[r][j][b]
    const int j = a;
    double acc = 0.;
    for(int b = 0; b < 10; ++b)
      for(int n = 0; n < 3; ++n)
        acc += sU[(3 * b + n) * EPB + lane] * (G[0][n] * Tt.d(0, j, b) + G[1][n] * Tt.d(1, j, b) + G[2][n] * Tt.d(2, j, b));
    const int32_t d = dm.adr[(int64_t)(30 + j) * nE + p];
    if(d < nInc) atomicAdd(rhs + d, -fc.divu * J * acc);
  }
}

// ---------------------------------------------------------------------------
// Residual of the Taylor-Hood forms in double-float (the mixed path): the
// FP64 kernel's integrals evaluated at the form's own quadrature nodes --
// the same nodes and weights the reference tensors are built from, so the
// same sums regrouped -- with every product and sum in float pairs on the
// FP32 pipes (the FP64 pipe of this part is ~64x slower).  Block: 32
// elements x 14 warps.  Nodes q = warp, warp + 14, ...: u, grad u, u-dot and
// p at the node, then the node's integrand coefficients (of phi_a, of the
// three reference derivatives of phi_a, of psi_j) in shared memory; then
// warp a < 10 forms the three velocity rows of P2 function a, warps 10-13
// the four pressure rows.  The source (non-polynomial) and the scatter are
// FP64, as in the FP64 kernel.  Inputs are float pairs: u, u-dot, geometry.
constexpr int DFW = 14;   // warps per block
constexpr int DFQ = 13;   // coefficients per node: f_m (3), F'_(r,m) (9), div (1)

size_t residual_df_smem(int nq)
{
  return sizeof(dfl) * (30 + 30 + 4 + 10 + (size_t)nq * DFQ) * EPB + sizeof(double) * (size_t)nq * EPB +
         sizeof(int32_t) * 34 * EPB;
}

__global__ void __launch_bounds__(EPB *DFW, 2) k_residual_tet_df(DeviceMesh dm, FormCoeffs fc,
                                                              const RefTensorsTet *__restrict__ gT,
                                                              const float2 *__restrict__ up,
                                                              const float2 *__restrict__ udp, int64_t nInc,
                                                              double *__restrict__ rhs, int64_t begin, int64_t end)
{
  extern __shared__ __align__(16) unsigned char dfsmem[];
  const int nq = gT->nq;
  dfl *sU = reinterpret_cast<dfl *>(dfsmem);  // [30][EPB]
  dfl *sUd = sU + 30 * EPB;                    // [30][EPB]
  dfl *sP = sUd + 30 * EPB;                    // [4][EPB]
  dfl *sG = sP + 4 * EPB;                      // [10][EPB]
  dfl *sQ = sG + 10 * EPB;                     // [nq][DFQ][EPB]
  double *sF = reinterpret_cast<double *>(sQ + (size_t)nq * DFQ * EPB);  // [nq][EPB]
  int32_t *sA = reinterpret_cast<int32_t *>(sF + (size_t)nq * EPB);      // [34][EPB]
  const int lane = threadIdx.x, w = threadIdx.y;
  const int64_t p = begin + (int64_t)blockIdx.x * EPB + lane;
  const bool live = p < end;
  const int64_t nE = dm.nElm;
  const bool src = fc.srcKind == SRC_SIN3_BODY;
  if(live) {
    for(int i = w; i < 34; i += DFW) {
      const int32_t d = dm.adr[(int64_t)i * nE + p];
      sA[i * EPB + lane] = d;
      const float2 v = up[d];
      if(i < 30) {
        sU[i * EPB + lane] = {v.x, v.y};
        if(fc.hasMass) {
          const float2 t = udp[d];
          sUd[i * EPB + lane] = {t.x, t.y};
        } else {
          sUd[i * EPB + lane] = df_zero();
        }
      } else {
        sP[(i - 30) * EPB + lane] = {v.x, v.y};
      }
    }
    if(w < 10) {
      const float2 g = dm.geoPair[(int64_t)w * nE + p];
      sG[w * EPB + lane] = {g.x, g.y};
    }
    if(src) {
      double X[4][3];
      for(int v = 0; v < 4; ++v)
        for(int k = 0; k < 3; ++k) X[v][k] = dm.xy[(int64_t)(3 * v + k) * nE + p];
      for(int q = w; q < nq; q += DFW) {
        const double r = gT->qr[q], s = gT->qs[q], t = gT->qt[q], l0 = 1. - r - s - t;
        double x[3];
        for(int k = 0; k < 3; ++k) x[k] = l0 * X[0][k] + r * X[1][k] + s * X[2][k] + t * X[3][k];
        sF[q * EPB + lane] = source_x(fc.srcKind, fc.srcParam, x[0], x[1], x[2]);
      }
    }
  }
  __syncthreads();
  if(live) {
    dfl G[3][3];
    for(int r = 0; r < 3; ++r)
      for(int k = 0; k < 3; ++k) G[r][k] = sG[(3 * r + k) * EPB + lane];
    const dfl J = sG[9 * EPB + lane];
    const dfl conv = {fc.pair[0][0], fc.pair[0][1]}, mass = {fc.pair[1][0], fc.pair[1][1]},
              sig = {fc.pair[2][0], fc.pair[2][1]}, mu = {fc.pair[3][0], fc.pair[3][1]},
              divu = {fc.pair[4][0], fc.pair[4][1]};
    for(int q = w; q < nq; q += DFW) {
      dfl uq[3], ur[3][3], udq[3];  // ur[r][m] = d u_m / d r_r
      for(int m = 0; m < 3; ++m) {
        uq[m] = df_zero();
        udq[m] = df_zero();
        for(int r = 0; r < 3; ++r) ur[r][m] = df_zero();
      }
      for(int b = 0; b < 10; ++b) {
        const dfl ph = {gT->phih[q][b], gT->phil[q][b]};
        const dfl dr[3] = {{gT->dphih[q][0][b], gT->dphil[q][0][b]},
                           {gT->dphih[q][1][b], gT->dphil[q][1][b]},
                           {gT->dphih[q][2][b], gT->dphil[q][2][b]}};
        for(int m = 0; m < 3; ++m) {
          const dfl v = sU[(3 * b + m) * EPB + lane];
          uq[m] = df_fma(ph, v, uq[m]);
          for(int r = 0; r < 3; ++r) ur[r][m] = df_fma(dr[r], v, ur[r][m]);
          if(fc.hasMass) udq[m] = df_fma(ph, sUd[(3 * b + m) * EPB + lane], udq[m]);
        }
      }
      dfl gu[3][3];  // gu[k][m] = d_k u_m = sum_r G[r][k] d u_m / d r_r
      for(int k = 0; k < 3; ++k)
        for(int m = 0; m < 3; ++m)
          gu[k][m] = df_add(df_add(df_mul(G[0][k], ur[0][m]), df_mul(G[1][k], ur[1][m])), df_mul(G[2][k], ur[2][m]));
      dfl pq = df_zero();
      for(int j = 0; j < 4; ++j) pq = df_fma({gT->psih[q][j], gT->psil[q][j]}, sP[j * EPB + lane], pq);
      const dfl wJ = df_mul({gT->qwh[q], gT->qwl[q]}, J);
      dfl *Q = sQ + (size_t)q * DFQ * EPB + lane;
      for(int m = 0; m < 3; ++m) {
        dfl f = df_zero();
        if(fc.hasConv)
          f = df_sub(f, df_mul(conv, df_add(df_add(df_mul(uq[0], gu[0][m]), df_mul(uq[1], gu[1][m])),
                                            df_mul(uq[2], gu[2][m]))));
        if(fc.hasMass) f = df_sub(f, df_mul(mass, udq[m]));
        Q[m * EPB] = df_mul(wJ, f);
      }
      // coefficient of d_k phi_a in component m, then of the reference
      // derivatives: F'[r][m] = sum_k G[r][k] Fg[k][m]
      dfl Fg[3][3];
      for(int k = 0; k < 3; ++k)
        for(int m = 0; m < 3; ++m) Fg[k][m] = df_zero();
      if(fc.hasSigma) {
        const dfl sw = df_neg(df_mul(sig, wJ));
        for(int k = 0; k < 3; ++k)
          for(int m = 0; m < 3; ++m)
            Fg[k][m] = df_mul(sw, df_sub(k == m ? pq : df_zero(), df_mul(mu, df_add(gu[k][m], gu[m][k]))));
      }
      for(int r = 0; r < 3; ++r)
        for(int m = 0; m < 3; ++m)
          Q[(3 + 3 * r + m) * EPB] =
              df_add(df_add(df_mul(G[r][0], Fg[0][m]), df_mul(G[r][1], Fg[1][m])), df_mul(G[r][2], Fg[2][m]));
      Q[12 * EPB] = fc.hasDivu ? df_neg(df_mul(df_mul(divu, wJ), df_add(df_add(gu[0][0], gu[1][1]), gu[2][2])))
                               : df_zero();
    }
  }
  __syncthreads();
  if(!live) return;
  if(w >= 10) {
    // pressure row j = w - 10:  Be_pj -= c int (div u) psi_j
    if(!fc.hasDivu) return;
    const int j = w - 10;
    dfl acc = df_zero();
    for(int q = 0; q < nq; ++q)
      acc = df_fma(sQ[((size_t)q * DFQ + 12) * EPB + lane], {gT->psih[q][j], gT->psil[q][j]}, acc);
    const int32_t d = sA[(30 + j) * EPB + lane];
    if(d < nInc) atomicAdd(rhs + d, df_to(acc));
    return;
  }
  const int a = w;
  dfl be[3] = {df_zero(), df_zero(), df_zero()};
  for(int q = 0; q < nq; ++q) {
    const dfl *Q = sQ + (size_t)q * DFQ * EPB + lane;
    const dfl ph = {gT->phih[q][a], gT->phil[q][a]};
    const dfl dr[3] = {{gT->dphih[q][0][a], gT->dphil[q][0][a]},
                       {gT->dphih[q][1][a], gT->dphil[q][1][a]},
                       {gT->dphih[q][2][a], gT->dphil[q][2][a]}};
    for(int m = 0; m < 3; ++m) {
      dfl t = df_mul(Q[m * EPB], ph);
      for(int r = 0; r < 3; ++r) t = df_add(t, df_mul(Q[(3 + 3 * r + m) * EPB], dr[r]));
      be[m] = df_add(be[m], t);
    }
  }
  double bd[3] = {df_to(be[0]), df_to(be[1]), df_to(be[2])};
  if(src) {
    // Be_(a,0) -= f phi_a J w over the form's rule, in FP64
    const double J = dm.geo[(int64_t)9 * nE + p];
    double srcA = 0.;
    for(int q = 0; q < nq; ++q) srcA += gT->phi[q][a] * sF[q * EPB + lane] * gT->qw[q];
    bd[0] -= fc.srcCoeff * srcA * J;
  } else if(fc.srcKind == SRC_CONST_VEC) {
    const double J = dm.geo[(int64_t)9 * nE + p];
    double ia = 0.;
    for(int q = 0; q < nq; ++q) ia += gT->phi[q][a] * gT->qw[q];
    for(int m = 0; m < 3; ++m) bd[m] -= fc.srcCoeff * fc.srcParam[m] * ia * J;
  }
  for(int m = 0; m < 3; ++m) {
    const int32_t d = sA[(3 * a + m) * EPB + lane];
    if(d < nInc) atomicAdd(rhs + d, bd[m]);
  }
}

// ---------------------------------------------------------------------------
// Jacobian, scalar P2 and Taylor-Hood, in V = double or float.
// ---------------------------------------------------------------------------
template <typename V>
__global__ void __launch_bounds__(EPB *TPB) k_matrix_tet(DeviceMesh dm, FormCoeffs fc, const RefTensorsTet *__restrict__ gT,
                                                         const double *__restrict__ u, double c0, V *__restrict__ values,
                                                         int64_t begin, int64_t end)
{
  extern __shared__ __align__(16) unsigned char smemRaw[];
  V *smem = (V *)smemRaw;
  const bool th = fc.elemType == 4;
  V *sTen = smem;
  V *sU = sTen + NTEN;       // [30][EPB]
  V *sG = sU + 30 * EPB;     // [10][EPB]
  V *sV0 = sG + 10 * EPB;    // [3][10][EPB]  V0[r][c] = sum_k G[r][k] u_(c,k)
  const int lane = threadIdx.x, a = threadIdx.y;
  const int64_t p0 = begin + (int64_t)blockIdx.x * EPB;
  const int64_t p = p0 + lane;
  const bool live = p < end;
  const int64_t nE = dm.nElm;
  const int nloc = th ? 34 : 10;
  const TetTensors<V> Tt = load_tet_tensors(sTen, gT);
  if(live) {
    sG[a * EPB + lane] = (V)dm.geo[(int64_t)a * nE + p];
    if(th && fc.hasConv)
      for(int m = 0; m < 3; ++m) sU[(3 * a + m) * EPB + lane] = (V)u[dm.adr[(int64_t)(3 * a + m) * nE + p]];
  } else {
    sG[a * EPB + lane] = 0;
    for(int m = 0; m < 3; ++m) sU[(3 * a + m) * EPB + lane] = 0;
  }
  __syncthreads();
  V G[3][3];
  for(int r = 0; r < 3; ++r)
    for(int k = 0; k < 3; ++k) G[r][k] = sG[(3 * r + k) * EPB + lane];
  const V J = sG[9 * EPB + lane];
  if(!th) {
    // A_ab += k J sum_rs (G G^T)[r][s] K[r][s][a][b]   (feSysElm.cpp:531-556)
    V GG[3][3];
    for(int r = 0; r < 3; ++r)
      for(int s = 0; s < 3; ++s) GG[r][s] = G[r][0] * G[s][0] + G[r][1] * G[s][1] + G[r][2] * G[s][2];
    const V cd = (V)fc.diff * J;
    for(int b = 0; b < 10; ++b) {
      V L = 0;
      for(int r = 0; r < 3; ++r)
        for(int s = 0; s < 3; ++s) L += GG[r][s] * Tt.k(r, s, a, b);
      const int32_t pos = live ? __ldg(dm.map + (int64_t)(a * 10 + b) * nE + p) : -1;
      if(pos >= 0) atomicAdd(values + pos, cd * L);
    }
    return;
  }
  if(fc.hasConv) {
    for(int r = 0; r < 3; ++r)
      sV0[(r * 10 + a) * EPB + lane] =
          G[r][0] * sU[(3 * a) * EPB + lane] + G[r][1] * sU[(3 * a + 1) * EPB + lane] + G[r][2] * sU[(3 * a + 2) * EPB + lane];
  }
  __syncthreads();
  // W_b = sum_c sum_r V0[r][c] T[r][a][c][b] (the u . grad phi_b term), all m
  V W[10];
  for(int b = 0; b < 10; ++b) {
    V w = 0;
    if(fc.hasConv)
      for(int c = 0; c < 10; ++c)
        for(int r = 0; r < 3; ++r) w += sV0[(r * 10 + c) * EPB + lane] * Tt.t(r, a, c, b);
    W[b] = w;
  }
  const V cc = (V)fc.conv * J, cs = -(V)fc.sigma * (V)fc.mu * J, cm = (V)fc.mass * (V)c0 * J;
  for(int m = 0; m < 3; ++m) {
    V A[30];
    for(int j = 0; j < 30; ++j) A[j] = 0;
    for(int b = 0; b < 10; ++b) {
      if(fc.hasConv) {
        // A_(a,m),(b,n) += c [delta_mn phi_a (u . grad phi_b) + phi_a phi_b d_n u_m]
        // (feVectorSysElm.cpp:1171-1240)
        V Z[3];
        for(int r = 0; r < 3; ++r) {
          V z = 0;
          for(int c = 0; c < 10; ++c) z += sU[(3 * c + m) * EPB + lane] * Tt.t(r, a, b, c);
          Z[r] = z;
        }
        for(int n = 0; n < 3; ++n) {
          V v = G[0][n] * Z[0] + G[1][n] * Z[1] + G[2][n] * Z[2];
          if(n == m) v += W[b];
          A[3 * b + n] += cc * v;
        }
      }
      if(fc.hasSigma) {
        // A_(a,m),(b,n) += -c mu [delta_mn grad phi_a . grad phi_b + d_n phi_a d_m phi_b]
        // (feVectorSysElm.cpp:1454-1492); S[k][l] = int d_k phi_a d_l phi_b / J
        V P[3][3];
        for(int r = 0; r < 3; ++r)
          for(int l = 0; l < 3; ++l) P[r][l] = Tt.k(r, 0, a, b) * G[0][l] + Tt.k(r, 1, a, b) * G[1][l] + Tt.k(r, 2, a, b) * G[2][l];
        V tr = 0;
        for(int k = 0; k < 3; ++k) tr += G[0][k] * P[0][k] + G[1][k] * P[1][k] + G[2][k] * P[2][k];
        for(int n = 0; n < 3; ++n) {
          const V snm = G[0][n] * P[0][m] + G[1][n] * P[1][m] + G[2][n] * P[2][m];
          A[3 * b + n] += cs * ((n == m ? tr : (V)0) + snm);
        }
      }
      if(fc.hasMass) A[3 * b + m] += cm * Tt.m(a, b);   // (feVectorSysElm.cpp:390-408)
    }
    if(!live) continue;
    const int row = 3 * a + m;
    for(int j = 0; j < 30; ++j) {
      const int32_t pos = __ldg(dm.map + (int64_t)(row * nloc + j) * nE + p);
      if(pos >= 0) atomicAdd(values + pos, A[j]);
    }
    // pressure columns of row (a,m) (sigma int psi_j d_m phi_a) and the
    // column (a,m) of the pressure rows (divu int psi_j d_m phi_a)
    for(int j = 0; j < 4; ++j) {
      const V bp = (G[0][m] * Tt.d(0, j, a) + G[1][m] * Tt.d(1, j, a) + G[2][m] * Tt.d(2, j, a)) * J;
      if(fc.hasSigma) {
        const int32_t pos = __ldg(dm.map + (int64_t)(row * nloc + 30 + j) * nE + p);
        if(pos >= 0) atomicAdd(values + pos, (V)fc.sigma * bp);
      }
      if(fc.hasDivu) {
        const int32_t pos = __ldg(dm.map + (int64_t)((30 + j) * nloc + row) * nE + p);
        if(pos >= 0) atomicAdd(values + pos, (V)fc.divu * bp);
      }
    }
  }
}

__global__ void k_build_map(const int32_t *__restrict__ adr, int64_t nE, int nloc, const uint8_t *__restrict__ mask,
                            const int32_t *__restrict__ ia, const int32_t *__restrict__ ja, int64_t nInc,
                            int32_t *__restrict__ map, unsigned long long *missing)
{
  const int64_t total = (int64_t)nloc * nloc * nE;
  for(int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = t % nE, ij = t / nE;
    const int i = (int)(ij / nloc), j = (int)(ij % nloc);
    int32_t pos = -1;
    if(mask[ij]) {
      const int32_t row = adr[(int64_t)i * nE + p], col = adr[(int64_t)j * nE + p];
      if(row < nInc && col < nInc) {
        int32_t lo = ia[row], hi = ia[row + 1] - 1;
        while(lo <= hi) {
          const int32_t mid = (lo + hi) >> 1, c = ja[mid];
          if(c == col) { pos = mid; break; }
          if(c < col) lo = mid + 1;
          else hi = mid - 1;
        }
        if(pos < 0) atomicAdd(missing, 1ull);
      }
    }
    map[t] = pos;
  }
}

// ---------------------------------------------------------------------------
// Row-owned FP32 Taylor-Hood Jacobian (RowAsmTet).
// ---------------------------------------------------------------------------
constexpr int RT_WARPS = 8;

// pack[p][0..29] = u at the velocity DOFs (local order 3 a + m), [30..38] =
// G, [39] = J: 32 elements per block, read per local DOF (coalesced over
// elements), written per element (coalesced) through shared memory.
__global__ void __launch_bounds__(256) k_pack_tet(DeviceMesh dm, int hasConv, const double *__restrict__ u,
                                                  float *__restrict__ pack)
{
  __shared__ float sh[32][ROWTET_PACK + 1];
  const int64_t nE = dm.nElm;
  for(int64_t p0 = (int64_t)blockIdx.x * 32; p0 < nE; p0 += (int64_t)gridDim.x * 32) {
    const int cnt = (int)(nE - p0 < 32 ? nE - p0 : 32);
    for(int idx = threadIdx.x; idx < 32 * ROWTET_PACK; idx += blockDim.x) {
      const int i = idx >> 5, l = idx & 31;
      if(l >= cnt) continue;
      const int64_t p = p0 + l;
      float v;
      if(i < 30) v = hasConv ? (float)u[dm.adr[(int64_t)i * nE + p]] : 0.f;
      else v = (float)dm.geo[(int64_t)(i - 30) * nE + p];
      sh[l][i] = v;
    }
    __syncthreads();
    for(int idx = threadIdx.x; idx < cnt * ROWTET_PACK; idx += blockDim.x)
      pack[p0 * ROWTET_PACK + idx] = sh[idx / ROWTET_PACK][idx % ROWTET_PACK];
    __syncthreads();
  }
}

__global__ void k_rowtet_offsets(int64_t nEnt, const int32_t *__restrict__ ent, const int32_t *__restrict__ entRow,
                                 const int32_t *__restrict__ map, int64_t nE, const int32_t *__restrict__ ia,
                                 uint8_t *__restrict__ offs)
{
  const int64_t total = nEnt * ROWTET_OFFS;
  for(int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t k = t / ROWTET_OFFS;
    const int j = (int)(t % ROWTET_OFFS);
    uint8_t o = 255;
    if(j < 34) {
      const int32_t e = ent[k];
      const int64_t p = e >> 6;
      const int li = e & 63;
      const int32_t pos = map[(int64_t)(li * 34 + j) * nE + p];
      if(pos >= 0) o = (uint8_t)(pos - ia[entRow[k]]);
    }
    offs[t] = o;
  }
}

// One lane's share of entry k: pack words lane and 32 + lane, offset word
// lane, and the entry's local DOF.
struct RowTetFetch {
  float pa, pb;
  uint32_t po;
  int li;
};

__device__ __forceinline__ RowTetFetch rowtet_fetch(const int32_t *__restrict__ ent, const float *__restrict__ pack,
                                                    const uint8_t *__restrict__ offs, int32_t k, int lane)
{
  RowTetFetch f{0.f, 0.f, 0u, 0};
  const int32_t e = ent[k];
  const float *pk = pack + (int64_t)(e >> 6) * ROWTET_PACK;
  f.pa = pk[lane];
  if(lane < ROWTET_PACK - 32) f.pb = pk[32 + lane];
  if(lane < ROWTET_OFFS / 4) f.po = reinterpret_cast<const uint32_t *>(offs + (int64_t)k * ROWTET_OFFS)[lane];
  f.li = e & 63;
  return f;
}

// A persistent grid walks the row blocks; per block the CSR values of its
// units live in shared memory.  Warp w takes units uA + w, uA + w + 8, ...
// and, for each of a unit's entries in order, the element's terms:
//   velocity unit, lane (m, b) = (lane / 10, lane % 10), lane < 30: the
//   columns (b, n) of row (a, m) -- k_matrix_tet's convection, stress and
//   mass terms; lanes (m, j) = (lane / 4, lane % 4), lane < 12: the pressure
//   columns sigma J sum_r G[r][m] D[r][j][a];
//   pressure unit (row of P1 function j), lane (a, m) = (lane / 3, lane % 3),
//   lane < 30: divu J sum_r G[r][m] D[r][j][a].
// Every value gets one contribution per element, in the entries' (color)
// order: the colored scatter's sum.
__global__ void __launch_bounds__(RT_WARPS * 32) k_matrix_tet_rows(RowAsmTet ra, FormCoeffs fc,
                                                                   const RefTensorsTet *__restrict__ gT, double c0,
                                                                   float *__restrict__ values, int accumulate)
{
  extern __shared__ __align__(16) unsigned char rtsm[];
  float *sTen = reinterpret_cast<float *>(rtsm);
  float *sv = sTen + NTEN;
  __shared__ float sE[RT_WARPS][ROWTET_PACK];
  __shared__ float sV0[RT_WARPS][30];
  __shared__ __align__(16) uint8_t sOff[RT_WARPS][ROWTET_OFFS];
  const TetTensors<float> Tt = load_tet_tensors(sTen, gT);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const float fconv = (float)fc.conv, fcs = -(float)fc.sigma * (float)fc.mu, fcm = (float)fc.mass * (float)c0;
  const float fsig = (float)fc.sigma, fdiv = (float)fc.divu;
  for(int blk = blockIdx.x; blk < ra.nBlocks; blk += gridDim.x) {
    const int32_t uA = ra.blockUnits[blk], uB = ra.blockUnits[blk + 1];
    const int32_t base = ra.ia[ra.unitRow[uA]], L = ra.ia[ra.unitRow[uB]] - base;
    __syncthreads();  // the previous block's values are written out (and the tensors loaded)
    for(int i = tid; i < L; i += blockDim.x) sv[i] = accumulate ? values[base + i] : 0.f;
    __syncthreads();
    for(int32_t un = uA + warp; un < uB; un += RT_WARPS) {
      const int32_t r = ra.unitRow[un];
      const bool vel = ra.unitKind[un] == 3;
      float *row0 = sv + (ra.ia[r] - base);
      const int32_t rl = ra.ia[r + 1] - ra.ia[r];
      const int32_t kb = ra.unitPtr[un], ke = ra.unitPtr[un + 1];
      // the next entry's packed element data and column offsets are loaded
      // into registers while the current one is computed
      RowTetFetch nx = kb < ke ? rowtet_fetch(ra.ent, ra.pack, ra.offs, kb, lane) : RowTetFetch{0.f, 0.f, 0u, 0};
      for(int32_t k = kb; k < ke; ++k) {
        const int li = nx.li;
        sE[warp][lane] = nx.pa;
        if(lane < ROWTET_PACK - 32) sE[warp][32 + lane] = nx.pb;
        if(lane < ROWTET_OFFS / 4) reinterpret_cast<uint32_t *>(sOff[warp])[lane] = nx.po;
        __syncwarp();
        if(k + 1 < ke) nx = rowtet_fetch(ra.ent, ra.pack, ra.offs, k + 1, lane);
        const float *E = sE[warp];
        const float J = E[39];
        float G[3][3];
#pragma unroll
        for(int q = 0; q < 3; ++q)
#pragma unroll
          for(int l = 0; l < 3; ++l) G[q][l] = E[30 + 3 * q + l];
        if(vel) {
          const int a = li / 3;
          if(fc.hasConv && lane < 30) {
            // (runtime row index: G read from shared memory, not indexed in registers)
            const int q = lane / 10, c = lane % 10;
            sV0[warp][lane] = E[30 + 3 * q] * E[3 * c] + E[31 + 3 * q] * E[3 * c + 1] + E[32 + 3 * q] * E[3 * c + 2];
          }
          __syncwarp();
          if(lane < 30) {
            const int m = lane / 10, b = lane % 10;
            // lanes b, b + 10, b + 20 hold the same column b: terms that do
            // not depend on m are split among them and exchanged by shuffles
            constexpr unsigned L30 = 0x3fffffffu;
            float A[3] = {0.f, 0.f, 0.f};
            if(fc.hasConv) {
              // W = sum_c sum_r V0[r][c] T[r][a][c][b] (lane m sums c = m, m + 3, ...),
              // Z_r = sum_c u_(c,m) T[r][a][b][c]
              float Wp = 0.f, Z[3] = {0.f, 0.f, 0.f};
#pragma unroll
              for(int cc = 0; cc < 4; ++cc) {
                const int c = m + 3 * cc;
                if(c < 10) {
#pragma unroll
                  for(int q = 0; q < 3; ++q) Wp += sV0[warp][q * 10 + c] * Tt.t(q, a, c, b);
                }
              }
#pragma unroll
              for(int c = 0; c < 10; ++c) {
                const float um = E[3 * c + m];
#pragma unroll
                for(int q = 0; q < 3; ++q) Z[q] += um * Tt.t(q, a, b, c);
              }
              const float W = __shfl_sync(L30, Wp, b) + __shfl_sync(L30, Wp, b + 10) + __shfl_sync(L30, Wp, b + 20);
              const float cc = fconv * J;
#pragma unroll
              for(int n = 0; n < 3; ++n) {
                float v = G[0][n] * Z[0] + G[1][n] * Z[1] + G[2][n] * Z[2];
                if(n == m) v += W;
                A[n] += cc * v;
              }
            }
            if(fc.hasSigma) {
              // row q = m of P formed here, rows q != m from lanes q * 10 + b
              float Pm3[3];
              {
                const float k0 = Tt.k(m, 0, a, b), k1 = Tt.k(m, 1, a, b), k2 = Tt.k(m, 2, a, b);
#pragma unroll
                for(int l = 0; l < 3; ++l) Pm3[l] = k0 * G[0][l] + k1 * G[1][l] + k2 * G[2][l];
              }
              float P[3][3];
#pragma unroll
              for(int q = 0; q < 3; ++q)
#pragma unroll
                for(int l = 0; l < 3; ++l) P[q][l] = __shfl_sync(L30, Pm3[l], q * 10 + b);
              float tr = 0.f;
#pragma unroll
              for(int kk = 0; kk < 3; ++kk) tr += G[0][kk] * P[0][kk] + G[1][kk] * P[1][kk] + G[2][kk] * P[2][kk];
              const float cs = fcs * J;
              // column m of P by selects (m is a runtime lane index)
              float Pm[3];
#pragma unroll
              for(int qq = 0; qq < 3; ++qq) Pm[qq] = m == 0 ? P[qq][0] : (m == 1 ? P[qq][1] : P[qq][2]);
#pragma unroll
              for(int n = 0; n < 3; ++n) {
                const float snm = G[0][n] * Pm[0] + G[1][n] * Pm[1] + G[2][n] * Pm[2];
                A[n] += cs * ((n == m ? tr : 0.f) + snm);
              }
            }
            if(fc.hasMass) {
              const float mv = fcm * J * Tt.m(a, b);
#pragma unroll
              for(int n = 0; n < 3; ++n)
                if(n == m) A[n] += mv;
            }
            float *row = row0 + m * rl;
#pragma unroll
            for(int n = 0; n < 3; ++n) {
              const uint8_t o = sOff[warp][3 * b + n];
              if(o != 255) row[o] += A[n];
            }
          }
          if(fc.hasSigma && lane < 12) {
            const int m = lane >> 2, j = lane & 3;
            const uint8_t o = sOff[warp][30 + j];
            if(o != 255) {
              const float bp = (E[30 + m] * Tt.d(0, j, a) + E[33 + m] * Tt.d(1, j, a) + E[36 + m] * Tt.d(2, j, a)) * J;
              row0[m * rl + o] += fsig * bp;
            }
          }
        } else if(fc.hasDivu && lane < 30) {
          const int j = li - 30, a = lane / 3, m = lane % 3;
          const uint8_t o = sOff[warp][lane];
          if(o != 255) {
            const float bp = (E[30 + m] * Tt.d(0, j, a) + E[33 + m] * Tt.d(1, j, a) + E[36 + m] * Tt.d(2, j, a)) * J;
            row0[o] += fdiv * bp;
          }
        }
        __syncwarp();
      }
    }
    __syncthreads();
    for(int i = tid; i < L; i += blockDim.x) values[base + i] = sv[i];
  }
}

size_t residual_smem(int nq) { return sizeof(double) * (NTEN + (30 + 30 + 10 + 4 + nq) * EPB); }
template <typename V>
size_t matrix_smem() { return sizeof(V) * (NTEN + (30 + 10 + 30) * EPB); }

int64_t nblk(int64_t begin, int64_t end) { return (end - begin + EPB - 1) / EPB; }

}  // namespace

void build_ref_tensors_tet(const QuadRule &q, RefTensorsTet &T)
{
  T = RefTensorsTet();
  T.nq = std::min(q.n(), TET_MAXQ);
  for(int k = 0; k < T.nq; ++k) {
    const double r = q.r[k], s = q.s[k], t = q.t[k], w = q.w[k];
    const double l[4] = {1. - r - s - t, r, s, t};
    const double dl[4][3] = {{-1, -1, -1}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    double phi[10], dphi[10][3];
    for(int v = 0; v < 4; ++v) {
      phi[v] = l[v] * (2. * l[v] - 1.);
      for(int d = 0; d < 3; ++d) dphi[v][d] = (4. * l[v] - 1.) * dl[v][d];
    }
    for(int e = 0; e < 6; ++e) {
      const int va = TET_EDGES[e][0], vb = TET_EDGES[e][1];
      phi[4 + e] = 4. * l[va] * l[vb];
      for(int d = 0; d < 3; ++d) dphi[4 + e][d] = 4. * (l[vb] * dl[va][d] + l[va] * dl[vb][d]);
    }
    T.qw[k] = w; T.qr[k] = r; T.qs[k] = s; T.qt[k] = t;
    for(int a = 0; a < 10; ++a) T.phi[k][a] = phi[a];
    auto pair = [](double x, float &h, float &lo) {
      h = (float)x;
      lo = (float)(x - (double)h);
    };
    pair(w, T.qwh[k], T.qwl[k]);
    for(int a = 0; a < 10; ++a) {
      pair(phi[a], T.phih[k][a], T.phil[k][a]);
      for(int d = 0; d < 3; ++d) pair(dphi[a][d], T.dphih[k][d][a], T.dphil[k][d][a]);
    }
    for(int j = 0; j < 4; ++j) pair(l[j], T.psih[k][j], T.psil[k][j]);
    for(int rr = 0; rr < 3; ++rr)
      for(int ss = 0; ss < 3; ++ss)
        for(int a = 0; a < 10; ++a)
          for(int b = 0; b < 10; ++b) T.K[rr][ss][a][b] += w * dphi[a][rr] * dphi[b][ss];
    for(int rr = 0; rr < 3; ++rr)
      for(int a = 0; a < 10; ++a)
        for(int c = 0; c < 10; ++c)
          for(int b = 0; b < 10; ++b) T.T[rr][a][c][b] += w * phi[a] * phi[c] * dphi[b][rr];
    for(int rr = 0; rr < 3; ++rr)
      for(int j = 0; j < 4; ++j)
        for(int a = 0; a < 10; ++a) T.D[rr][j][a] += w * l[j] * dphi[a][rr];
    for(int a = 0; a < 10; ++a)
      for(int b = 0; b < 10; ++b) T.M[a][b] += w * phi[a] * phi[b];
  }
}

void launch_assemble_residual_tet(const DeviceMesh &dm, const FormCoeffs &fc, const RefTensorsTet *dT,
                                  const double *u, const double *udot, int64_t nInc, double *rhs, int64_t begin,
                                  int64_t end, cudaStream_t s)
{
  if(end <= begin) return;
  const size_t sm = residual_smem(TET_MAXQ);
  static bool set = false;
  if(!set) {
    cudaFuncSetAttribute(k_residual_tet, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    set = true;
  }
  (k_residual_tet<<<(unsigned)nblk(begin, end), dim3(EPB, TPB), sm, s>>>(dm, fc, dT, u, udot, nInc, rhs, begin, end),
   ::feng::count_launch());
}

void launch_assemble_residual_tet_df(const DeviceMesh &dm, const FormCoeffs &fc, const RefTensorsTet *dT, int nq,
                                     const float2 *up, const float2 *udp, int64_t nInc, double *rhs, int64_t begin,
                                     int64_t end, cudaStream_t s)
{
  if(end <= begin) return;
  const size_t sm = residual_df_smem(nq);
  static bool set = false;
  if(!set) {
    cudaFuncSetAttribute(k_residual_tet_df, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)residual_df_smem(TET_DF_MAXQ));
    set = true;
  }
  (k_residual_tet_df<<<(unsigned)nblk(begin, end), dim3(EPB, DFW), sm, s>>>(dm, fc, dT, up, udp, nInc, rhs, begin,
                                                                            end),
   ::feng::count_launch());
}

template <typename V>
static void launch_matrix_tet(const DeviceMesh &dm, const FormCoeffs &fc, const RefTensorsTet *dT, const double *u,
                              double c0, V *values, int64_t begin, int64_t end, cudaStream_t s)
{
  if(end <= begin) return;
  const size_t sm = matrix_smem<V>();
  static bool set = false;
  if(!set) {
    cudaFuncSetAttribute(k_matrix_tet<V>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    set = true;
  }
  (k_matrix_tet<V><<<(unsigned)nblk(begin, end), dim3(EPB, TPB), sm, s>>>(dm, fc, dT, u, c0, values, begin, end),
   ::feng::count_launch());
}

void launch_assemble_matrix_tet_f64(const DeviceMesh &dm, const FormCoeffs &fc, const RefTensorsTet *dT,
                                    const double *u, double c0, double *values, int64_t begin, int64_t end,
                                    cudaStream_t s)
{
  launch_matrix_tet<double>(dm, fc, dT, u, c0, values, begin, end, s);
}

void launch_assemble_matrix_tet_f32(const DeviceMesh &dm, const FormCoeffs &fc, const RefTensorsTet *dT,
                                    const double *u, double c0, float *values, int64_t begin, int64_t end,
                                    cudaStream_t s)
{
  launch_matrix_tet<float>(dm, fc, dT, u, c0, values, begin, end, s);
}

void launch_pack_tet_f32(const DeviceMesh &dm, const FormCoeffs &fc, const double *u, float *pack, cudaStream_t s)
{
  const int64_t blocks = std::min<int64_t>((dm.nElm + 31) / 32, 152 * 16);
  (k_pack_tet<<<(unsigned)std::max<int64_t>(blocks, 1), 256, 0, s>>>(dm, fc.hasConv, u, pack), ::feng::count_launch());
}

void launch_rowtet_offsets(int64_t nEnt, const int32_t *ent, const int32_t *entRow, const int32_t *map,
                           int64_t nElm, const int32_t *ia, uint8_t *offs, cudaStream_t s)
{
  const int64_t blocks = std::min<int64_t>((nEnt * ROWTET_OFFS + 255) / 256, 152 * 32);
  (k_rowtet_offsets<<<(unsigned)std::max<int64_t>(blocks, 1), 256, 0, s>>>(nEnt, ent, entRow, map, nElm, ia, offs),
   ::feng::count_launch());
}

void launch_matrix_tet_rows_f32(const RowAsmTet &ra, const FormCoeffs &fc, const RefTensorsTet *dT, double c0,
                                float *values, int accumulate, cudaStream_t s)
{
  if(ra.nBlocks <= 0) return;
  const size_t sm = sizeof(float) * NTEN + (size_t)ra.capBytes;
  static size_t set = 0;
  if(set != sm) {
    cudaFuncSetAttribute(k_matrix_tet_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    set = sm;
  }
  int dev = 0, nsm = 152, perSM = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, k_matrix_tet_rows, RT_WARPS * 32, sm);
  const int grid = (int)std::min<int64_t>(ra.nBlocks, (int64_t)nsm * std::max(perSM, 1));
  (k_matrix_tet_rows<<<grid, RT_WARPS * 32, sm, s>>>(ra, fc, dT, c0, values, accumulate), ::feng::count_launch());
}

void launch_build_map(const int32_t *adr, int64_t nElm, int nloc, const uint8_t *mask, const int32_t *ia,
                      const int32_t *ja, int64_t nInc, int32_t *map, unsigned long long *missing, cudaStream_t s)
{
  const int64_t total = (int64_t)nloc * nloc * nElm;
  const int64_t blocks = std::min<int64_t>((total + 255) / 256, 152 * 32);
  (k_build_map<<<(unsigned)std::max<int64_t>(blocks, 1), 256, 0, s>>>(adr, nElm, nloc, mask, ia, ja, nInc, map, missing),
   ::feng::count_launch());
}

}  // namespace feng
