// BDF2 time stepping on device-resident history with extrapolated or learned
// Newton initial guesses (see fe_transient.h).
#include "fe_transient.h"

#include <algorithm>
#include <cmath>
#include <vector>

#include "fe_common.h"

namespace feng {

#define CKT(x)                                                                         \
  do {                                                                                 \
    cudaError_t _e = (x);                                                              \
    if(_e != cudaSuccess) {                                                            \
      set_error("CUDA error %s at %s:%d", cudaGetErrorString(_e), __FILE__, __LINE__); \
      return FE_CUDA_FAIL;                                                             \
    }                                                                                  \
  } while(0)

namespace {

constexpr int NF = MLPDims::NIN, NO = MLPDims::NOUT;

int grid_of(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 8192)); }

// ue = h1 + ratio (h1 - h2) on the unknowns; essential values copied from h1.
__global__ void k_extrapolate(int64_t nDofs, int64_t nInc, const double *__restrict__ h1,
                              const double *__restrict__ h2, double ratio, double *__restrict__ ue)
{
  for(int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nDofs; i += (int64_t)gridDim.x * blockDim.x)
    ue[i] = i < nInc ? h1[i] + ratio * (h1[i] - h2[i]) : h1[i];
}

__device__ __forceinline__ void atomic_max_pos(float *a, float v)
{
  // Non-negative floats order like their bit patterns.
  atomicMax(reinterpret_cast<int *>(a), __float_as_int(v));
}

// Scales of the last solution difference: max |h1 - h2| over velocity and
// over pressure unknowns (sig must be zeroed before).
__global__ void k_sigma(int64_t nNodes, int64_t nInc, const int32_t *__restrict__ nd, const double *__restrict__ h1,
                        const double *__restrict__ h2, float *__restrict__ sig)
{
  float su = 0.f, sp = 0.f;
  for(int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nNodes; k += (int64_t)gridDim.x * blockDim.x) {
    const int32_t u = nd[4 * k], v = nd[4 * k + 1], p = nd[4 * k + 2];
    if(u < nInc) su = nan_maxf(su, (float)fabs(h1[u] - h2[u]));
    if(v < nInc) su = nan_maxf(su, (float)fabs(h1[v] - h2[v]));
    if(p == nd[4 * k + 3] && p < nInc) sp = nan_maxf(sp, (float)fabs(h1[p] - h2[p]));
  }
  for(int o = 16; o > 0; o >>= 1) {
    su = nan_maxf(su, __shfl_xor_sync(0xffffffffu, su, o));
    sp = nan_maxf(sp, __shfl_xor_sync(0xffffffffu, sp, o));
  }
  if((threadIdx.x & 31) == 0) {
    atomic_max_pos(sig, su);
    atomic_max_pos(sig + 1, sp);
  }
}

__device__ __forceinline__ float safe_scale(float s) { return s > 0.f ? s : 1.f; }

__device__ __forceinline__ void node_q(const int32_t *nd, int64_t k, const double *h, double q[3])
{
  q[0] = h[nd[4 * k]];
  q[1] = h[nd[4 * k + 1]];
  q[2] = 0.5 * (h[nd[4 * k + 2]] + h[nd[4 * k + 3]]);
}

// Per-node inputs: u^n (3), (u^n - u^{n-1}) / s (3), (u^{n-1} - u^{n-2}) / s (3),
// 6 geometry features, one zero pad.  s = velocity or pressure scale.
__global__ void k_features(int64_t nNodes, const int32_t *__restrict__ nd, const float *__restrict__ geo,
                           const double *__restrict__ h1, const double *__restrict__ h2,
                           const double *__restrict__ h3, const float *__restrict__ sig, float *__restrict__ X)
{
  const float iu = 1.f / safe_scale(sig[0]), ip = 1.f / safe_scale(sig[1]);
  for(int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nNodes; k += (int64_t)gridDim.x * blockDim.x) {
    double a[3], b[3], c[3];
    node_q(nd, k, h1, a);
    node_q(nd, k, h2, b);
    node_q(nd, k, h3, c);
    float *x = X + k * NF;
    for(int q = 0; q < 3; ++q) {
      const float is = q < 2 ? iu : ip;
      x[q] = (float)a[q];
      x[3 + q] = (float)(a[q] - b[q]) * is;
      x[6 + q] = (float)(b[q] - c[q]) * is;
    }
    for(int g = 0; g < 6; ++g) x[9 + g] = geo[6 * k + g];
    x[15] = 0.f;
  }
}

// um = ue + scale * s * y on the node's unknowns (pressure at vertex nodes only).
__global__ void k_apply(int64_t nNodes, int64_t nInc, const int32_t *__restrict__ nd, const float *__restrict__ Y,
                        const float *__restrict__ sig, float scale, const double *__restrict__ ue,
                        double *__restrict__ um)
{
  const float su = scale * safe_scale(sig[0]), sp = scale * safe_scale(sig[1]);
  for(int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nNodes; k += (int64_t)gridDim.x * blockDim.x) {
    const int32_t u = nd[4 * k], v = nd[4 * k + 1], p = nd[4 * k + 2];
    if(u < nInc) um[u] = ue[u] + (double)(su * Y[k * NO]);
    if(v < nInc) um[v] = ue[v] + (double)(su * Y[k * NO + 1]);
    if(p == nd[4 * k + 3] && p < nInc) um[p] = ue[p] + (double)(sp * Y[k * NO + 2]);
  }
}

// d = um - ue on the unknowns.
__global__ void k_diff(int64_t n, const double *__restrict__ a, const double *__restrict__ b, double *__restrict__ d)
{
  for(int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    d[i] = a[i] - b[i];
}

// um = ue + alpha d on the unknowns (the essential entries of um are ue's).
__global__ void k_add_scaled(int64_t n, const double *__restrict__ ue, double alpha, const double *__restrict__ d,
                             double *__restrict__ um)
{
  for(int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    um[i] = ue[i] + alpha * d[i];
}

// Training targets (u^{n+1} - ue) / s with their mask.
__global__ void k_targets(int64_t nNodes, int64_t nInc, const int32_t *__restrict__ nd, const double *__restrict__ u,
                          const double *__restrict__ ue, const float *__restrict__ sig, float *__restrict__ T,
                          float *__restrict__ M)
{
  const float iu = 1.f / safe_scale(sig[0]), ip = 1.f / safe_scale(sig[1]);
  for(int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nNodes; k += (int64_t)gridDim.x * blockDim.x) {
    const int32_t dof[3] = {nd[4 * k], nd[4 * k + 1], nd[4 * k + 2]};
    const bool vertex = nd[4 * k + 2] == nd[4 * k + 3];
    for(int q = 0; q < 3; ++q) {
      const bool ok = dof[q] < nInc && (q < 2 || vertex);
      T[k * NO + q] = ok ? (float)(u[dof[q]] - ue[dof[q]]) * (q < 2 ? iu : ip) : 0.f;
      M[k * NO + q] = ok ? 1.f : 0.f;
    }
    T[k * NO + 3] = 0.f;
    M[k * NO + 3] = 0.f;
  }
}

// Variable-step BDF coefficients (computeBDFCoefficients,
// src/feSolutionContainer.cpp:82-101).
void bdf_coefficients(int order, double d0, double d1, double cn[3])
{
  cn[0] = cn[1] = cn[2] = 0.;
  if(order == 1) {
    cn[0] = 1.0 / d0;
    cn[1] = -1.0 / d0;
  } else if(order == 2) {
    cn[0] = 1.0 / d0 + 1.0 / (d0 + d1);
    cn[1] = -1.0 / d0 - 1.0 / d1;
    cn[2] = d0 / d1 * 1.0 / (d0 + d1);
  }
}

}  // namespace

Transient::~Transient()
{
  cudaFree(nodeDof_);
  cudaFree(geo_);
  cudaFree(h3_);
  cudaFree(ue_);
  cudaFree(um_);
  cudaFree(dv_);
  cudaFree(jd_);
  cudaFree(X_);
  cudaFree(Y_);
  cudaFree(T_);
  cudaFree(M_);
  cudaFree(sig_);
  cudaFree(loss_);
  cudaFree(idx_);
  if(e0_) cudaEventDestroy(e0_);
  if(e1_) cudaEventDestroy(e1_);
  if(e2_) cudaEventDestroy(e2_);
  if(e3_) cudaEventDestroy(e3_);
}

int Transient::init(SystemCUDA *sys, const TransientOptions &o, const NewtonOptions &n)
{
  if(!sys || !(o.dt > 0) || o.guess < GUESS_PREVIOUS || o.guess > GUESS_LEARNED || o.trainIters < 0 ||
     o.batch < 1 || !(o.lr >= 0)) {
    set_error("invalid transient options");
    return FE_INVALID_ARG;
  }
  sys_ = sys;
  o_ = o;
  no_ = n;
  no_.stationary = 0;
  cudaStream_t s = sys->stream();
  const int64_t nDofs = sys->nDofs(), nInc = sys->nInc();
  CKT(cudaMalloc(&h3_, sizeof(double) * nDofs));
  CKT(cudaMalloc(&ue_, sizeof(double) * nDofs));
  CKT(cudaMalloc(&um_, sizeof(double) * nDofs));
  CKT(cudaMalloc(&dv_, sizeof(double) * std::max<int64_t>(1, sys->nInc())));
  CKT(cudaMalloc(&jd_, sizeof(double) * std::max<int64_t>(1, sys->nInc())));
  CKT(cudaEventCreate(&e0_));
  CKT(cudaEventCreate(&e1_));
  CKT(cudaEventCreate(&e2_));
  CKT(cudaEventCreate(&e3_));
  const double cn[3] = {1.0 / o.dt, -1.0 / o.dt, 0.0};
  FE_TRY(sys->setBDFCoefficients(2, cn));  // allocates the device history
  // Preconditioner for the time-dependent saddle point: the BDF2 coefficient
  // of u^{n+1} at constant steps, 1.5 / dt (the two starter solves differ).
  FE_TRY(sys->setTransientShift(1.5 / o.dt));
  CKT(cudaMemsetAsync(sys->dHist(1), 0, sizeof(double) * nDofs, s));
  CKT(cudaMemsetAsync(sys->dHist(2), 0, sizeof(double) * nDofs, s));
  CKT(cudaMemsetAsync(h3_, 0, sizeof(double) * nDofs, s));

  if(o.guess == GUESS_LEARNED) {
    if(sys->elemType() != ELEM_TAYLOR_HOOD) {
      set_error("the learned guess needs a Taylor-Hood system");
      return FE_INVALID_ARG;
    }
    // P2 nodes (vertices, then edge midpoints as met) with their DOFs and geometry.
    const auto &adr = sys->elementTable();
    const auto &xy = sys->elementXY();
    const int nl = sys->nloc();
    const int64_t nE = sys->nElm();
    std::vector<int32_t> nodeOf(nDofs, -1), nd;
    std::vector<double> px, py, hsum, hcnt;
    std::vector<int8_t> isVertex;
    double xmin = 1e300, xmax = -1e300, ymin = 1e300, ymax = -1e300;
    for(int64_t e = 0; e < nE; ++e) {
      const double *c = &xy[6 * e];
      const double area = 0.5 * std::fabs((c[2] - c[0]) * (c[5] - c[1]) - (c[4] - c[0]) * (c[3] - c[1]));
      const double h = std::sqrt(2.0 * area);
      for(int a = 0; a < 6; ++a) {
        const int64_t du = adr[e * nl + 2 * a];
        int32_t k = nodeOf[du];
        if(k < 0) {
          k = nodeOf[du] = (int32_t)px.size();
          int64_t p0, p1;
          double x, y;
          if(a < 3) {
            p0 = p1 = adr[e * nl + 12 + a];
            x = c[2 * a];
            y = c[2 * a + 1];
          } else {
            const int v0 = a - 3, v1 = (a - 2) % 3;  // local edge a-3 joins vertices (a-3, a-2 mod 3)
            p0 = adr[e * nl + 12 + v0];
            p1 = adr[e * nl + 12 + v1];
            x = 0.5 * (c[2 * v0] + c[2 * v1]);
            y = 0.5 * (c[2 * v0 + 1] + c[2 * v1 + 1]);
          }
          nd.push_back((int32_t)du);
          nd.push_back((int32_t)adr[e * nl + 2 * a + 1]);
          nd.push_back((int32_t)p0);
          nd.push_back((int32_t)p1);
          px.push_back(x);
          py.push_back(y);
          hsum.push_back(0.);
          hcnt.push_back(0.);
          isVertex.push_back(a < 3);
          xmin = std::min(xmin, x);
          xmax = std::max(xmax, x);
          ymin = std::min(ymin, y);
          ymax = std::max(ymax, y);
        }
        hsum[k] += h;
        hcnt[k] += 1;
      }
    }
    nNodes_ = (int64_t)px.size();
    double hmean = 0.;
    for(int64_t k = 0; k < nNodes_; ++k) hmean += hsum[k] / hcnt[k];
    hmean /= std::max<int64_t>(1, nNodes_);
    const double L = std::max(xmax - xmin, ymax - ymin);
    std::vector<float> geo(6 * nNodes_);
    for(int64_t k = 0; k < nNodes_; ++k) {
      const double x = px[k], y = py[k];
      const double dw = std::min(std::min(x - xmin, xmax - x), std::min(y - ymin, ymax - y));
      geo[6 * k + 0] = (float)((x - xmin) / L);
      geo[6 * k + 1] = (float)((y - ymin) / L);
      geo[6 * k + 2] = (float)(dw / L);
      geo[6 * k + 3] = (float)(hsum[k] / hcnt[k] / hmean);
      geo[6 * k + 4] = isVertex[k] ? 1.f : 0.f;
      geo[6 * k + 5] = nd[4 * k] >= nInc ? 1.f : 0.f;
    }
    CKT(cudaMalloc(&nodeDof_, sizeof(int32_t) * 4 * nNodes_));
    CKT(cudaMalloc(&geo_, sizeof(float) * 6 * nNodes_));
    CKT(cudaMalloc(&X_, sizeof(float) * NF * nNodes_));
    CKT(cudaMalloc(&Y_, sizeof(float) * NO * nNodes_));
    CKT(cudaMalloc(&T_, sizeof(float) * NO * nNodes_));
    CKT(cudaMalloc(&M_, sizeof(float) * NO * nNodes_));
    CKT(cudaMalloc(&sig_, sizeof(float) * 2));
    CKT(cudaMalloc(&loss_, sizeof(float)));
    CKT(cudaMalloc(&idx_, sizeof(int32_t) * o.batch));
    CKT(cudaMemcpyAsync(nodeDof_, nd.data(), sizeof(int32_t) * nd.size(), cudaMemcpyHostToDevice, s));
    CKT(cudaMemcpyAsync(geo_, geo.data(), sizeof(float) * geo.size(), cudaMemcpyHostToDevice, s));
    FE_TRY(mlp_.init(o.seed, o.batch, s));
  }
  CKT(cudaStreamSynchronize(s));
  tHist_[0] = tHist_[1] = tHist_[2] = o.t0;
  nHist_ = 0;
  steps_ = 0;
  trained_ = 0;
  lostStreak_ = 0;
  skipUntil_ = 0;
  return FE_OK;
}

int Transient::residualNorm(double *norm)
{
  FE_TRY(sys_->computeSolDot());
  FE_TRY(sys_->setResidualToZero());
  FE_TRY(sys_->assembleResiduals());
  return sys_->getRHSMaxNorm(norm);
}

int Transient::newton(double scale, NewtonStats &ns, bool residualReady)
{
  NewtonOptions n = no_;
  n.residualScale = scale;
  n.residualReady = residualReady ? 1 : 0;
  // A step whose Newton solve did not converge is reported to the caller
  // (the reference exits there, src/feNonLinearSolver.cpp:174-180).
  return newton_solve(*sys_, n, ns);
}

// Rotation of the history and the step's time-level set-up (rotate,
// src/feSolutionContainer.cpp:291-304): u^{n-2} <- u^{n-1} <- u^n <- u.
static int rotate(SystemCUDA *sys, double *h3, double tHist[3], int &nHist, double tCur)
{
  cudaStream_t s = sys->stream();
  const size_t bytes = sizeof(double) * sys->nDofs();
  CKT(cudaMemcpyAsync(h3, sys->dHist(2), bytes, cudaMemcpyDeviceToDevice, s));
  CKT(cudaMemcpyAsync(sys->dHist(2), sys->dHist(1), bytes, cudaMemcpyDeviceToDevice, s));
  CKT(cudaMemcpyAsync(sys->dHist(1), sys->dU(), bytes, cudaMemcpyDeviceToDevice, s));
  tHist[2] = tHist[1];
  tHist[1] = tHist[0];
  tHist[0] = tCur;
  nHist = std::min(3, nHist + 1);
  return FE_OK;
}

// First step, as BDF2Integrator::startWithBDF1 (src/feTimeIntegration.cpp:383-435):
// a BDF1 step of 0.1 dt, then variable-step BDF2 to t0 + dt, each Newton
// solve starting from the previous solution.
int Transient::bdf1Start(StepStats &st)
{
  const double dt1 = 0.1 * o_.dt, dt2 = o_.dt - dt1;
  double cn[3];
  NewtonStats ns;
  FE_TRY(rotate(sys_, h3_, tHist_, nHist_, o_.t0));
  bdf_coefficients(1, dt1, 0., cn);
  FE_TRY(sys_->setBDFCoefficients(1, cn));
  sys_->setTime(o_.t0 + dt1, cn[0]);
  double rref = 0.;
  FE_TRY(residualNorm(&rref));
  FE_TRY(newton(rref, ns));
  st.newtonIterations += ns.iterations;
  st.krylovIterations += ns.krylovIterations;
  FE_TRY(rotate(sys_, h3_, tHist_, nHist_, o_.t0 + dt1));
  bdf_coefficients(2, dt2, dt1, cn);
  FE_TRY(sys_->setBDFCoefficients(2, cn));
  sys_->setTime(o_.t0 + o_.dt, cn[0]);
  FE_TRY(residualNorm(&rref));
  FE_TRY(newton(rref, ns));
  st.newtonIterations += ns.iterations;
  st.krylovIterations += ns.krylovIterations;
  st.residualRef = rref;
  st.residualGuess = ns.residual0;
  st.residual = ns.residual;
  st.status = ns.status;
  st.guessUsed = GUESS_PREVIOUS;
  st.t = o_.t0 + o_.dt;
  return FE_OK;
}

int Transient::step(StepStats &st)
{
  st = StepStats();
  st.step = steps_ + 1;
  cudaStream_t s = sys_->stream();
  CKT(cudaEventRecord(e0_, s));
  CKT(cudaEventRecord(e1_, s));
  if(steps_ == 0) {
    FE_TRY(bdf1Start(st));
  } else {
    // Time of the current solution u: the last step's end.
    const double tu = o_.t0 + steps_ * o_.dt;
    FE_TRY(rotate(sys_, h3_, tHist_, nHist_, tu));
    const double tnew = tu + o_.dt;
    const double d0 = tnew - tHist_[0], d1 = tHist_[0] - tHist_[1];
    const int order = nHist_ >= 2 ? 2 : 1;
    double cn[3];
    bdf_coefficients(order, d0, d1, cn);
    FE_TRY(sys_->setBDFCoefficients(order, cn));
    sys_->setTime(tnew, cn[0]);
    st.t = tnew;
    // Reference residual: the previous solution at the new time level.
    double rref = 0.;
    FE_TRY(residualNorm(&rref));
    st.residualRef = rref;
    const int64_t nDofs = sys_->nDofs(), nInc = sys_->nInc();
    const size_t bytes = sizeof(double) * nDofs;
    const bool canExtrap = o_.guess != GUESS_PREVIOUS && nHist_ >= 2;
    // Back-off: after LOSE_LIMIT consecutive steps where the learned
    // candidate did not beat the extrapolation, the network is neither
    // evaluated nor trained for BACKOFF_STEPS steps, then tried again.
    constexpr int LOSE_LIMIT = 8, BACKOFF_STEPS = 32;
    const bool backoff = st.step < skipUntil_;
    const bool learn = o_.guess == GUESS_LEARNED && nHist_ >= 3 && !backoff;
    int used = GUESS_PREVIOUS;
    if(canExtrap) {
      (k_extrapolate<<<grid_of(nDofs), 256, 0, s>>>(nDofs, nInc, sys_->dHist(1), sys_->dHist(2), d0 / d1, ue_),
       ::feng::count_launch());
      CKT(cudaGetLastError());
      used = GUESS_EXTRAPOLATE;
    }
    if(learn) {
      CKT(cudaMemsetAsync(sig_, 0, sizeof(float) * 2, s));
      (k_sigma<<<grid_of(nNodes_), 256, 0, s>>>(nNodes_, nInc, nodeDof_, sys_->dHist(1), sys_->dHist(2), sig_),
       ::feng::count_launch());
      (k_features<<<grid_of(nNodes_), 256, 0, s>>>(nNodes_, nodeDof_, geo_, sys_->dHist(1), sys_->dHist(2), h3_, sig_,
                                                   X_),
       ::feng::count_launch());
      CKT(cudaGetLastError());
    }
    bool residualReady = false;
    if(learn && trained_ > 0 && st.step >= o_.useFrom) {
      // One learned candidate ue + alpha d (d: the network's correction),
      // judged against the extrapolation by the FP64 residual; the
      // extrapolation is kept when the candidate does not beat it.  alpha
      // minimises the linearised residual ||R(ue) - alpha J d||_2 with the
      // Jacobian still held from the previous step: alpha = <R, J d> /
      // <J d, J d>, kept in [0, 2] (1 without a Jacobian).  The candidate's
      // residual is evaluated last, so when it wins that residual is
      // Newton's first one.  A non-finite candidate residual never wins
      // (the comparison is false for NaN).
      FE_TRY(mlp_.forward(X_, nNodes_, Y_));
      double re = 0., rm = 0.;
      CKT(cudaMemcpyAsync(sys_->dU(), ue_, bytes, cudaMemcpyDeviceToDevice, s));
      FE_TRY(residualNorm(&re));
      st.residualExtrap = re;
      CKT(cudaMemcpyAsync(um_, ue_, bytes, cudaMemcpyDeviceToDevice, s));
      (k_apply<<<grid_of(nNodes_), 256, 0, s>>>(nNodes_, nInc, nodeDof_, Y_, sig_, 1.f, ue_, um_),
       ::feng::count_launch());
      CKT(cudaGetLastError());
      double alpha = 1.;
      (k_diff<<<grid_of(nInc), 256, 0, s>>>(nInc, um_, ue_, dv_), ::feng::count_launch());
      if(sys_->jacobianTimes(dv_, jd_) == FE_OK) {
        const double jj = sys_->krylov().dot(jd_, jd_), rj = sys_->krylov().dot(sys_->dRhs(), jd_);
        if(jj > 0 && std::isfinite(jj) && std::isfinite(rj)) alpha = std::min(2., std::max(0., rj / jj));
        (k_add_scaled<<<grid_of(nInc), 256, 0, s>>>(nInc, ue_, alpha, dv_, um_), ::feng::count_launch());
        CKT(cudaGetLastError());
      }
      st.guessScale = alpha;
      CKT(cudaMemcpyAsync(sys_->dU(), um_, bytes, cudaMemcpyDeviceToDevice, s));
      const int r = residualNorm(&rm);
      if(r != FE_OK && r != FE_NONFINITE) return r;
      if(r == FE_OK && rm < re) {
        used = GUESS_LEARNED;
        residualReady = true;
        lostStreak_ = 0;
      } else {
        CKT(cudaMemcpyAsync(sys_->dU(), ue_, bytes, cudaMemcpyDeviceToDevice, s));
        if(++lostStreak_ >= LOSE_LIMIT) {
          skipUntil_ = st.step + 1 + BACKOFF_STEPS;
          lostStreak_ = 0;
        }
      }
    } else if(canExtrap) {
      CKT(cudaMemcpyAsync(sys_->dU(), ue_, bytes, cudaMemcpyDeviceToDevice, s));
    }
    st.guessUsed = used;
    CKT(cudaEventRecord(e1_, s));
    NewtonStats ns;
    const int ns_status = newton(rref, ns, residualReady);
    if(ns_status != FE_OK && ns_status != FE_NOT_CONVERGED) return ns_status;
    st.newtonIterations = ns.iterations;
    st.krylovIterations = ns.krylovIterations;
    st.residualGuess = ns.residual0;
    if(used == GUESS_EXTRAPOLATE && st.residualExtrap == 0.) st.residualExtrap = ns.residual0;
    st.residual = ns.residual;
    st.status = ns.status;
    // Online training on the correction this step revealed (a step that
    // did not converge reveals none).
    if(learn && ns_status == FE_OK && st.step >= o_.trainFrom && o_.trainIters > 0) {
      CKT(cudaEventRecord(e2_, s));
      (k_targets<<<grid_of(nNodes_), 256, 0, s>>>(nNodes_, nInc, nodeDof_, sys_->dU(), ue_, sig_, T_, M_),
       ::feng::count_launch());
      CKT(cudaGetLastError());
      const int64_t nb = std::min<int64_t>(o_.batch, nNodes_);
      for(int it = 0; it < o_.trainIters; ++it) {
        FE_TRY(mlp_.sample(nNodes_, nb, idx_));
        FE_TRY(mlp_.gradient(X_, T_, M_, idx_, nb));
        FE_TRY(mlp_.adam((float)o_.lr, 0.9f, 0.999f, 1e-8f, nullptr, it + 1 == o_.trainIters ? loss_ : nullptr));
      }
      float l = 0.f;
      CKT(cudaMemcpyAsync(&l, loss_, sizeof(float), cudaMemcpyDeviceToHost, s));
      CKT(cudaEventRecord(e3_, s));
      CKT(cudaStreamSynchronize(s));
      float tm = 0.f;
      CKT(cudaEventElapsedTime(&tm, e2_, e3_));
      st.trainMs = tm;
      st.trainLoss = l;
      ++trained_;
    }
  }
  CKT(cudaEventRecord(e3_, s));
  CKT(cudaStreamSynchronize(s));
  float ms = 0.f, gm = 0.f;
  CKT(cudaEventElapsedTime(&ms, e0_, e3_));
  CKT(cudaEventElapsedTime(&gm, e0_, e1_));
  st.stepMs = ms;
  st.guessMs = gm;
  ++steps_;
  // A step whose Newton solve did not converge is reported (the reference
  // exits there, src/feNonLinearSolver.cpp:174-180); its statistics are kept.
  return st.status;
}

}  // namespace feng
