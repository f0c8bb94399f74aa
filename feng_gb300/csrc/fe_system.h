// The CUDA linear-system backend: device-resident matrix, right-hand side,
// solution and the operations of feNG's feLinearSystem interface
// (src/feLinearSystem.h:43-169), plus the Newton driver that calls them
// (solveNewtonRaphson, src/feNonLinearSolver.cpp:38-181) and the BDF time
// derivative (BDFContainer, src/feSolutionContainer.cpp:82-101, 338-349).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <memory>
#include <vector>

#include "fe_amg.h"
#include "fe_device.h"
#include "fe_krylov.h"
#include "fe_setup.h"

namespace feng {

struct FormDesc {
  int kind;          // FormKind
  double coeff;      // constant coefficient
  double coeff2;     // second coefficient (viscosity of DIV_NEWTONIAN_STRESS)
  int source;        // SourceKind for SOURCE / VECTOR_SOURCE
  double params[4];  // source parameters
};

struct SystemOptions {
  KrylovOptions kry;
  int pcBlockRows = 256;   // target rows per block-Jacobi block (0: a single block)
  int precision = 0;       // 0 FP64 matrix, 1 FP32 matrix + mixed Krylov
  int mgInner = 0;         // multigrid: inner CG steps per component (0: one V-cycle)
  int mgSmooth = 1;        // multigrid: Chebyshev degree
};

// Everything the backend needs from the set-up, in the original element order.
struct SystemTables {
  int elemType = 0;
  int64_t nElm = 0;
  int nloc = 0;
  int64_t nInc = 0, nDofs = 0;
  const int64_t *adr = nullptr;       // [nElm*nloc]
  const double *elemXY = nullptr;     // [nElm*6] x0 y0 x1 y1 x2 y2 (tetrahedra: [nElm*12] x0 y0 z0 ... z3)
  // optional (computed when null/empty):
  const Coloring *coloring = nullptr;
  const CSRPattern *pattern = nullptr;
  const std::vector<int32_t> *blockOfRow = nullptr;  // block-Jacobi partition of unknowns
  QuadRule quad;
};

struct PhaseTimes {
  double residual_ms = 0, matrix_ms = 0, factor_ms = 0, solve_ms = 0, other_ms = 0;
  int residual_calls = 0, matrix_calls = 0, solve_calls = 0;
};

class SystemCUDA {
 public:
  ~SystemCUDA();
  int init(const SystemTables &t, const FormDesc *forms, int nforms, const SystemOptions &opt);

  // feLinearSystem operations
  int setToZero();
  int setMatrixToZero();
  int setResidualToZero();
  int assembleResiduals();
  int assembleMatrices();
  int getRHSMaxNorm(double *norm);
  // Partially essential vector components and periodic DOFs
  // (feLinearSystemMklPardiso.cpp:994-1149): rows/columns set once, applied
  // after each assembly (idempotent on an already constrained matrix).
  int setConstrainedRows(const int64_t *rows, int64_t n);
  int constrainEssentialComponents();
  int setPeriodicPairs(const int64_t *master, const int64_t *slave, int64_t n);
  int applyPeriodicity();
  // Builds the preconditioner of the current matrix if it changed.
  int factorIfPending();
  // BDF time stepping with c0 = dudt coefficient of the current step: adapts
  // the multigrid saddle-point preconditioner (Krylov::setTransientShift)
  // with c0 times the mass coefficient and the form's viscosity.
  int setTransientShift(double c0);
  int solve(double *normDx, double *normRHS, double *normAxb, int *nIter);
  int correctSolution();

  // Solution state (device), time and BDF coefficient c0.
  int setSolution(const double *hostU, const double *hostUdot);
  int getSolution(double *hostU) const;
  int getSolutionDot(double *hostUdot) const;
  void setTime(double t, double c0)
  {
    t_ = t;
    c0_ = c0;
  }
  // BDF history: hist[k] = u^{n+1-k}; udot = sum_k cn[k] hist[k] with hist[0] = u.
  int setBDF(int order, const double *cn, const double *const *hostHist);
  // Coefficients only (device history kept; buffers allocated on first use).
  int setBDFCoefficients(int order, const double *cn);
  int computeSolDot();
  // Device history u^{n+1-k} (k = 1, 2), owned by the system.
  double *dHist(int k) { return k >= 1 && k <= 2 ? hist_[k] : nullptr; }
  double time() const { return t_; }

  int64_t nInc() const { return nInc_; }
  int64_t nDofs() const { return nDofs_; }
  int64_t nnz() const { return pat_.nnz(); }
  int64_t nElm() const { return dm_.nElm; }
  int nColors() const { return dm_.nColors; }
  const CSRPattern &pattern() const { return pat_; }
  const Coloring &coloring() const { return col_; }
  int getMatrix(double *hostValues) const;  // FP64 copy of the current values
  int getRHS(double *hostRhs) const;
  int getDu(double *hostDu) const;
  int applyPreconditioner(const double *hostR, double *hostZ);
  // y = J x with the Jacobian last assembled (device vectors of nInc
  // entries); FE_INVALID_ARG when no assembled Jacobian is held.
  int jacobianTimes(const double *x, double *y);
  int validateColoring() const;
  // Error norms of feNorm (src/feNorm.cpp:323-391, 1399-1443) on the
  // system's quadrature rule: normPoints gives the rule's nodes on every
  // element (system element order, nq per element) where the caller
  // evaluates its exact solution; l2Error returns sqrt(sum_e sum_k
  // sum_c |u_ex - u_h|^2 |J| w_k) for field 0 (the P2 field, 1 or 2
  // components) or field 1 (the P1 pressure of Taylor-Hood), exact values
  // host-side [nElm][nq][ncomp].
  int normPoints(int *nq, double *hostX, double *hostY);
  int l2Error(int field, const double *hostExact, double *err);
  // Times `reps` runs of one phase with CUDA events on the system stream, each
  // preceded by an L2 flush (a write of flushBytes, then a read of it, so
  // that no dirty lines remain to be written back): which = 0 residual
  // assembly, 1 matrix assembly, 2 SpMV with the system matrix, 3 one
  // preconditioner application, 4 one finest-level multigrid smoother step
  // (two components).  Returns the mean milliseconds per run.
  int benchPhase(int which, int reps, size_t flushBytes, double *avgMs);
  // 1 when the Jacobian is assembled row-owned (no scatter), 0 colored.
  int jacobianRoute() const { return useRows_ || useRowsTet_ ? 1 : 0; }

  // Host copies of the set-up tables (original element order).
  const std::vector<int64_t> &elementTable() const { return adrHost_; }
  const std::vector<double> &elementXY() const { return elemXYHost_; }
  int elemType() const { return elemType_; }
  int nloc() const { return nloc_; }

  double *dU() { return u_; }
  double *dUdot() { return udot_; }
  double *dRhs() { return rhs_; }
  double *dDu() { return du_; }
  cudaStream_t stream() const { return s_; }
  Krylov &krylov() { return kry_; }
  PhaseTimes times;
  KrylovStats lastSolve;
  SystemOptions opt;
  int timing = 1;  // record CUDA events around the phases

 private:
  int64_t nInc_ = 0, nDofs_ = 0;
  int nloc_ = 0;
  double t_ = 0, c0_ = 0;
  Coloring col_;
  CSRPattern pat_;
  std::vector<int64_t> adrHost_;      // element table, original element order
  std::vector<double> elemXYHost_;    // vertex coordinates per element
  int elemType_ = 0;
  int exact5_ = 0;   // the rule integrates degree 5 exactly (quadrature residual kernel)
  DeviceMesh dm_;
  FormCoeffs fc_{};
  RefTensors *dT_ = nullptr;
  int nq_ = 0;  // nodes of the system's quadrature rule
  // Row-owned Taylor-Hood FP32 Jacobian (used when every row is shorter
  // than 255).
  RowAsm ra_;
  bool useRows_ = false;
  // Row-owned FP32 Jacobian of tetrahedral Taylor-Hood systems.
  RowAsmTet rat_;
  bool useRowsTet_ = false;
  int build_row_assembly_tet(const std::vector<int32_t> &adrP, const std::vector<uint8_t> &mask);
  // setMatrixToZero is deferred: the next row-owned assembly overwrites the
  // values instead of adding to them; any other use of the values zeroes
  // them first.
  mutable bool zeroPending_ = false;
  int ensureMatrixZeroed() const;
  // The mixed path assembles the Taylor-Hood residual in double-float on
  // the FP32 pipes (FP64-class accuracy, the 7-node rule); otherwise FP64.
  // the mixed path's residual in double-float (triangles: rules exact to
  // degree 5; tetrahedra: Taylor-Hood with rules of at most TET_DF_MAXQ nodes)
  int dfResidual() const { return dm_.geoPair && (exact5_ || tet()) ? 1 : 0; }
  void launch_residual(double *out);  // the residual launches of assembleResiduals
  float2 *uPair_ = nullptr, *udotPair_ = nullptr;
  int launch_matrix();  // the Jacobian launches of assembleMatrices
  int build_row_assembly(const std::vector<int32_t> &adrP, const std::vector<int32_t> &map);
  DeviceCSR csr_;
  double *vals64_ = nullptr;
  float *vals32_ = nullptr;
  double *rhs_ = nullptr, *du_ = nullptr, *u_ = nullptr, *udot_ = nullptr;
  double *hist_[3] = {nullptr, nullptr, nullptr};
  double cn_[3] = {0, 0, 0};
  int bdfOrder_ = 0;
  double *scratch_ = nullptr;
  Krylov kry_;
  cudaStream_t s_ = nullptr;
  cudaEvent_t ev0_ = nullptr, ev1_ = nullptr;
  bool hostTmp_ = false;
  bool matrixValid_ = false;
  bool factorPending_ = false;
  bool constrained_ = false, periodic_ = false;
  int64_t *conRows_ = nullptr, *conColPos_ = nullptr, *perMaster_ = nullptr, *perSlave_ = nullptr;
  int64_t nCon_ = 0, nConPos_ = 0, nPer_ = 0;
  HostCSR massV_, lapP_;   // preconditioner operators kept for transient re-set-ups
  int32_t nPLap_ = 0;
  int begin_phase();
  float end_phase();
  int build_precond_info(const SystemTables &t, const RefTensors &T, HostCSR &lap, PrecondInfo &pi);
  int build_precond_info_tet(const SystemTables &t, const RefTensorsTet &T, HostCSR &lap, PrecondInfo &pi);
  int build_precond_info_tet_th(const SystemTables &t, const RefTensorsTet &T, HostCSR &lap, PrecondInfo &pi);
  RefTensorsTet *dTt_ = nullptr;  // tetrahedral reference tensors (device)
  bool tet() const { return elemType_ == ELEM_TET_P2 || elemType_ == ELEM_TET_TAYLOR_HOOD; }
};

// Reference-element tensors of a quadrature rule (host, FP64).
void build_ref_tensors(const QuadRule &q, RefTensors &T);

struct NewtonOptions {
  double tolResidual = 1e-10;     // feNLSolverOptions (feNonLinearSolver.h:12-40)
  double tolCorrection = 1e-10;
  double tolDivergence = 1e4;
  int maxIter = 20;
  int recomputeEvery = 3;
  double residualDecrease = 0.1;
  int stationary = 1;
  double relResidual = 0.0;       // extra stop: ||R||inf <= relResidual * ||R0||inf (0: off)
  double linearRtolMin = 0.0;     // >0: adaptive linear tolerance max(min, 0.1*||R||/||R0||)
  double residualScale = 0.0;     // >0: replaces ||R0||inf in the two relative tests above
  int residualReady = 0;          // 1: u-dot and the residual of the current u are already assembled
};

struct NewtonStats {
  int iterations = 0;
  int krylovIterations = 0;
  int matrixAssemblies = 0;
  double residual0 = 0, residual = 0, correction = 0;
  int status = 0;
  int converged = 0;
};

int newton_solve(SystemCUDA &sys, const NewtonOptions &o, NewtonStats &st);

}  // namespace feng
