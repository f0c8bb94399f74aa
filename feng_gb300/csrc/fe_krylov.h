// Sparse linear algebra on the device: CSR SpMV, fused vector reductions,
// block-Jacobi ILU(0) preconditioning, CG and flexible GMRES.
//
// These replace the solve of the reference backends: PETSc KSP
// (feLinearSystemPETSc.cpp:900-1031, GMRES + ILU(0) by default, FGMRES and
// block Jacobi through run-time options) and MKL Pardiso
// (feLinearSystemMklPardiso.cpp:893-965).  The algorithms follow Saad,
// "Iterative Methods for Sparse Linear Systems", 2nd ed.: ILU(0) (Alg. 10.4),
// preconditioned CG (Alg. 9.1), flexible GMRES (Alg. 9.6) with classical
// Gram-Schmidt applied twice for the Arnoldi step (FP64 path; the mixed
// path's FP32 Arnoldi uses one pass by default, its FP64 restart residual
// corrects any loss of orthogonality).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

namespace feng {

struct DeviceCSR {
  int64_t n = 0, nnz = 0;
  int32_t *ia = nullptr;  // [n+1]
  int32_t *ja = nullptr;  // [nnz]
  int32_t *diag = nullptr;  // [n] position of the diagonal entry
};

// Block-Jacobi ILU(0): the matrix restricted to the diagonal blocks (rows and
// columns of one block), factored in place as L (unit lower) and U.
struct DeviceBlockILU {
  int64_t nBlocks = 0;
  int32_t *blockStart = nullptr;  // [nBlocks+1] into perm
  int32_t *perm = nullptr;        // [n] rows of each block, ascending
  int32_t *lia = nullptr;         // [n+1] block-local CSR, indexed by row
  int32_t *lja = nullptr;         // [lnnz] global column indices (same block only)
  int32_t *ldiag = nullptr;       // [n] position of the diagonal in lja
  int32_t *srcPos = nullptr;      // [lnnz] position of the entry in the full CSR
  int64_t lnnz = 0;
  void *vals = nullptr;           // [lnnz] factor values (double or float)
  int *status = nullptr;          // device flag: 0 ok, 1 zero pivot, 2 non-finite
  // Level schedules: a row's lower (upper) level is one more than the
  // highest level of the rows its L (U) part references, so the rows of one
  // level are independent.  rowsL/rowsU: rows by level, ascending within a
  // level; lvlL/lvlU: [nLevels+1] offsets.  Segments: runs of narrow levels
  // processed by one block (a block barrier between levels) or one wide
  // level launched over many blocks.
  int32_t *rowsL = nullptr, *lvlL = nullptr, *rowsU = nullptr, *lvlU = nullptr;
  struct Segment {
    int wide;          // 1: one level over many blocks; 0: levels [lv0, lv1) in one block
    int32_t lv0, lv1;
    int32_t rows;      // rows of the segment
    int32_t q0, q1;    // their range in rowsL / rowsU
  };
  std::vector<Segment> segL, segU;
  int32_t nLevL = 0, nLevU = 0;
};

// Host description of the multigrid-based preconditioners:
//  kind 3 (scalar field):  z = M^-1 r with M = s K, K the P2 stiffness
//                          matrix on the unknown nodes (AMG V-cycle);
//  kind 4 (Taylor-Hood):   block upper-triangular saddle-point
//                          preconditioner  [A  G; 0  S]^-1  with
//                          A^-1 ~ (s K)^-1 per velocity component (AMG) and
//                          S^-1 ~ (mu / c_div) M_p^-1 (lumped pressure mass).
// s is measured from the diagonal of the current Jacobian at each factor().
struct HostCSR;
struct PrecondInfo {
  const HostCSR *lap = nullptr;          // scalar stiffness on the nodes
  const HostCSR *massV = nullptr;        // scalar P2 mass on the nodes (same pattern as lap)
  const HostCSR *lapP = nullptr;         // P1 stiffness on the pressure unknowns (kind 4)
  std::vector<int32_t> nodeDofX, nodeDofY;  // unknown DOF of each node (per component)
  std::vector<int32_t> nodeDofZ;         // third velocity component (tetrahedra; empty in 2D)
  std::vector<int32_t> pRows;            // pressure unknowns (kind 4)
  std::vector<double> pMass;             // lumped pressure mass of pRows
  double sigma = 1, divu = 1;            // DIV_NEWTONIAN_STRESS / MIXED_DIVERGENCE coefficients
  int innerIterations = 0;               // inner AMG-preconditioned CG steps per component (0: one V-cycle)
  int chebyDegree = 2;                   // Chebyshev smoother degree
};

struct KrylovOptions {
  int method = 1;          // 0 CG, 1 FGMRES
  int restart = 50;
  int maxIter = 10000;
  double rtol = 1e-8;      // relative to ||b||_2 (PETSc default test)
  double atol = 1e-14;
  double dtol = 1e6;
  int precond = 1;         // 0 none, 1 block-Jacobi ILU(0), 2 Jacobi, 3 AMG, 4 saddle-point AMG
  int mixed = 0;           // 1: FP32 matrix/preconditioner/SpMV inside FP64 refinement
  int refineMax = 20;      // outer refinement steps in mixed mode
  double innerRtol = 1e-4; // inner FP32 solve tolerance in mixed mode
  int gsPasses = 1;        // mixed FGMRES Gram-Schmidt: 1 = once + second pass when needed, 2 = always
                           // twice, 3 = as 1 with the norm of the update by Pythagoras from the dot pass
};

struct KrylovStats {
  int iterations = 0;      // total inner iterations
  int refinements = 0;     // outer refinement steps (mixed mode)
  int status = 0;          // 0 converged, FE_NOT_CONVERGED, FE_PC_FAILED, FE_NONFINITE
  double rnorm0 = 0, rnorm = 0;
};

class Krylov {
 public:
  ~Krylov();
  // Allocates the workspace for systems of size n with the given pattern.
  int setup(const DeviceCSR &A, const std::vector<int32_t> &blockOfRow, int64_t nBlocksHint,
            const KrylovOptions &opt, cudaStream_t s, const PrecondInfo *pinfo = nullptr);
  // Factors the preconditioner from the current matrix values.
  int factor(const double *values64, const float *values32);
  // Solves A x = b (x initial guess is zero).  Returns a Status.
  int solve(const double *values64, const float *values32, const double *b, double *x,
            KrylovStats &st);
  // y = A x (FP64 values, FP64 vectors) on this object's stream.
  void spmv64(const double *values, const double *x, double *y);
  // The inner-loop FP32 product: x rounded to FP32, FP32 accumulation.
  void spmv32(const float *values, const double *x, double *y);
  // One preconditioner application z = M^-1 r (the FP32 path rounds r).
  int applyPrecond(const double *r, double *z);
  double dot(const double *x, const double *y);
  double norm2(const double *x);
  double norminf(const double *x);
  KrylovOptions opt;

 private:
  int solve_fgmres64(const double *vals, const double *b, double *x, double rtolAbs, int maxIt,
                     KrylovStats &st);
  int solve_fgmres_mixed(const float *vals32, const double *b, double *x, double rtolAbs,
                         int maxIt, KrylovStats &st);
  int solve_cg64(const double *vals, const double *b, double *x, double tolAbs, int maxIt,
                 KrylovStats &st);
  int build_ilu_levels(const std::vector<int32_t> &lia, const std::vector<int32_t> &lja,
                       const std::vector<int32_t> &ldiag);
  template <typename VF>
  void ilu_factor_levels(const double *values64, const float *values32);
  template <typename VF, typename VV>
  void ilu_solve_levels(const VV *r, VV *z, const int *done);
  void precond64(const double *r, double *z, const int *skip);
  void precond32(const float *r, float *z, const int *skip);

  DeviceCSR A_;
  DeviceBlockILU ilu_;
  cudaStream_t s_ = 0;
  int64_t n_ = 0;
  int lanes_ = 8;
  // workspace
  double *V_ = nullptr;   // (m+1) x n  Krylov basis, FP64
  double *Z_ = nullptr;   // m x n      preconditioned directions (FP64 path)
  float *Z32_ = nullptr;  // m x n      preconditioned directions (mixed path)
  float *V32_ = nullptr;  // (m+1) x n  Krylov basis of the mixed path, FP32, in row blocks of 1024
                          // rows (column c of row block k at (k (m+1) + c) 1024)
  float *vc32_ = nullptr;  // the newest basis vector, contiguous (the preconditioner's input)
  void *xs2_ = nullptr;     // float2 split of the FP64 iterate (the mixed restart residual)
  // The mixed restart residual in double-float (k_resid_sell_df) when the
  // solve's tolerance is at least 1e-9 relative (its error, ~1e-13 of
  // sum |a x| per row, stays far below the stop), else in FP64.
  bool dfResid_ = false;
  // Sliced-ELL copy of the FP32 matrix for the Arnoldi SpMV of the mixed
  // path (slices of 32 rows padded to the longest row, entries column-major
  // in the slice; padding: the row's own column, value 0), refreshed from the
  // CSR values at each factor().
  int32_t *sellPtr_ = nullptr, *sellCol_ = nullptr, *sellSrc_ = nullptr;  // sellSrc_: CSR position or -1
  float *sellVal_ = nullptr;
  int64_t sellN_ = 0;  // entries with padding
  int build_sell();
  bool allDots_ = true;       // dot pass k_gs_dots_all (else k_gs_dots)
  int *zeroFlag_ = nullptr;  // a device 0 ("not done") for gsStep
  int gsParts_ = 0;       // blocks of the FP32 Gram-Schmidt update passes
  int nSM_ = 1;           // multiprocessors of the device
  int64_t ld32_ = 0;      // rows of V32_ / Z32_ / w32_ (n rounded up to whole row blocks of V32_)
  // pass: 0 first pass (the update + norm decides on reorthogonalisation),
  // 1 the conditional second pass, 2 the last pass of an unconditional CGS2
  void gs32(int mode, int ncols, const double *hprev, double *hcur, double *Hcol, const int *done, int pass);
  float *v32_ = nullptr, *w32_ = nullptr;
  double *w_ = nullptr, *r_ = nullptr, *t_ = nullptr, *p_ = nullptr, *q_ = nullptr;
  double *diag_ = nullptr;    // inverse diagonal (Jacobi)
  float *diag32_ = nullptr;
  double *red_ = nullptr;     // partial sums [nParts * 64]
  double *hred_ = nullptr;    // pinned host mirror of final reductions
  double *dsum_ = nullptr;    // device final sums
  int nParts_ = 0;
  bool factoredOk_ = false;
  // Device-resident solver state (opaque here, defined in fe_krylov.cu).
  void *red_state_ = nullptr, *gmres_ = nullptr, *cg_ = nullptr;
  void *h_gmres_ = nullptr, *h_cg_ = nullptr;
  // Multigrid preconditioners (kinds 3, 4).
  struct MG;
  MG *mg_ = nullptr;
  const double *cur64_ = nullptr;  // matrix values of the last factor()
  const float *cur32_ = nullptr;
  int *hflag_ = nullptr;           // pinned copy of the device done flag
  double *htol_ = nullptr;         // pinned absolute tolerance read by the cycle
  bool poll_done(const int *dflag, int j);
  void launch_cycle(bool mixed, const void *vals, const double *b, double *x, int jmax, bool poll);
  void launch_cycle_mixed(const float *vals, const double *b, double *x, int jmax, bool poll);
  void mixed_part(const float *vals, const double *b, double *x, int j0, int j1, bool poll, bool pro, bool epi);
  int run_cycle_chunked(const float *vals, const double *b, double *x);
  int chunk_ = 5;               // Arnoldi steps per part graph of a mixed cycle
  int *hdone_ = nullptr;        // pinned: the done flag after each part
  std::vector<cudaEvent_t> evs_;
  int run_cycle(bool mixed, const void *vals, const double *b, double *x, int jmax);
  struct GraphKey {
    bool mixed;
    const void *vals;
    const double *b;
    double *x;
    bool dfResid;
    int part;  // -1: the whole cycle; else a part of a chunked mixed cycle
  };
  int part_graph(const GraphKey &key, int part, int P, int K, const float *vals, const double *b, double *x,
                 cudaGraphExec_t *out, size_t *nKernels);
  std::vector<std::pair<GraphKey, cudaGraphExec_t>> graphs_;
  std::vector<size_t> graphKernels_;  // kernel nodes of each graph

 public:
  bool useGraphs_ = true;  // replay full restart cycles from CUDA graphs
  int setup_mg(const PrecondInfo &pi);
  // Time-dependent saddle-point problems (velocity block ~ c0 M + mu K):
  // rebuilds the velocity multigrid on K + (c0/mu) M and adds the
  // Cahouet-Chabard term c0 L_p^-1 (pressure Laplacian multigrid) to the
  // Schur complement approximation mu M_p^-1.  c0 = 0 restores the steady
  // preconditioner.  Replayed cycle graphs are rebuilt.
  int setTransientShift(double c0, double mu);
  // The multigrid's finest-level smoother step alone (benchmarking); bytes:
  // its algorithmic bytes, 0 when there is no multigrid.
  int smootherStep(int64_t *bytes);
  // One pass of the mixed FGMRES Gram-Schmidt on the current FP32 basis with
  // ncols columns (benchmark phases): mode 0 the dot pass (k_gs_dots), mode
  // 4 the update + norm pass (k_gs_upd).  bytes: algorithmic bytes.
  int gsStep(int mode, int ncols, int64_t *bytes);
  // The same pass launched reps times back to back, cycling through copies
  // of the basis and w that together exceed three times the L2 (each launch
  // reads data evicted by the others), timed as a batch with CUDA events:
  // the average time of a pass as it runs inside the Arnoldi loop.
  int gsStepStream(int mode, int ncols, int reps, double *avgMs);
  // The Arnoldi SpMV of the mixed path on the current FP32 matrix (sliced
  // ELL when built, else CSR), FP32 vectors (benchmark phase).
  int spmvHot();
  void spmv_sell(const float *x, float *y, const int *done);
  void resid32(const float *vals, const double *x, const double *b, double *r);
  // The preconditioner application of an Arnoldi step (the mixed path: the
  // FP32 basis column 0 into Z column 0; FP64 otherwise), reps of them
  // captured in one CUDA graph and replayed (after a warm replay) without
  // anything between: ms per application (benchmark phase).
  int precondGraph(int reps, double *avgMs);
  // One full FGMRES(m) restart cycle of the current system (vals, b) from
  // x, replayed from its captured CUDA graph with the convergence test
  // disabled, so that all m Arnoldi steps run: ms per Arnoldi step, the
  // cycle's residual and update included (benchmark phase; x is scratch).
  int cycleGraph(bool mixed, const void *vals, const double *b, double *x, int reps, double *msPerStep);
  int factor_mg(const double *values64, const float *values32);
  template <typename V> void apply_mg(const V *vals, const V *r, V *z, const int *skip);
};

}  // namespace feng
