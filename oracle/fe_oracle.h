/* CPU oracle for the assembly + Krylov hot path.  TEST INFRASTRUCTURE ONLY:
 * the parity tests, __graft_entry__.smoke() and bench.py's CPU-baseline leg
 * use it as the checker; the product never calls it.
 *
 * It restates, in plain C, the reference algorithms the GPU path replaces:
 *   element kernels per quadrature node   feSysElm.cpp:16-27, 530-583;
 *                                         feVectorSysElm.cpp:112-130, 390-427,
 *                                         685-747, 1171-1240, 1454-1530
 *   physical gradients                    feSpace.cpp:669-768, feCncGeo.cpp:651-670
 *   colored scatter (sorted local indices + linear scan of the CSR row)
 *                                         feLinearSystemMklPardiso.cpp:501-749
 *   Newton-Raphson                        feNonLinearSolver.cpp:38-181
 * and the published Krylov algorithms (Saad, Iterative Methods for Sparse
 * Linear Systems, 2nd ed.): ILU(0) Alg. 10.4, PCG Alg. 9.1, FGMRES Alg. 9.6.
 * Its pins: the golden fixtures produced by the reference library itself
 * (tests/golden), checked by the CPU tests.
 */
#ifndef FE_ORACLE_H
#define FE_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Forms (same ids as FE_FORM_* of include/feng_cuda.h). */
typedef struct fo_forms {
  int elem_type;   /* 1 scalar P2, 2 Taylor-Hood */
  int has_diff; double diff;
  int has_conv; double conv;
  int has_sigma; double sigma, mu;
  int has_divu; double divu;
  int has_mass; double mass;
  int src_kind; double src_coeff; double src_param[4];
} fo_forms;

typedef struct fo_problem {
  int elem_type;
  int64_t n_elm;
  int nloc;
  int64_t n_inc, n_dofs;
  const int64_t *adr;        /* [n_elm*nloc] */
  const double *elem_xy;     /* [n_elm*6] */
  int n_colors;
  const int64_t *color_offsets;
  const int32_t *color_elements;
  const int64_t *ia;         /* [n_inc+1] */
  const int32_t *ja;         /* [nnz] */
  int nq;
  const double *qr, *qs, *qw;
  fo_forms forms;
} fo_problem;

/* rhs (n_inc) and values (nnz) are accumulated (caller zeroes them).
 * elem_begin/elem_end select a range of the color order (for sampling). */
int fo_assemble_residual(const fo_problem *p, const double *u, const double *udot, double *rhs,
                         int64_t elem_begin, int64_t elem_end, int nthreads);
int fo_assemble_matrix(const fo_problem *p, const double *u, double c0, double *values,
                       int64_t elem_begin, int64_t elem_end, int nthreads);

/* Sparse helpers on the n_inc x n_inc CSR system. */
void fo_spmv(int64_t n, const int64_t *ia, const int32_t *ja, const double *a, const double *x,
             double *y, int nthreads);

/* Preconditioners.  kind: 0 none, 1 block-Jacobi ILU(0) (block_of_row may be
 * NULL for one block), 2 Jacobi, 3 block-triangular Schur for Taylor-Hood
 * (velocity block: block-Jacobi ILU(0); pressure: lumped mass / viscosity). */
typedef struct fo_precond fo_precond;
fo_precond *fo_precond_create(int kind, int64_t n, const int64_t *ia, const int32_t *ja,
                              const int32_t *block_of_row, const int32_t *is_pressure,
                              const double *pmass_lumped, double viscosity);
int fo_precond_factor(fo_precond *pc, const double *values);
void fo_precond_apply(fo_precond *pc, const double *r, double *z);
void fo_precond_destroy(fo_precond *pc);

/* Smoothed-aggregation multigrid and the block-triangular saddle-point
 * preconditioner (fe_oracle_mg.c).  kind 4: Taylor-Hood (nn velocity nodes
 * with rows dofx/dofy, np pressure rows prows with lumped masses pmass; K the
 * scalar P2 stiffness on the nodes; sigma, divu the stress and divergence
 * coefficients); kind 5: scalar (nodes = unknown rows dofx, K on them).
 * The index arrays of the system (ia, ja) must outlive the object. */
typedef struct fo_mg fo_mg;
fo_mg *fo_mg_create(int64_t n, const int64_t *ia, const int32_t *ja, const double *a, double theta,
                    int64_t coarse_size);
void fo_mg_vcycle(fo_mg *M, const double *b, double *x, int nv);
int fo_mg_levels(const fo_mg *M);
double fo_mg_diag_sum(const fo_mg *M);
void fo_mg_destroy(fo_mg *M);
typedef struct fo_spmg fo_spmg;
fo_spmg *fo_spmg_create(int kind, int64_t n, const int64_t *ia, const int32_t *ja, int64_t nn,
                        const int64_t *kia, const int32_t *kja, const double *ka, const int32_t *dofx,
                        const int32_t *dofy, int64_t np, const int32_t *prows, const double *pmass,
                        double sigma, double divu);
int fo_spmg_factor(fo_spmg *S, const double *values);
void fo_spmg_apply(fo_spmg *S, const double *r, double *z);
void fo_spmg_destroy(fo_spmg *S);
/* A preconditioner object that applies S (kinds 4 and 5; S stays owned by
 * the caller). */
fo_precond *fo_precond_from_spmg(fo_spmg *S);

/* Greedy vertex-sharing coloring of elements given by nvpe vertices each
 * (feCncGeo::colorElements algorithm 1, src/feCncGeo.cpp:752-790): writes
 * the color of each element; returns the number of colors (< 0 on error). */
int fo_color_elements(const int32_t *ev, int nvpe, int64_t ne, int64_t nv, int32_t *color);

/* Threads of the OpenMP regions without an explicit count. */
void fo_set_threads(int n);

typedef struct fo_krylov_stats {
  int iterations;
  int converged;
  double rnorm0, rnorm;
} fo_krylov_stats;

/* method 0 CG, 1 FGMRES(restart).  x starts at zero.  Converged when
 * ||b - A x||_2 <= max(rtol ||b||_2, atol). */
int fo_krylov_solve(int method, int restart, int max_iter, double rtol, double atol, int64_t n,
                    const int64_t *ia, const int32_t *ja, const double *a, fo_precond *pc,
                    const double *b, double *x, fo_krylov_stats *st, int nthreads);

/* Essential components / periodicity (feLinearSystemMklPardiso.cpp:994-1149). */
void fo_constrain(int64_t n, const int64_t *ia, const int32_t *ja, double *values, double *rhs,
                  const int64_t *rows, int64_t nrows);
void fo_periodicity(int64_t n, const int64_t *ia, const int32_t *ja, double *values, double *rhs,
                    const int64_t *master, const int64_t *slave, int64_t npairs);

#ifdef __cplusplus
}
#endif
#endif
