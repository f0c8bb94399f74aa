/*
 * feng_cuda.h -- C ABI of the GB300 (sm_103a) backend for feNG's element
 * assembly + Krylov solve hot path.
 *
 * Plain C types only: caller-owned host arrays in, opaque handles out, every
 * function returns an int status (0 = OK, < 0 = error, mirroring feStatus in
 * feNG's src/feMessage.h:44-62).  fe_cuda_last_error() gives the message of
 * the last failure on the calling thread.  Handles are not thread-safe.
 *
 * Two ways in:
 *  1. The drop-in route.  A feLinearSystemCUDA subclass of feNG's
 *     feLinearSystem (src/feLinearSystem.h:43-169) flattens its
 *     feBilinearForm list into fe_form_desc, its element addressing into an
 *     element-to-DOF table, and passes feNG's own CSR pattern and coloring:
 *     fe_cuda_system_create_from_tables().
 *  2. The standalone route.  The library builds mesh, numbering, pattern and
 *     coloring itself with the same algorithms (fe_mesh_*, fe_cuda_system_create).
 * Either way the per-Newton-iteration calls are the feLinearSystem
 * operations below.
 */
#ifndef FENG_CUDA_H
#define FENG_CUDA_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes: feStatus FE_STATUS_OK / FE_STATUS_ERROR and refinements */
#define FE_CUDA_OK 0
#define FE_CUDA_ERROR (-1)
#define FE_CUDA_READ_ERROR (-2)
#define FE_CUDA_INVALID_ARG (-3)
#define FE_CUDA_DEVICE_FAIL (-4)
#define FE_CUDA_NOT_CONVERGED (-5)
#define FE_CUDA_PC_FAILED (-6)
#define FE_CUDA_NONFINITE (-7)
#define FE_CUDA_BAD_COLORING (-8)

/* ---- weak forms (feSysElm elementSystemType, src/feSysElm.h:13-77) */
#define FE_FORM_SOURCE 1
#define FE_FORM_DIFFUSION 2
#define FE_FORM_VECTOR_SOURCE 3
#define FE_FORM_TRANSIENT_VECTOR_MASS 4
#define FE_FORM_MIXED_DIVERGENCE 5
#define FE_FORM_VECTOR_CONVECTIVE_ACCELERATION 6
#define FE_FORM_DIV_NEWTONIAN_STRESS 7

/* ---- device-evaluated source functions (feFunction callbacks cannot run on
 * the device; src/feFunction.h:44-56) */
#define FE_SRC_NONE 0
#define FE_SRC_SIN_SIN 1      /* p0 sin(pi x) sin(pi y)                         */
#define FE_SRC_NS_MMS_POLY 2  /* NS manufactured source, tests/withLinearSolver/navier_stokes.cpp:33-51 */
#define FE_SRC_CONST_VEC 3    /* (p0, p1)                                        */
#define FE_SRC_SIN_BODY 4     /* (p0 sin(pi x) sin(pi y), 0)                     */
#define FE_SRC_SIN3 5         /* p0 sin(pi x) sin(pi y) sin(pi z)      (tetrahedra) */
#define FE_SRC_SIN3_BODY 6    /* (p0 sin(pi x) sin(pi y) sin(pi z), 0, 0) (tetrahedra) */

/* ---- element types of the fused kernels */
#define FE_ELEM_P2 1            /* scalar Lagrange P2 triangle, 6 local DOFs          */
#define FE_ELEM_TAYLOR_HOOD 2   /* vector P2 (interleaved x,y) + P1, 12 + 3 local DOFs */
#define FE_ELEM_TET_P2 3        /* scalar P2 tetrahedron, 10 local DOFs */
#define FE_ELEM_TET_TAYLOR_HOOD 4  /* vector P2 (interleaved x,y,z) + P1 on tetrahedra, 30 + 4 */

/* ---- connectivities a space lives on (feMesh physical names) */
#define FE_CNC_DOMAIN 0    /* "Domaine"       */
#define FE_CNC_BOUNDARY 1  /* "Bord"          */
#define FE_CNC_POINT 2     /* "PointPression" */

typedef struct fe_mesh fe_mesh;
typedef struct fe_mesh3d fe_mesh3d;
typedef struct fe_cuda_system fe_cuda_system;

/* One bilinear/linear form: createBilinearForm(spaces, new feSysElm_*(coeffs)),
 * src/feBilinearForm.cpp:6-73.  Coefficients are constants
 * (feConstantFunction, src/feFunction.h:113-118). */
typedef struct fe_form_desc {
  int32_t kind;       /* FE_FORM_* */
  double coeff;       /* scalar coefficient */
  double coeff2;      /* viscosity of FE_FORM_DIV_NEWTONIAN_STRESS */
  int32_t source;     /* FE_SRC_* for the source forms */
  double params[4];   /* source parameters */
} fe_form_desc;

/* One FE space: createFiniteElementSpace(..., LAGRANGE/VECTOR_LAGRANGE, degree,
 * field, cnc), src/feSpace.cpp:11-420; essential = listed in essentialSpaces
 * of feMetaNumber, src/feNumber.cpp:677. */
typedef struct fe_space_desc {
  int32_t field;      /* field index, in order of first appearance */
  int32_t degree;     /* 0 (point), 1, 2 */
  int32_t ncomp;      /* 1 or 2 */
  int32_t cnc;        /* FE_CNC_* */
  int32_t essential;  /* 0 / 1 */
} fe_space_desc;

/* Linear solver options (feLinearSystem tolerances, src/feLinearSystem.h:66-69;
 * KSP/PC choice of the PETSc backend, src/feLinearSystemPETSc.cpp:337-352). */
typedef struct fe_cuda_options {
  int32_t krylov;         /* 0 CG, 1 FGMRES */
  int32_t restart;        /* FGMRES restart length (<= 128) */
  int32_t max_iter;
  double rel_tol;         /* ||b - A x||_2 <= max(rel_tol ||b||_2, abs_tol) */
  double abs_tol;
  double div_tol;
  int32_t precond;        /* 0 none, 1 block-Jacobi ILU(0), 2 Jacobi, 3 multigrid: AMG on the
                             scalar P2 stiffness (scalar field) or block-triangular
                             saddle-point preconditioner with AMG velocity blocks and
                             lumped pressure mass Schur complement (Taylor-Hood) */
  int32_t pc_block_rows;  /* target rows per block-Jacobi block; 0 = one block (plain ILU(0)) */
  int32_t precision;      /* 0 FP64; 1 FP32 matrix, SpMV, preconditioner inside FP64 refinement */
  int32_t quad_degree;    /* triangle rule degree: 1, 2, 4, 5, 8 */
  int32_t mg_inner;       /* multigrid: inner AMG-preconditioned CG steps per velocity
                             component (0 = a single V-cycle) */
  int32_t mg_smooth;      /* multigrid: Chebyshev smoother degree (1..6; 0 = default 1) */
  int32_t gs_passes;      /* mixed FGMRES Gram-Schmidt: 1 = one pass, a second when the update keeps
                             less than a tenth of the norm; 2 = always two; 3 = as 1, the norm of
                             the update taken as ||w||^2 - ||h||^2 from the dot pass and the next
                             basis vector written by the update pass (0 = default 1) */
} fe_cuda_options;

/* Newton options (feNLSolverOptions, src/feNonLinearSolver.h:12-40) plus the
 * relative stop ||R||inf <= rel_residual ||R0||inf used for benchmarking. */
typedef struct fe_newton_options {
  double tol_residual;
  double tol_correction;
  double tol_divergence;
  int32_t max_iter;
  int32_t recompute_every;
  double residual_decrease;
  int32_t stationary;
  double rel_residual;
  double linear_rtol_min;   /* > 0: inexact Newton, linear rtol = max(this, 0.1 ||R||/||R0||) */
  double residual_scale;    /* > 0: replaces ||R0||inf in the two relative tests above (time
                               steps: the residual of the previous step's solution, so that
                               the stop does not depend on the initial guess) */
} fe_newton_options;

typedef struct fe_newton_stats {
  int32_t iterations;
  int32_t krylov_iterations;
  int32_t matrix_assemblies;
  int32_t status;
  double residual0;
  double residual;
  double correction;
  double residual_ms;  /* device time of the phases, CUDA events */
  double matrix_ms;
  double factor_ms;
  double solve_ms;
} fe_newton_stats;

/* ---- library */
const char *fe_cuda_last_error(void);
int fe_cuda_version(void);
int fe_cuda_device_count(int *count);

/* ---- mesh (feMesh2DP1, src/feMesh.h:357-497; reader src/feMeshRead.cpp:645) */
int fe_mesh_generate_square(int n, double x0, double x1, double y0, double y1, double jitter,
                            uint64_t seed, fe_mesh **out);
int fe_mesh_read_msh(const char *path, fe_mesh **out);
/* As fe_mesh_read_msh with the physical groups named by the caller: the
 * triangles of `domain` become "Domaine", the lines of the n_boundary groups
 * in `boundary` (merged in the file's entity order) "Bord", the vertex of
 * `point` (NULL or "": none) "PointPression".  feNG selects a space's
 * connectivity by physical name (createFiniteElementSpace cncGeoID,
 * src/feSpace.cpp:11-60); this maps a file's names onto the three roles. */
int fe_mesh_read_msh_groups(const char *path, const char *domain, const char *const *boundary,
                            int n_boundary, const char *point, fe_mesh **out);
int fe_mesh_write_msh(const fe_mesh *m, const char *path);
/* A mesh from caller arrays (0-based): vertices x, y; counter-clockwise
 * triangles of "Domaine"; boundary lines of "Bord" (oriented like the
 * triangle edge they lie on); the "PointPression" vertex or -1.  Same result
 * as reading a msh file that holds these entities in this order. */
int fe_mesh_from_arrays(int64_t n_vertices, const double *x, const double *y, int64_t n_triangles,
                        const int32_t *tri, int64_t n_boundary, const int32_t *bnd, int32_t point,
                        fe_mesh **out);
int fe_mesh_sizes(const fe_mesh *m, int64_t *n_vertices, int64_t *n_triangles, int64_t *n_edges,
                  int64_t *n_boundary);
/* Any output may be NULL.  x,y [nv]; tri [3 nt]; tri_edges [3 nt]; bnd [2 nb]; point [1]. */
int fe_mesh_arrays(const fe_mesh *m, double *x, double *y, int32_t *tri, int32_t *tri_edges,
                   int32_t *bnd, int32_t *point);
void fe_mesh_destroy(fe_mesh *m);

/* ---- 3D tetrahedral meshes ("Domaine" tetrahedra, "Bord" boundary
 * triangles; read by the reference as feMesh2DP1, src/feMeshRead.cpp:1481-1538).
 * fe_mesh3d_generate_cube: n^3 cells of box {x0,x1,y0,y1,z0,z1}, 6 Kuhn
 * tetrahedra per cell (positive volumes, conforming), interior vertices
 * jittered by U(-jitter h, jitter h) per axis from SplitMix64(seed); boundary
 * triangles oriented outwards. */
int fe_mesh3d_generate_cube(int n, const double *box, double jitter, uint64_t seed, fe_mesh3d **out);
int fe_mesh3d_write_msh(const fe_mesh3d *m, const char *path);
/* Reads "Domaine" tetrahedra and "Bord" triangles (the triangles must precede
 * the tetrahedra in the file, as Gmsh writes them). */
int fe_mesh3d_read_msh(const char *path, fe_mesh3d **out);
/* A mesh from caller arrays (0-based): vertices; tetrahedra of "Domaine";
 * boundary triangles of "Bord".  Same result as reading a msh file holding
 * these entities in this order. */
int fe_mesh3d_from_arrays(int64_t n_vertices, const double *x, const double *y, const double *z,
                          int64_t n_tets, const int32_t *tet, int64_t n_boundary, const int32_t *bnd,
                          fe_mesh3d **out);
int fe_mesh3d_sizes(const fe_mesh3d *m, int64_t *n_vertices, int64_t *n_tets, int64_t *n_boundary);
/* Any output may be NULL.  x,y,z [nv]; tet [4 nt]; bnd [3 nb]. */
int fe_mesh3d_arrays(const fe_mesh3d *m, double *x, double *y, double *z, int32_t *tet, int32_t *bnd);
void fe_mesh3d_destroy(fe_mesh3d *m);

/* ---- set-up of the standalone route: DOF numbering (feMetaNumber,
 * src/feNumber.cpp:677-835), element-to-DOF tables of elem_type (the P2
 * space on "Domaine" is the scalar / velocity field, the P1 space on
 * "Domaine" the pressure), element coloring (feCncGeo::colorElements(1),
 * src/feCncGeo.cpp:735), CSR pattern (feEZCompressedRowStorage,
 * src/feCompressedRowStorage.cpp:15-135), quadrature rule (getGQTPts,
 * src/feQuadratureTri.cpp:874) and a block-Jacobi partition with about
 * pc_block_rows unknowns per block.  All on the host threads except the CSR
 * pattern, which is built on the current CUDA device when one is present
 * (the same pattern, bit for bit; fe_setup_set_pattern_mode). */
typedef struct fe_setup fe_setup;
int fe_setup_create(const fe_mesh *m, const fe_space_desc *spaces, int nspaces, int elem_type,
                    int quad_degree, int pc_block_rows, fe_setup **out);
void fe_setup_destroy(fe_setup *s);
/* The same host set-up on a tetrahedral mesh, elem_type FE_ELEM_TET_P2 (scalar
 * P2, 10 local DOFs: 4 vertices, then the edges (0,2) (2,1) (1,0) (1,3) (3,0)
 * (3,2), feSpaceTetPn(2)) or FE_ELEM_TET_TAYLOR_HOOD (3-vector P2
 * interleaved + P1, 34 local DOFs; no reference counterpart).  Spaces on
 * FE_CNC_DOMAIN (tetrahedra) and FE_CNC_BOUNDARY (triangles).  Numbering,
 * element tables, coloring and CSR pattern as the reference builds them on
 * the same msh file; no quadrature rule (get_* of the triangle set-up work,
 * fe_cuda_system_create refuses it). */
int fe_setup3d_create(const fe_mesh3d *m, const fe_space_desc *spaces, int nspaces, int elem_type,
                      int pc_block_rows, fe_setup **out);
/* Replaces the set-up's quadrature rule (nq rows (r, s, w) or, on
 * tetrahedra, (r, s, t, w)), e.g. with the reference's tabulated values;
 * without it a tetrahedral set-up takes the rule of the options' degree. */
int fe_setup_set_quadrature(fe_setup *s, int nq, const double *rule);
/* z coordinate of every DOF (tetrahedral set-ups only). */
int fe_setup_get_dof_z(const fe_setup *s, double *z);
/* Where the set-ups created afterwards (and the systems created from tables
 * without a pattern) build the CSR pattern: -1 on the current CUDA device
 * when one is present, else on the host (the default; also the host when a
 * row has more than 1023 candidate columns), 0 on the host threads, 1 on the
 * device (an error without one).  Process-wide. */
int fe_setup_set_pattern_mode(int mode);
/* 1 when the set-up's pattern was built on the device. */
int fe_setup_pattern_on_device(const fe_setup *s, int *on_device);
int fe_setup_sizes(const fe_setup *s, int64_t *n_inc, int64_t *n_dofs, int64_t *nnz,
                   int64_t *n_elm, int *n_colors, int *nloc);
/* Outputs may be NULL.  ia [n_inc+1], ja [nnz]. */
int fe_setup_get_pattern(const fe_setup *s, int64_t *ia, int32_t *ja);
/* offsets [n_colors+1], elements [n_elm]. */
int fe_setup_get_coloring(const fe_setup *s, int64_t *offsets, int32_t *elements);
/* adr [n_elm*nloc], original element order. */
int fe_setup_get_element_dofs(const fe_setup *s, int64_t *adr);
/* DOF locations: x, y, field, component, is_vertex [n_dofs]. */
int fe_setup_get_dof_info(const fe_setup *s, double *x, double *y, int32_t *field, int32_t *comp,
                          int32_t *is_vertex);
/* block_of_row [n_inc]. */
int fe_setup_get_blocks(const fe_setup *s, int32_t *block_of_row);
/* Quadrature rule: n points (<= 16), r, s, w [n]. */
int fe_quadrature_rule(int degree, int *n, double *r, double *s, double *w);
/* Tetrahedral rule of degree 1..8 (1, 4, 5, 11, 14, 24, 31, 43 points; the
 * orbit structures of getGQTetPts, src/feQuadratureTet.cpp:3342), weights
 * summing to 1/6; outputs may be NULL to query n. */
int fe_tet_quadrature_rule(int degree, int *n, double *r, double *s, double *t, double *w);

/* ---- VTK export (feExporterVTK::writeStep, src/feExporter.h:36-116,
 * src/feExporter.cpp:854-990), on the host, no device needed.
 * Writes the legacy ASCII VTK file the reference writes for continuous
 * fields on a P1 triangle mesh: the vertices, then one node per edge midpoint
 * (edges in ascending (min vertex, max vertex) order) when a field is P2;
 * 6-node quadratic triangles (VTK type 22), or 3-node triangles (5) when every
 * field is P1; one FIELD array per field (2-vectors with a zero third
 * component).  solution [n_dofs] holds every DOF (unknowns, then essential
 * DOFs).  field_names [n_field_names = number of fields] name the fields in
 * the order of fe_space_desc.field; required [n_required] selects fields by
 * name (0: every field with a space on "Domaine").  Fields are written in the
 * reverse order of their first space on "Domaine", as the reference writes
 * "U" then "P" (P first).  precision: significant digits, 0 = 6 (the
 * reference's stream default), up to 17 for a lossless file.  m must be the
 * mesh s was created on. */
int fe_export_vtk(const fe_mesh *m, const fe_setup *s, const double *solution,
                  const char *const *field_names, int n_field_names, const char *const *required,
                  int n_required, int precision, const char *path);
/* The same for a tetrahedral set-up: VTK_QUADRATIC_TETRA cells (24, VTK's node
 * order: vertices, then edges (0,1) (1,2) (0,2) (0,3) (1,3) (2,3)), or
 * VTK_TETRA (10) when every field is P1; 3-vectors written as they are.  The
 * reference has no tetrahedral P2 layout to follow. */
int fe_export_vtk3d(const fe_mesh3d *m, const fe_setup *s, const double *solution,
                    const char *const *field_names, int n_field_names, const char *const *required,
                    int n_required, int precision, const char *path);

/* ---- system creation */
/* Standalone route: device system from a host set-up. */
int fe_cuda_system_create(const fe_setup *setup, const fe_form_desc *forms, int nforms,
                          const fe_cuda_options *opt, fe_cuda_system **out);
/* Drop-in route: the caller's tables.  adr [n_elm * nloc] global DOFs per
 * element in the fused layout; elem_xy [n_elm * 6] vertex coordinates;
 * color_offsets [n_colors+1] / color_elements [n_elm] (may be NULL);
 * ia [n_inc+1] / ja [nnz] the caller's pattern (may be NULL);
 * block_of_row [n_inc] block-Jacobi partition (may be NULL). */
int fe_cuda_system_create_from_tables(int elem_type, int64_t n_elm, const int64_t *adr,
                                      const double *elem_xy, int64_t n_inc, int64_t n_dofs,
                                      int n_colors, const int64_t *color_offsets,
                                      const int32_t *color_elements, const int64_t *ia,
                                      const int32_t *ja, const int32_t *block_of_row,
                                      const fe_form_desc *forms, int nforms,
                                      const fe_cuda_options *opt, fe_cuda_system **out);
/* As fe_cuda_system_create_from_tables, with the quadrature rule given as nq
 * rows (r, s, w) on triangles or (r, s, t, w) on tetrahedra (the reference's
 * own tabulated values, feSpace::getRQuadraturePoints / getSQuadraturePoints /
 * getTQuadraturePoints / getQuadratureWeights); nq = 0: the rule of
 * opt->quad_degree.  Element types: FE_ELEM_P2, FE_ELEM_TAYLOR_HOOD (elem_xy
 * [n_elm*6]) and FE_ELEM_TET_P2, FE_ELEM_TET_TAYLOR_HOOD (elem_xy [n_elm*12],
 * x y z of the four vertices). */
int fe_cuda_system_create_from_tables_rule(int elem_type, int64_t n_elm, const int64_t *adr,
                                           const double *elem_xy, int64_t n_inc, int64_t n_dofs,
                                           int n_colors, const int64_t *color_offsets,
                                           const int32_t *color_elements, const int64_t *ia,
                                           const int32_t *ja, const int32_t *block_of_row,
                                           const fe_form_desc *forms, int nforms,
                                           const fe_cuda_options *opt, int nq, const double *rule,
                                           fe_cuda_system **out);
void fe_cuda_system_destroy(fe_cuda_system *s);

int fe_cuda_system_sizes(const fe_cuda_system *s, int64_t *n_inc, int64_t *n_dofs, int64_t *nnz,
                         int64_t *n_elm, int *n_colors);
/* How the Jacobian is assembled: 1 row-owned (each CSR row summed by its
 * owner in color order; the FP32 Taylor-Hood Jacobians whose rows hold fewer
 * than 255 entries), 0 the colored scatter.  Both give the same sums in
 * the same order. */
int fe_cuda_jacobian_route(const fe_cuda_system *s, int *route);
int fe_cuda_get_pattern(const fe_cuda_system *s, int64_t *ia, int32_t *ja);
int fe_cuda_get_coloring(const fe_cuda_system *s, int64_t *offsets, int32_t *elements);
/* Rejects a coloring in which two elements of one color share a vertex DOF. */
int fe_cuda_validate_coloring(const fe_cuda_system *s);

/* ---- state (feSolution: _sol / _dsoldt, src/feSolution.h) */
int fe_cuda_set_solution(fe_cuda_system *s, const double *u, const double *udot);
int fe_cuda_get_solution(const fe_cuda_system *s, double *u);
int fe_cuda_set_time(fe_cuda_system *s, double t, double c0);
/* BDF history for the time derivative (BDFContainer, src/feSolutionContainer.cpp:82-101,338-349):
 * udot = cn[0] u + cn[1] hist1 + cn[2] hist2.  hist1/hist2 may be NULL to keep the device copy. */
int fe_cuda_set_bdf(fe_cuda_system *s, int order, const double *cn, const double *hist1,
                    const double *hist2);
int fe_cuda_compute_soldot(fe_cuda_system *s);

/* ---- error norms (feNorm L2_ERROR / VECTOR_L2_ERROR, src/feNorm.cpp:152-163,323-391,1399-1443)
 * on the quadrature rule of the system's forms.  fe_cuda_norm_points gives the
 * rule's nodes on every element (nq per element, the system's element order;
 * x, y: n_elm * nq doubles, or NULL to query nq only): the caller evaluates
 * its exact solution there (feNorm's feFunction calls) and passes the values
 * to fe_cuda_l2_error as [n_elm][nq][ncomp].  field 0: the P2 field (scalar
 * P2 systems: 1 component; Taylor-Hood: the velocity, 2 components), field 1:
 * the P1 pressure of Taylor-Hood (1 component).  error = sqrt(sum over
 * elements, nodes and components of |exact - u_h|^2 |J| w), computed on the
 * device from the current solution. */
int fe_cuda_norm_points(fe_cuda_system *s, int *nq, double *x, double *y);
int fe_cuda_l2_error(fe_cuda_system *s, int field, const double *exact, double *error);

/* ---- feLinearSystem operations (src/feLinearSystem.h:96-145) */
int fe_cuda_set_to_zero(fe_cuda_system *s);
int fe_cuda_set_matrix_to_zero(fe_cuda_system *s);
int fe_cuda_set_residual_to_zero(fe_cuda_system *s);
int fe_cuda_assemble_residuals(fe_cuda_system *s);
int fe_cuda_assemble_matrices(fe_cuda_system *s);
int fe_cuda_get_rhs_max_norm(fe_cuda_system *s, double *norm);
/* setRelativeTol / setAbsoluteTol / setMaxIter (src/feLinearSystem.h:86-89). */
int fe_cuda_set_tolerances(fe_cuda_system *s, double rel_tol, double abs_tol, int max_iter);
/* Returns FE_CUDA_OK when converged (solve() -> true). */
int fe_cuda_solve(fe_cuda_system *s, double *norm_dx, double *norm_rhs, double *norm_axb,
                  int *n_iter);
int fe_cuda_correct_solution(fe_cuda_system *s);
int fe_cuda_get_matrix(const fe_cuda_system *s, double *values);
int fe_cuda_get_rhs(const fe_cuda_system *s, double *rhs);
int fe_cuda_get_du(const fe_cuda_system *s, double *du);
/* max |du| of the last correction on the device (getResidualMaxNorm,
 * src/feLinearSystemMklPardiso.cpp:352-355), without copying du to the host;
 * FE_CUDA_NONFINITE if it holds a NaN or an infinity. */
int fe_cuda_get_du_max_norm(fe_cuda_system *s, double *norm);
/* One application z = M^-1 r of the preconditioner (PETSc's PCApply),
 * built from the current matrix first if needed; r, z host arrays [n_inc]. */
int fe_cuda_apply_preconditioner(fe_cuda_system *s, const double *r, double *z);

/* ---- Newton driver (solveNewtonRaphson, src/feNonLinearSolver.cpp:38-181) */
int fe_cuda_newton(fe_cuda_system *s, const fe_newton_options *o, fe_newton_stats *st);
/* Phase timers since creation or the last reset. */
int fe_cuda_get_times(const fe_cuda_system *s, double *residual_ms, double *matrix_ms,
                      double *factor_ms, double *solve_ms);
int fe_cuda_reset_times(fe_cuda_system *s);
/* Mean device milliseconds of one phase over `reps` runs timed with CUDA
 * events on the system stream, each run preceded by an L2 flush (a write, then a read, of
 * flush_bytes): which = 0 residual assembly (all colors), 1 Jacobian assembly
 * (a zeroed matrix, then the Jacobian), 2 SpMV with the system matrix, 3 one preconditioner
 * application, 4 one finest-level multigrid pre-smoothing pass (zero start
 * fused with the first Chebyshev step, both velocity components), 5 one
 * Gram-Schmidt dot pass of the mixed FGMRES over restart/2 basis vectors,
 * 6 one Gram-Schmidt update + norm pass over restart/2 basis vectors;
 * 7 and 8 the passes of 5 and 6 launched 10 * reps times back to back, with
 * no flush between them, cycling through copies of the basis that together
 * exceed three times the L2 (the mean time of a pass inside the Arnoldi
 * loop, where the launches follow one another; flush_bytes unused);
 * 9 the dot pass of 5 by the column-group kernel (k_gs_dots; phase 5 runs
 * k_gs_dots_all, one pass over w and every column);
 * 11 the preconditioner application of an Arnoldi step, 5 * reps of them
 * captured in one CUDA graph and replayed back to back (flush_bytes unused);
 * 12 one Arnoldi step of a full FGMRES restart cycle replayed from its CUDA
 * graph with the convergence test disabled (reps / 5 cycles, at least one;
 * the cycle's restart residual and solution update included; flush_bytes
 * unused).
 * Phases 5 to 9 need a mixed-precision system that has solved once, 11 and 12 a system that has solved
 * once (12: FGMRES).  Uses the current solution state. */
int fe_cuda_bench_phase(fe_cuda_system *s, int which, int reps, int64_t flush_bytes, double *avg_ms);
/* Algorithmic bytes of one run of phase 4 (finest multigrid operator read
 * once, each vector entry read or written once). */
int fe_cuda_smoother_bytes(fe_cuda_system *s, int64_t *bytes);
/* Algorithmic bytes of one run of phase 4 to 10 (every operand read or
 * written once). */
int fe_cuda_phase_bytes(fe_cuda_system *s, int which, int64_t *bytes);
/* Kernel launches of the library since load (graph replays count their
 * kernel nodes). */
int fe_cuda_launch_count(int64_t *count);
/* Device-side copy of the solution vector: save / restore (no host traffic). */
int fe_cuda_save_solution(fe_cuda_system *s);
int fe_cuda_restore_solution(fe_cuda_system *s);
/* CUDA events on the system stream: record event `slot` (0..7); elapsed
 * milliseconds between two recorded slots (synchronizes on the later one). */
int fe_cuda_event_record(fe_cuda_system *s, int slot);
int fe_cuda_event_elapsed(fe_cuda_system *s, int slot0, int slot1, double *ms);
/* Selects the CUDA device of the calling thread (one process per GPU). */
int fe_cuda_set_device(int device);
int fe_cuda_synchronize(fe_cuda_system *s);

/* ---- partially essential vector components and periodic DOFs
 * (feLinearSystemMklPardiso::constrainEssentialComponents, src/feLinearSystemMklPardiso.cpp:994-1117;
 *  applyPeriodicity, :1119-1149).  The rows (unknowns of the essential components of vector
 * spaces) and the (master, slave) pairs are set once; each apply then zeroes the constrained
 * rows and their column occurrences with 1 on the diagonal and 0 in the right-hand side, and
 * turns each slave row into u_slave - u_master = 0.  Entries >= the unknown count are ignored.
 * fe_cuda_newton applies both after every assembly.  The preconditioner is rebuilt at the
 * next solve. */
int fe_cuda_set_constrained_rows(fe_cuda_system *s, const int64_t *rows, int64_t n);
int fe_cuda_constrain_essential_components(fe_cuda_system *s);
int fe_cuda_set_periodic_pairs(fe_cuda_system *s, const int64_t *master, const int64_t *slave, int64_t n);
int fe_cuda_apply_periodicity(fe_cuda_system *s);

/* ---- BDF2 time integration on device-resident history (BDF2Integrator::makeSteps,
 * src/feTimeIntegration.cpp:449-547, started as startWithBDF1, :383-435; BDF
 * coefficients and history rotation, src/feSolutionContainer.cpp:82-101,291-304).
 * The system's current solution (fe_cuda_set_solution) is the initial
 * condition, with its essential values; the forms must include
 * FE_FORM_TRANSIENT_VECTOR_MASS.  Each step's Newton solve stops when
 * ||R||inf <= rel_residual * ||R(u^n)||inf at the new time level (and on the
 * absolute tests), whatever its initial guess:
 *   FE_GUESS_PREVIOUS     u^n, as the reference;
 *   FE_GUESS_EXTRAPOLATE  u^n + dt_n/dt_{n-1} (u^n - u^{n-1});
 *   FE_GUESS_LEARNED      the extrapolation plus the correction of a per-node
 *                         MLP (16 -> 64 -> 64 -> 4, tanh, FP32; inputs: the last
 *                         three solutions and 6 geometry features) trained online
 *                         with device forward/backward/Adam kernels on the
 *                         corrections of converged steps from step train_from;
 *                         from step use_from the correction d is scaled by the
 *                         step length alpha minimising the linearised residual
 *                         with the Jacobian held from the previous step, the
 *                         extrapolation and ue + alpha d are both evaluated with
 *                         the FP64 residual and the smaller one is used; after 8
 *                         losses in a row the network is neither evaluated nor
 *                         trained for 32 steps (no counterpart in the reference). */
#define FE_GUESS_PREVIOUS 0
#define FE_GUESS_EXTRAPOLATE 1
#define FE_GUESS_LEARNED 2
typedef struct fe_transient fe_transient;
typedef struct fe_transient_options {
  double dt;
  double t0;
  int32_t guess;         /* FE_GUESS_* */
  int32_t train_from;    /* first step that trains the network */
  int32_t use_from;      /* first step that may use the learned guess */
  int32_t train_iters;   /* Adam steps per time step */
  int64_t batch;         /* nodes per Adam step */
  double lr;             /* Adam learning rate */
  uint64_t seed;         /* weights and minibatch sampling */
} fe_transient_options;
typedef struct fe_step_stats {
  int32_t step;
  int32_t newton_iterations;
  int32_t krylov_iterations;
  int32_t status;
  int32_t guess_used;      /* FE_GUESS_* */
  double t;
  double residual_ref;     /* ||R(u^n)||inf at the new time level */
  double residual_guess;   /* ||R||inf at the guess used */
  double residual_extrap;  /* ||R||inf at the extrapolation (0 if not formed) */
  double residual;         /* final ||R||inf */
  double step_ms;          /* device time of the whole step */
  double guess_ms;         /* ... up to the end of the guess */
  double train_ms;         /* ... of the training after the step */
  double train_loss;       /* loss of the last Adam step (-1: no training) */
  double guess_scale;      /* step length alpha of the learned correction (0: none formed) */
} fe_step_stats;
int fe_cuda_transient_create(fe_cuda_system *s, const fe_transient_options *o,
                             const fe_newton_options *newton, fe_transient **out);
/* Advances nsteps steps; stats [nsteps] may be NULL. */
int fe_cuda_transient_steps(fe_transient *t, int nsteps, fe_step_stats *stats);
/* The learned guess's network (fe_mlp_sizes' nparams floats, the packing of
 * fe_mlp_set_params): saved after a run, restored to warm-start another (a
 * restored network may be used from use_from on; no counterpart in the
 * reference). */
int fe_cuda_transient_get_network(const fe_transient *t, float *params);
int fe_cuda_transient_set_network(fe_transient *t, const float *params);
void fe_cuda_transient_destroy(fe_transient *t);

/* ---- the learned-guess MLP alone, through host buffers (tests and tools; same
 * kernels as the integrator; no counterpart in the reference).  Parameters are
 * packed W1 [64x16], b1 [64], W2 [64x64], b2 [64], W3 [4x64], b3 [4] (row-major);
 * loss = sum mask (y - t)^2 / (4 n). */
typedef struct fe_mlp fe_mlp;
int fe_mlp_sizes(int *nin, int *h1, int *h2, int *nout, int64_t *nparams);
int fe_mlp_create(uint64_t seed, int64_t max_batch, fe_mlp **out);
void fe_mlp_destroy(fe_mlp *m);
int fe_mlp_set_params(fe_mlp *m, const float *params);
int fe_mlp_get_params(fe_mlp *m, float *params_out);
int fe_mlp_forward(fe_mlp *m, const float *x, int64_t n, float *y);
/* Loss and gradient of the batch (x [n x 16], t and mask [n x 4]) before one
 * Adam step with learning rate lr (beta 0.9 / 0.999, eps 1e-8). */
int fe_mlp_train_step(fe_mlp *m, const float *x, const float *t, const float *mask, int64_t n,
                      double lr, float *grad, double *loss);

/* ---- allocation-free variant (no counterpart in the reference)
 * Max-norm max_i |x_i| of a caller-owned device vector, for callers that may
 * not allocate device memory (a host framework that owns every device byte
 * through its own pool, a loop that cannot afford cudaMalloc's implicit
 * synchronization).  Same reduction as fe_cuda_get_rhs_max_norm, but its
 * scratch is a static device array of the library (about 8 KB per GPU, held
 * until the process exits): nothing is allocated or freed.  n may be at most
 * FE_NOALLOC_MAX_N; larger n is rejected with FE_CUDA_INVALID_ARG.  `stream`
 * is a cudaStream_t (NULL: the legacy default stream); the call waits for it
 * and writes the result to host memory.  The first call on each device looks
 * up the scratch's device address (make it before any stream capture); that
 * address is kept for the life of the process, so the call must not be used
 * on a device after cudaDeviceReset.  All calls share the one scratch array:
 * calls that overlap on the GPU race.  A NaN in x gives a NaN result. */
#define FE_NOALLOC_MAX_N 4194304
int fe_cuda_max_norm_noalloc(const double *x, int64_t n, void *stream, double *result);

#ifdef __cplusplus
}
#endif

#endif /* FENG_CUDA_H */
