// Device-side data of one linear system and the kernel entry points.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace feng {

struct QuadRule;

// Weak forms the fused element kernels know, named after feNG's
// elementSystemType (feSysElm.h:13-77).
enum FormKind : int {
  FORM_SOURCE = 1,                           // feSysElm_Source
  FORM_DIFFUSION = 2,                        // feSysElm_Diffusion<2>
  FORM_VECTOR_SOURCE = 3,                    // feSysElm_VectorSource<2>
  FORM_TRANSIENT_VECTOR_MASS = 4,            // feSysElm_TransientVectorMass<2>
  FORM_MIXED_DIVERGENCE = 5,                 // feSysElm_MixedDivergence<2>
  FORM_VECTOR_CONVECTIVE_ACCELERATION = 6,   // feSysElm_VectorConvectiveAcceleration<2>
  FORM_DIV_NEWTONIAN_STRESS = 7,             // feSysElm_DivergenceNewtonianStress<2>
};

// Closed registry of non-constant source functions evaluated on the device
// at quadrature nodes (std::function callbacks cannot run there).
enum SourceKind : int {
  SRC_NONE = 0,
  SRC_SIN_SIN = 1,        // scalar  f = p0 * sin(pi x) sin(pi y)
  SRC_NS_MMS_POLY = 2,    // vector  manufactured NS source of u=(x^4y^4, -4/5 x^3y^5), p=x^2y^2
  SRC_CONST_VEC = 3,      // vector  f = (p0, p1)
  SRC_SIN_BODY = 4,       // vector  f = (p0 sin(pi x) sin(pi y), 0)
  SRC_SIN3 = 5,           // scalar  f = p0 sin(pi x) sin(pi y) sin(pi z)          (tetrahedra)
  SRC_SIN3_BODY = 6,      // vector  f = (p0 sin(pi x) sin(pi y) sin(pi z), 0, 0)  (tetrahedra)
};

// Reference-element tensors of a tetrahedral rule (sums over its nodes,
// weights included; r, s, t the reference directions, a, b, c P2 functions
// in the local order of feSpaceTetPn(2): vertices, then TET_EDGES; j P1):
//   K[r][s][a][b] = sum_q w dphi_a/dr dphi_b/ds
//   T[r][a][c][b] = sum_q w phi_a phi_c dphi_b/dr
//   D[r][j][a]    = sum_q w psi_j dphi_a/dr
//   M[a][b]       = sum_q w phi_a phi_b
// plus the rule itself and the P2 values at its nodes for the sources.
constexpr int TET_MAXQ = 64;
struct RefTensorsTet {
  double K[3][3][10][10];
  double T[3][10][10][10];
  double D[3][4][10];
  double M[10][10];
  int nq;
  double qw[TET_MAXQ], qr[TET_MAXQ], qs[TET_MAXQ], qt[TET_MAXQ];
  double phi[TET_MAXQ][10];
  // The rule as float pairs (hi + lo, lo = the double minus hi) for the
  // double-float residual: weights, P2 values and reference gradients
  // (dphi[q][r][a] = d phi_a / d r_r at node q), P1 values.
  float qwh[TET_MAXQ], qwl[TET_MAXQ];
  float phih[TET_MAXQ][10], phil[TET_MAXQ][10];
  float dphih[TET_MAXQ][3][10], dphil[TET_MAXQ][3][10];
  float psih[TET_MAXQ][4], psil[TET_MAXQ][4];
};
// The double-float tetrahedral residual keeps every node's terms in shared
// memory: rules of up to this many nodes (degree 6; higher degrees use the
// FP64 kernel).
constexpr int TET_DF_MAXQ = 24;

// Reference-element tensors of one quadrature rule (all sums over the rule's
// nodes, weights included):
//   K[r][s][a][b] = sum_q w dphi_a/dr dphi_b/ds
//   T[r][a][c][b] = sum_q w phi_a phi_c dphi_b/dr
//   D[r][j][a]    = sum_q w psi_j dphi_a/dr        (psi: P1, phi: P2)
//   M[a][b]       = sum_q w phi_a phi_b
// with r,s in {r,s} reference directions, a,b,c P2 and j P1 functions.
struct RefTensors {
  double K[2][2][6][6];
  double T[2][6][6][6];
  double D[2][3][6];
  double M[6][6];
  int nq;
  double qw[16], qr[16], qs[16];  // the rule, for non-polynomial sources
  double phi[16][6];              // P2 functions at the nodes
  // A 7-node rule exact to degree 5 (every polynomial integrand of the
  // residual on affine triangles has degree <= 5).  Used when the rule above
  // is itself exact to degree 5 (exact5), so both give the exact integrals.
  int exact5;
  double w5[7], phi5[7][6], dr5[7][6], ds5[7][6], psi5[7][3];
  // The same 7-node rule as float pairs (hi + lo, lo = the double minus hi
  // rounded to float) for the double-float residual.
  float w5h[7], w5l[7], phi5h[7][6], phi5l[7][6], dr5h[7][6], dr5l[7][6], ds5h[7][6], ds5l[7][6];
  float psi5h[7][3], psi5l[7][3];
};

// Constant coefficients of the fused forms (0 = form absent).
struct FormCoeffs {
  int elemType;     // 1 scalar P2, 2 Taylor-Hood P2-P1
  double diff;      // DIFFUSION coefficient
  double conv;      // VECTOR_CONVECTIVE_ACCELERATION coefficient
  double sigma;     // DIV_NEWTONIAN_STRESS coefficient
  double mu;        // DIV_NEWTONIAN_STRESS viscosity
  double divu;      // MIXED_DIVERGENCE coefficient
  double mass;      // TRANSIENT_VECTOR_MASS coefficient
  int hasSigma, hasDivu, hasConv, hasMass, hasDiff;
  int srcKind;      // SourceKind of SOURCE / VECTOR_SOURCE
  double srcParam[4];
  double srcCoeff;  // multiplies the source (1 when present)
  // conv, mass, sigma, mu, divu as float pairs (hi, lo) for the
  // double-float residual
  float pair[5][2];
};

// Colors of an element coloring (tetrahedral meshes need more than triangles).
constexpr int MAX_COLORS = 256;

struct DeviceMesh {
  int64_t nElm = 0;
  int nloc = 0;
  int nColors = 0;
  int64_t colorOff[MAX_COLORS + 1];
  int32_t *adr = nullptr;    // [nloc][nElm]  global DOF per local DOF, color order
  double *geo = nullptr;     // [5][nElm]     G00 G01 G10 G11 |J|   (G[r][k] = d r / d x_k)
                             // tetrahedra: [10][nElm] G[3][3] row-major, J
  double *xy = nullptr;      // [6][nElm]     x0 y0 x1 y1 x2 y2 (tetrahedra: [12][nElm] x0 y0 z0 ... z3)
  int32_t *map = nullptr;    // [nloc*nloc][nElm] CSR position or -1
  float2 *geoPair = nullptr; // [5][nElm] geo as float pairs (double-float residual; tetrahedra [10][nElm])
};

// Row-owned Jacobian assembly of Taylor-Hood systems: one thread builds one
// CSR row from the (element, local row) entries whose DOF is that row, in
// color order of the elements, inside a shared-memory copy of its block's
// contiguous range of CSR values, which the block then writes once.  No
// atomics, no element-to-nonzero map; each value is the same sum, in the
// same order, as the colored scatter.
// Units: a velocity node's two component rows together when they hold the
// same columns (one thread builds both, sharing the element terms), else one
// row.
struct RowAsm {
  int nBlocks = 0;
  int capBytes = 0;               // dynamic shared memory of a block
  int32_t *blockUnits = nullptr;  // [nBlocks + 1] first unit of each block
  int32_t *unitRow = nullptr;     // [nUnits + 1] first row of each unit (the last entry: nInc)
  int8_t *unitTwo = nullptr;      // [nUnits] 1: rows r (component 0) and r + 1 (component 1)
  int32_t *rowPtr = nullptr;      // [nInc + 1] entries of each row
  int32_t *rowEnt = nullptr;      // [nEnt] p * 16 + local row (p: color-order element)
  uint8_t *offs = nullptr;        // [nEnt][16] column offset in the row of each local column (255: none)
  void *pack = nullptr;           // [nElm][20] per element: u at the 12 velocity DOFs, G (4), J
  const int32_t *ia = nullptr;    // CSR row pointers
};
constexpr int ROWASM_PACK = 20;

// Row-owned FP32 Jacobian of tetrahedral Taylor-Hood systems: one warp per
// unit -- the three component rows of a velocity node (rows r, r + 1, r + 2,
// which hold the same columns and the same elements), or one pressure row --
// sums the element-matrix rows of the elements holding its DOF, in color
// order, inside a shared-memory copy of its block's contiguous range of CSR
// values, which the block then writes once.  Lane (m, b) of a velocity unit
// forms the three columns (b, n) of row m; the element's packed data (u at
// the 30 velocity DOFs, G, J) and the entry's column offsets are staged per
// warp.  No atomics and no element-to-nonzero map at assembly time.
struct RowAsmTet {
  int nBlocks = 0;
  int capBytes = 0;               // row values of a block in shared memory
  int32_t *blockUnits = nullptr;  // [nBlocks + 1] first unit of each block
  int32_t *unitRow = nullptr;     // [nUnits + 1] first row of each unit (the last entry: nInc)
  int8_t *unitKind = nullptr;     // [nUnits] 3: velocity node (three rows), 1: pressure row
  int32_t *unitPtr = nullptr;     // [nUnits + 1] entries of each unit
  int32_t *ent = nullptr;         // [nEnt] p * 64 + local DOF of the unit's first row (3 a, or 30 + j)
  uint8_t *offs = nullptr;        // [nEnt][ROWTET_OFFS] offset of local column j in the row (255: none)
  float *pack = nullptr;          // [nElm][ROWTET_PACK] u at the 30 velocity DOFs, G[3][3], J
  const int32_t *ia = nullptr;    // CSR row pointers
};
constexpr int ROWTET_PACK = 40;
constexpr int ROWTET_OFFS = 40;

void launch_pack_tet_f32(const DeviceMesh &dm, const FormCoeffs &fc, const double *u, float *pack, cudaStream_t s);
// Column offsets of every entry from the element-to-nonzero map: entry k
// (ent[k], first row entRow[k]) gets map[(li * 34 + j) * nElm + p] - ia[row].
void launch_rowtet_offsets(int64_t nEnt, const int32_t *ent, const int32_t *entRow, const int32_t *map,
                           int64_t nElm, const int32_t *ia, uint8_t *offs, cudaStream_t s);
void launch_matrix_tet_rows_f32(const RowAsmTet &ra, const FormCoeffs &fc, const RefTensorsTet *dT, double c0,
                                float *values, int accumulate, cudaStream_t s);

// Per-element data of the row-owned assembly (RowAsm::pack), from u.
void launch_pack_th_f32(const DeviceMesh &dm, const FormCoeffs &fc, const double *u, float *pack, cudaStream_t s);
void launch_pack_th_f64(const DeviceMesh &dm, const FormCoeffs &fc, const double *u, double *pack, cudaStream_t s);
// Row-owned Taylor-Hood Jacobian; accumulate = 0 overwrites the values
// (the matrix was zeroed), 1 adds to them.
void launch_matrix_th_rows_f32(const RowAsm &ra, const FormCoeffs &fc, const RefTensors *dT, double c0,
                               float *values, int accumulate, cudaStream_t s);
void launch_matrix_th_rows_f64(const RowAsm &ra, const FormCoeffs &fc, const RefTensors *dT, double c0,
                               double *values, int accumulate, cudaStream_t s);

// Residual (FP64) of the fused forms on elements [begin,end) of the color
// order, accumulated into rhs with feNG's sign (rhs = sum of element Be).
// exact5: the rule integrates degree 5 exactly (RefTensors::exact5), so the
// Taylor-Hood residual may use the 7-node quadrature kernel.
// dfloat: the Taylor-Hood 7-node kernel in double-float arithmetic (pairs of
// floats, ~44-bit significands, on the FP32 pipes) instead of FP64.
void launch_assemble_residual(const DeviceMesh &dm, const FormCoeffs &fc, const RefTensors *dT,
                              const double *u, const double *udot, double t, int64_t nInc,
                              double *rhs, int64_t begin, int64_t end, cudaStream_t s, int exact5);
// The Taylor-Hood 7-node residual in double-float arithmetic (pairs of
// floats, ~44-bit significands, on the FP32 pipes) from u and u-dot split
// into float pairs (launch_split_pairs) and dm.geoPair.
void launch_assemble_residual_df(const DeviceMesh &dm, const FormCoeffs &fc, const RefTensors *dT,
                                 const float2 *uPair, const float2 *udotPair, double t, int64_t nInc,
                                 double *rhs, int64_t begin, int64_t end, cudaStream_t s);
// out[i] = (hi, lo) of x[i]: hi = x rounded to float, lo = the rest rounded.
void launch_split_pairs(int64_t n, const double *x, float2 *out, cudaStream_t s);
// Jacobian of the fused forms, in double or float.
void launch_assemble_matrix_f64(const DeviceMesh &dm, const FormCoeffs &fc, const RefTensors *dT,
                                const double *u, double c0, double *values, int64_t begin,
                                int64_t end, cudaStream_t s);
void launch_assemble_matrix_f32(const DeviceMesh &dm, const FormCoeffs &fc, const RefTensors *dT,
                                const double *u, double c0, float *values, int64_t begin,
                                int64_t end, cudaStream_t s);

// Tetrahedra (fe_assembly_tet.cu): residual (FP64) and Jacobian (FP64 or
// FP32) of the fused forms on elements [begin, end) of the color order, the
// Jacobian scattered through the element-to-nonzero map (dm.map); scalar P2
// (DIFFUSION + SOURCE) or Taylor-Hood P2-P1 (the vector forms).
void build_ref_tensors_tet(const QuadRule &q, RefTensorsTet &T);
void launch_assemble_residual_tet(const DeviceMesh &dm, const FormCoeffs &fc, const RefTensorsTet *dT,
                                  const double *u, const double *udot, int64_t nInc, double *rhs,
                                  int64_t begin, int64_t end, cudaStream_t s);
// The Taylor-Hood residual in double-float from float pairs of u, u-dot and
// the geometry (dm.geoPair), rules of at most TET_DF_MAXQ nodes (nq).
void launch_assemble_residual_tet_df(const DeviceMesh &dm, const FormCoeffs &fc, const RefTensorsTet *dT, int nq,
                                     const float2 *up, const float2 *udp, int64_t nInc, double *rhs, int64_t begin,
                                     int64_t end, cudaStream_t s);
void launch_assemble_matrix_tet_f64(const DeviceMesh &dm, const FormCoeffs &fc, const RefTensorsTet *dT,
                                    const double *u, double c0, double *values, int64_t begin, int64_t end,
                                    cudaStream_t s);
void launch_assemble_matrix_tet_f32(const DeviceMesh &dm, const FormCoeffs &fc, const RefTensorsTet *dT,
                                    const double *u, double c0, float *values, int64_t begin, int64_t end,
                                    cudaStream_t s);
// Element-to-nonzero map on the device: map[(i nloc + j) nElm + p] = CSR
// position of (adr[i][p], adr[j][p]) (binary search in the row), -1 where
// either DOF is essential or the pair is outside mask [nloc*nloc]; *missing
// counts coupled pairs absent from the pattern (must stay 0).
void launch_build_map(const int32_t *adr, int64_t nElm, int nloc, const uint8_t *mask, const int32_t *ia,
                      const int32_t *ja, int64_t nInc, int32_t *map, unsigned long long *missing,
                      cudaStream_t s);

}  // namespace feng
