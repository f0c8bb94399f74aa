// Host-side set-up of one finite element problem: quadrature, DOF numbering,
// element-to-DOF tables, element coloring, the CSR sparsity pattern and the
// element-to-nonzero scatter map consumed by the device assembly kernels.
//
// Each piece restates the reference algorithm it must agree with:
//   numbering      feMetaNumber ctor, feNumber::numberUnknowns/numberEssential
//                  (feNumber.cpp:370-480, 677-835)
//   element DOFs   feSpaceTriP2 / feSpaceVecTriP2 / feSpaceTriP1
//                  ::initializeAddressingVector (feSpace_2D.cpp:154-159,
//                  772-784, 1018-1040) concatenated along the fields layout
//                  (feBilinearForm.cpp:250-274)
//   coloring       feCncGeo::colorElements(1) (feCncGeo.cpp:735-790)
//   CSR pattern    feEZCompressedRowStorage (feCompressedRowStorage.cpp:15-135)
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "fe_mesh.h"
#include "fe_mesh3d.h"

namespace feng {

struct QuadRule {
  int degree = 0;
  std::vector<double> r, s, w;
  std::vector<double> t;  // third reference coordinate (tetrahedral rules only)
  int n() const { return (int)w.size(); }
};
int triangle_rule(int degree, QuadRule &q);
// Fully symmetric rules on the reference tetrahedron (0,0,0)-(1,0,0)-(0,1,0)-
// (0,0,1), weights summing to 1/6, degrees 1 to 8 with the orbit structure of
// the reference's rules (getGQTetPts, src/feQuadratureTet.cpp:3342): number
// of points 1, 4, 5, 11, 14, 24, 31, 43.
int tet_rule(int degree, QuadRule &q);

// Geometric connectivities a space can live on.
enum Cnc : int { CNC_DOMAIN = 0, CNC_BOUNDARY = 1, CNC_POINT = 2 };

struct SpaceDesc {
  int field;      // index of the field, in order of first appearance
  int degree;     // Lagrange degree: 0 (point), 1 or 2
  int ncomp;      // 1 scalar, 2 vector (interleaved components)
  int cnc;        // Cnc
  int essential;  // listed among the essential spaces
};

// Element types of the fused device kernels.
enum ElemType : int {
  ELEM_P2 = 1,            // scalar P2 triangle, 6 local DOFs
  ELEM_TAYLOR_HOOD = 2,   // vector P2 (interleaved) + scalar P1, 12 + 3 local DOFs
  ELEM_TET_P2 = 3,        // scalar P2 tetrahedron, 4 vertex + 6 edge DOFs
  ELEM_TET_TAYLOR_HOOD = 4,  // 3-vector P2 (interleaved) + scalar P1, 30 + 4 local DOFs
};

struct Numbering {
  int64_t nInc = 0, nDofs = 0;
  int nFields = 0;
  std::vector<int> fieldComp;                  // components of each field
  std::vector<std::vector<int64_t>> vdof;      // [field][vertex*comp + c]  (-1: none)
  std::vector<std::vector<int64_t>> edof;      // [field][edge*comp + c]
  // Physical location and field/component of every DOF.
  std::vector<double> dof_x, dof_y, dof_z;  // dof_z: tetrahedral meshes only
  std::vector<int32_t> dof_field, dof_comp;
  std::vector<uint8_t> dof_is_vertex;
};

int build_numbering(const Mesh2D &m, const std::vector<SpaceDesc> &spaces, Numbering &num);

struct ElementTables {
  int type = 0;
  int nloc = 0;                      // local DOFs per element
  int64_t nElm = 0;
  std::vector<int64_t> adr;          // [nElm*nloc] global DOF of each local DOF
  std::vector<uint8_t> mask;         // [nloc*nloc] local (i,j) coupled by a matrix form
};

// Builds the fused element DOF tables for a scalar P2 field (ELEM_P2) or a
// (vector P2 velocity, P1 pressure) pair (ELEM_TAYLOR_HOOD).
int build_element_tables(const Mesh2D &m, const Numbering &num, int type, int fieldU, int fieldP,
                         ElementTables &et);

struct Coloring {
  int nColors = 0;
  std::vector<int32_t> elm_color;    // [nElm]
  std::vector<int64_t> offsets;      // [nColors+1]
  std::vector<int32_t> elements;     // elements listed color by color, ascending within a color
};

// feCncGeo::colorElements(1) (src/feCncGeo.cpp:735) on elements given by
// nvpe vertices each (ev [ne*nvpe]): triangles or tetrahedra.
int color_by_vertices(const int32_t *ev, int nvpe, int64_t ne, int64_t nv, int maxColors, Coloring &col);
int color_elements(const Mesh2D &m, Coloring &col);
// Checks that no two elements of one color share a vertex.
int validate_coloring(const Mesh2D &m, const Coloring &col);

// Tetrahedral meshes.  The numbering restates feMetaNumber for spaces on
// "Domaine" (tetrahedra, feSpaceTetPn) and "Bord" (triangles): per pass
// (unknown DOFs, then essential DOFs) and per field, the vertices in index
// order, then the edges in Mesh3D::build_topology order, components
// interleaved (src/feNumber.cpp:677-835, the same rule as on triangles).
int build_numbering3d(const Mesh3D &m, const std::vector<SpaceDesc> &spaces, Numbering &num);
// ELEM_TET_P2: 4 vertex DOFs then the 6 edge DOFs in TET_EDGES order
// (feSpaceTetPn::initializeAddressingVector, src/feSpace_3D.cpp:293-320).
// ELEM_TET_TAYLOR_HOOD: velocity node k (vertices, then edges) component c at
// 3k + c, pressure vertex j at 30 + j.
int build_element_tables3d(const Mesh3D &m, const Numbering &num, int type, int fieldU, int fieldP,
                           ElementTables &et);
int color_elements3d(const Mesh3D &m, Coloring &col);

struct CSRPattern {
  int64_t n = 0;
  std::vector<int64_t> ia;           // [n+1]
  std::vector<int32_t> ja;           // [nnz], ascending within each row
  int64_t nnz() const { return ia.empty() ? 0 : ia.back(); }
};

int build_csr_pattern(const ElementTables &et, int64_t nInc, CSRPattern &pat);
// The same pattern built on the current CUDA device (fe_pattern.cu).
int build_csr_pattern_device(const ElementTables &et, int64_t nInc, CSRPattern &pat);
// Where set-ups build their pattern: -1 on the device when one is present
// (the default; the host when a row exceeds the device path's capacity),
// 0 on the host, 1 on the device.
int set_pattern_mode(int mode);
int pattern_mode();
// The pattern by the current mode; *onDevice (may be NULL) tells which ran.
int build_csr_pattern_auto(const ElementTables &et, int64_t nInc, CSRPattern &pat, int *onDevice);

// For each element (in coloring order) and each coupled local pair (i,j), the
// position of (adr_i, adr_j) in the CSR arrays, or -1 when either DOF is
// essential.  Layout [nloc*nloc][nElm] so that consecutive elements of a
// color read consecutive words.
int build_scatter_map(const ElementTables &et, const Coloring &col, const CSRPattern &pat,
                      int64_t nInc, std::vector<int32_t> &map);

}  // namespace feng
