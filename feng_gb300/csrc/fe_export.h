// Legacy VTK export of a solution vector on the host, in the layout of feNG's
// feExporterVTK::writeStep (src/feExporter.cpp:854-990, continuous fields on
// a P1 triangle mesh):
//
//   header "# vtk DataFile Version 4.2" / "test output" / "ASCII";
//   DATASET UNSTRUCTURED_GRID with the mesh vertices in file order, followed,
//   when a field is P2, by one node per edge at its midpoint, the edges taken
//   in ascending (min vertex, max vertex) order (feMesh::_edges is a set
//   ordered by EdgeLessThan, src/feEdge.h:50-62);
//   CELLS: per triangle "6 v0 v1 v2 e01 e12 e20 " (VTK_QUADRATIC_TRIANGLE, 22)
//   or "3 v0 v1 v2 " (VTK_TRIANGLE, 5) when every field is P1;
//   POINT_DATA / FIELD FieldData: per field its name, 1 or 3 components
//   (2-vectors padded with a zero third component) and one value per line.
//
// Values: at a vertex the field's DOF there; at an edge midpoint the P2
// field's edge DOF (the reference evaluates the interpolant at the located
// midpoint, which is that DOF up to rounding) or, for a P1 field, the mean of
// the two vertex values (the P1 interpolant there).  Values below 1e-20 in
// magnitude are written as 0 where the reference does so: at vertices, and at
// midpoints for scalar fields (src/feExporter.cpp:388-391, 416-419).  Numbers
// are printed as the reference's std::ostream default does (%.6g), or with
// more significant digits on request.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "fe_mesh.h"
#include "fe_mesh3d.h"
#include "fe_setup.h"

namespace feng {

struct ExportField {
  int field;          // field index of the numbering
  std::string name;   // name written to the file (feSpace fieldID)
  int degree;         // 1 or 2: degree of the field's space on the domain
};

// Writes `fields` in the given order.  `solution` holds every DOF (unknowns
// then essential DOFs, as feSolution).  precision: significant digits
// (1..17; the reference writes 6).
int export_vtk(const Mesh2D &m, const Numbering &num, const double *solution,
               const std::vector<ExportField> &fields, int precision, const std::string &path);

// The same file for a tetrahedral mesh, with the same rules for nodes and
// values (vertices, then edge midpoints in ascending vertex-pair order;
// 3-vectors written as they are).  Cells are VTK_QUADRATIC_TETRA (24, VTK's
// node order: vertices, then edges (0,1) (1,2) (0,2) (0,3) (1,3) (2,3)) or
// VTK_TETRA (10) when every field is P1.  The reference's exporter has no
// tetrahedral P2 layout (it writes 6-node triangle cells for any
// P2 field), so this one follows VTK's.
int export_vtk3d(const Mesh3D &m, const Numbering &num, const double *solution,
                 const std::vector<ExportField> &fields, int precision, const std::string &path);

}  // namespace feng
