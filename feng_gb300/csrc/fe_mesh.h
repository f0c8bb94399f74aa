// 2D triangle meshes made of P1 triangles, with the three named physical
// groups feNG's solvers address: the domain "Domaine", its boundary "Bord"
// (line elements) and an optional 0-D "PointPression" vertex used to pin the
// pressure.
//
// Vertex order is the order of the $Nodes section of a .msh file, and edges
// are numbered by first appearance while walking the triangles in file order,
// local edge k joining local vertices k and (k+1)%3.  This is exactly how
// feNG's reader tags edges (feMeshRead.cpp:1407-1453, set keyed by the
// unordered vertex pair, EdgeLessThan in feEdge.h:50-62), so DOF numbers and
// the CSR pattern built from this mesh coincide with the reference's.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace feng {

struct Mesh2D {
  // Vertices in file order.
  std::vector<double> x, y;
  // Triangles (counter-clockwise), 3 vertex indices each.
  std::vector<int32_t> tri;
  // Boundary line elements of "Bord", 2 vertex indices each, oriented like
  // the triangle edge they lie on.
  std::vector<int32_t> bnd;
  // Vertex of the "PointPression" group, or -1.
  int32_t point = -1;

  // Derived by build_topology():
  int32_t n_edges = 0;
  std::vector<int32_t> tri_edges;  // [nTri*3] 0-based edge index of local edge k
  std::vector<int32_t> edge_v;     // [nEdges*2] vertices of each edge (first-seen orientation)
  std::vector<int32_t> bnd_edges;  // [nBnd] edge index of each boundary line

  int64_t n_vertices() const { return (int64_t)x.size(); }
  int64_t n_triangles() const { return (int64_t)tri.size() / 3; }
  int64_t n_boundary() const { return (int64_t)bnd.size() / 2; }

  // Numbers the edges and checks that every boundary line is a triangle edge
  // with the same orientation (feMeshRead.cpp:1836-1870).
  int build_topology();
};

// Structured n x n grid on [x0,x1] x [y0,y1], each cell split into two
// counter-clockwise triangles by the diagonal from its lower-left to its
// upper-right corner: (v00, v10, v11) then (v00, v11, v01).  Vertices are
// numbered row by row.  Interior vertices are moved by independent uniform
// offsets in [-jitter*h, +jitter*h] in x and y, drawn from a SplitMix64
// stream seeded with `seed` (h = cell width along each axis).  "Bord" is the
// counter-clockwise boundary loop starting at (x0,y0); "PointPression" is the
// vertex at (x0,y0).
int mesh_generate_square(Mesh2D &m, int n, double x0, double x1, double y0, double y1,
                         double jitter, uint64_t seed);

// Writes the mesh as an ASCII Gmsh 4.1 file readable by feMesh2DP1.
int mesh_write_msh41(const Mesh2D &m, const std::string &path);

// Physical groups of a msh file that play the three roles of Mesh2D: the
// triangles of `domain`, the lines of every group in `boundary` (merged, in
// the file's entity order) and the vertex of `point` (empty: none).  feNG
// addresses groups by name (createFiniteElementSpace(..., cncGeoID, ...),
// src/feSpace.cpp:11-60); the defaults are the names its test meshes use.
struct MeshGroups {
  std::string domain = "Domaine";
  std::vector<std::string> boundary = {"Bord"};
  std::string point = "PointPression";
};

// Reads an ASCII Gmsh 4.1 file: the triangles of groups.domain (required),
// the lines of groups.boundary and the vertex of groups.point (optional).
int mesh_read_msh41(Mesh2D &m, const std::string &path, const MeshGroups &groups = MeshGroups());

}  // namespace feng
