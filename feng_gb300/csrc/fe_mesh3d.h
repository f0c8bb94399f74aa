// 3D tetrahedral meshes (P1 tetrahedra) with feNG's physical groups
// "Domaine" (tetrahedra) and "Bord" (boundary triangles), the layout of the
// reference's cube meshes (data/cube*.msh) and of the 3D configuration
// (unit cube, 6 tetrahedra per cell).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace feng {

struct Mesh3D {
  std::vector<double> x, y, z;   // vertices
  std::vector<int32_t> tet;      // [nTet*4], positive volume
  std::vector<int32_t> bnd;      // [nBnd*3] boundary triangles, normal pointing out

  int64_t n_vertices() const { return (int64_t)x.size(); }
  int64_t n_tets() const { return (int64_t)tet.size() / 4; }
  int64_t n_boundary() const { return (int64_t)bnd.size() / 3; }

  // Derived by build_topology():
  int64_t n_edges = 0;
  std::vector<int32_t> edge_v;     // [nEdges*2] vertices of each edge (first-seen orientation)
  std::vector<int32_t> tet_edges;  // [nTet*6] edge of local edge k, in TET_EDGES order
  std::vector<int32_t> bnd_edges;  // [nBnd*3] edge joining local vertices k and (k+1)%3

  // Numbers the edges in the order the reference's reader creates them for a
  // file holding the "Bord" triangles before the tetrahedra
  // (src/feMeshRead.cpp:1320-1345, 1481-1538): the edges (k, k+1) of each
  // boundary triangle, then, for each tetrahedron, the edges (0,1), (1,2),
  // (2,0) of its facets taken in TET_FACES order (Tetrahedron::createBoundary,
  // src/feTetrahedron.cpp:6-72).  Checks that every edge of a boundary
  // triangle is an edge of the tetrahedra.
  int build_topology();
};

// Facets and edges of a tetrahedron in the reference's local order
// (_facesOrder, _edgesOrder, src/feTetrahedron.h:30-31); edge k of a P2
// tetrahedron carries its local DOF 4 + k.
extern const int TET_FACES[4][3];
extern const int TET_EDGES[6][2];

// Structured n x n x n grid on the box, each cell split into the 6
// tetrahedra of the Kuhn (Freudenthal) triangulation: for each ordering
// (a, b, c) of the axes, in the order xyz, xzy, yxz, yzx, zxy, zyx, the
// tetrahedron v000, v000+e_a, v000+e_a+e_b, v111 (two vertices swapped for
// the odd orderings so that every volume is positive).  Every square face is
// then cut along the diagonal from its lowest to its highest corner, so the
// tetrahedra are conforming and each boundary square gives two "Bord"
// triangles.  Vertices are numbered x fastest, then y, then z; cells in the
// same order.  Interior vertices move by independent uniform offsets in
// [-jitter*h, +jitter*h] along each axis (x, y, z draws in vertex order,
// SplitMix64 seeded with `seed`, as the 2D generator).  Boundary triangles:
// faces x = x0, x = x1, y = y0, y = y1, z = z0, z = z1 in that order, squares
// in the order of their two in-plane indices, oriented outwards.
int mesh3d_generate_cube(Mesh3D &m, int n, const double box[6], double jitter, uint64_t seed);

// ASCII Gmsh 4.1 file: "Bord" (2 1, triangles), then "Domaine" (3 2,
// tetrahedra), all nodes in the volume's block.
int mesh3d_write_msh41(const Mesh3D &m, const std::string &path);

// Reads an ASCII Gmsh 4.1 file: the tetrahedra of the `domain` volumes and
// the triangles of the `boundary` surfaces, each in file order; nodes in
// file order.  Boundary triangles must precede the tetrahedra in the file
// (as Gmsh writes them), the order in which the edges are numbered.
int mesh3d_read_msh41(Mesh3D &m, const std::string &path, const std::string &domain = "Domaine",
                      const std::vector<std::string> &boundary = {"Bord"});

}  // namespace feng
