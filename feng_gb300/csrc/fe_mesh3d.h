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
};

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

}  // namespace feng
