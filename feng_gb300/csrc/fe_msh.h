// ASCII Gmsh 4.1 parser shared by the triangle and tetrahedron readers: the
// nodes (in file order), the physical names, the entity -> physical tag map
// and the element blocks in file order (points, lines, triangles, tetrahedra).
#pragma once

#include <cstdint>
#include <map>
#include <string>
#include <vector>

namespace feng {

struct MshBlock {
  int dim = 0, tag = 0, type = 0;   // entity dimension and tag, gmsh element type
  std::vector<int32_t> nodes;       // 0-based vertex indices, npe per element
};

struct MshData {
  std::vector<double> x, y, z;
  std::map<std::pair<int, int>, std::string> physNames;  // (dim, physical tag) -> name
  std::map<std::pair<int, int>, int> entityPhys;          // (dim, entity tag) -> first physical tag
  std::vector<MshBlock> blocks;                           // file order

  // Physical name of an entity ("" when it has none).
  std::string name_of(int dim, int tag) const;
};

int read_msh41(const std::string &path, MshData &out);

}  // namespace feng
