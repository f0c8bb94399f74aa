#include "fe_export.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <memory>

#include "fe_common.h"

namespace feng {

namespace {

// Magnitude below which the reference writes a value as 0 (TOL_ZERO_VTK,
// src/feExporter.cpp:13).
constexpr double kZeroTol = 1e-20;

inline double zeroed(double v) { return std::fabs(v) < kZeroTol ? 0.0 : v; }

inline void put(std::string &s, double v, int prec, char sep)
{
  char buf[48];
  const int n = snprintf(buf, sizeof buf, "%.*g", prec, v);
  s.append(buf, (size_t)n);
  s.push_back(sep);
}

inline void put_int(std::string &s, int64_t v, char sep)
{
  char buf[24];
  const int n = snprintf(buf, sizeof buf, "%lld", (long long)v);
  s.append(buf, (size_t)n);
  s.push_back(sep);
}

// Formats rows [0, n) in contiguous chunks on the host threads (row(i, s)
// appends row i to s) and writes the chunks to f in order.
template <typename Row>
bool write_rows(FILE *f, int64_t n, Row &&row)
{
  constexpr int64_t kRows = 1 << 15;
  const int64_t nChunks = (n + kRows - 1) / kRows;
  std::vector<std::string> parts((size_t)nChunks);
  parallel_for(
      nChunks,
      [&](int64_t cb, int64_t ce) {
        for(int64_t c = cb; c < ce; ++c) {
          std::string &s = parts[(size_t)c];
          s.reserve((size_t)kRows * 16);
          const int64_t e = std::min(n, (c + 1) * kRows);
          for(int64_t i = c * kRows; i < e; ++i) row(i, s);
        }
      },
      1);
  for(const std::string &s : parts)
    if(fwrite(s.data(), 1, s.size(), f) != s.size()) return false;
  return true;
}

}  // namespace

namespace {

// A P1 simplex mesh as the writer sees it.
struct MeshView {
  int64_t nv = 0, ne = 0, ncell = 0;
  int nvpc = 0, nepc = 0;              // vertices and edges per cell
  const double *x = nullptr, *y = nullptr, *z = nullptr;  // z: null in 2D
  const int32_t *cellV = nullptr;      // [ncell*nvpc]
  const int32_t *cellE = nullptr;      // [ncell*nepc] edges in the mesh's local order
  const int32_t *edgeV = nullptr;      // [ne*2]
  const int *vtkEdge = nullptr;        // VTK edge slot k -> local edge index
  int linearType = 0, quadType = 0;    // VTK cell types
};

int write_vtk(const MeshView &m, const Numbering &num, const double *solution,
              const std::vector<ExportField> &fields, int precision, const std::string &path)
{
  if(!solution) { set_error("null solution"); return FE_INVALID_ARG; }
  if(precision < 1 || precision > 17) {
    set_error("precision %d outside 1..17", precision);
    return FE_INVALID_ARG;
  }
  if(fields.empty()) { set_error("no field to export"); return FE_INVALID_ARG; }
  const int64_t nv = m.nv, nt = m.ncell, ne = m.ne;
  bool quadratic = false;
  for(const ExportField &fd : fields) {
    if(fd.field < 0 || fd.field >= num.nFields) {
      set_error("field %d does not exist", fd.field);
      return FE_INVALID_ARG;
    }
    if(fd.degree != 1 && fd.degree != 2) {
      set_error("field %d: only P1 and P2 fields on the domain can be exported", fd.field);
      return FE_INVALID_ARG;
    }
    if(fd.name.empty() || fd.name.find_first_of(" \t\n") != std::string::npos) {
      set_error("field %d: a field name must be one non-empty word", fd.field);
      return FE_INVALID_ARG;
    }
    const int C = num.fieldComp[fd.field];
    if((int64_t)num.vdof[fd.field].size() != nv * C || (int64_t)num.edof[fd.field].size() != ne * C) {
      set_error("the numbering was not built on this mesh");
      return FE_INVALID_ARG;
    }
    for(int64_t i = 0; i < nv * C; ++i)
      if(num.vdof[fd.field][i] < 0 || num.vdof[fd.field][i] >= num.nDofs) {
        set_error("field %d has no DOF at vertex %lld", fd.field, (long long)(i / C));
        return FE_INVALID_ARG;
      }
    if(fd.degree == 2)
      for(int64_t i = 0; i < ne * C; ++i)
        if(num.edof[fd.field][i] < 0 || num.edof[fd.field][i] >= num.nDofs) {
          set_error("field %d has no DOF on edge %lld", fd.field, (long long)(i / C));
          return FE_INVALID_ARG;
        }
    quadratic |= fd.degree == 2;
  }

  // Visualisation node of each edge: after the vertices, edges in ascending
  // (min vertex, max vertex) order.
  std::vector<int64_t> edgeNode;
  std::vector<int32_t> edgeOrder;
  if(quadratic) {
    edgeOrder.resize((size_t)ne);
    for(int64_t e = 0; e < ne; ++e) edgeOrder[(size_t)e] = (int32_t)e;
    auto key = [&](int32_t e) {
      const int64_t a = m.edgeV[2 * (size_t)e], b = m.edgeV[2 * (size_t)e + 1];
      return (std::min(a, b) << 32) | std::max(a, b);
    };
    std::sort(edgeOrder.begin(), edgeOrder.end(), [&](int32_t p, int32_t q) { return key(p) < key(q); });
    edgeNode.resize((size_t)ne);
    for(int64_t k = 0; k < ne; ++k) edgeNode[(size_t)edgeOrder[(size_t)k]] = nv + k;
  }
  const int64_t nNodes = nv + (quadratic ? ne : 0);
  const int nodesPerCell = m.nvpc + (quadratic ? m.nepc : 0);

  std::unique_ptr<FILE, int (*)(FILE *)> file(fopen(path.c_str(), "wb"), &fclose);
  if(!file) {
    set_error("cannot open %s for writing", path.c_str());
    return FE_READ_ERROR;
  }
  FILE *f = file.get();
  bool ok = true;
  fprintf(f, "# vtk DataFile Version 4.2\ntest output\nASCII\n");
  fprintf(f, "DATASET UNSTRUCTURED_GRID\nPOINTS %lld double\n", (long long)nNodes);
  ok &= write_rows(f, nNodes, [&](int64_t i, std::string &s) {
    double x, y, z;
    if(i < nv) {
      x = m.x[i];
      y = m.y[i];
      z = m.z ? m.z[i] : 0.0;
    } else {
      const int32_t e = edgeOrder[(size_t)(i - nv)];
      const int32_t a = m.edgeV[2 * (size_t)e], b = m.edgeV[2 * (size_t)e + 1];
      x = (m.x[a] + m.x[b]) / 2.;
      y = (m.y[a] + m.y[b]) / 2.;
      z = m.z ? (m.z[a] + m.z[b]) / 2. : 0.0;
    }
    put(s, x, precision, ' ');
    put(s, y, precision, ' ');
    put(s, z, precision, '\n');
  });
  fprintf(f, "CELLS %lld %lld\n", (long long)nt, (long long)nt * (nodesPerCell + 1));
  ok &= write_rows(f, nt, [&](int64_t t, std::string &s) {
    put_int(s, nodesPerCell, ' ');
    for(int j = 0; j < m.nvpc; ++j) put_int(s, m.cellV[(size_t)t * m.nvpc + j], ' ');
    if(quadratic)
      for(int k = 0; k < m.nepc; ++k) put_int(s, edgeNode[(size_t)m.cellE[(size_t)t * m.nepc + m.vtkEdge[k]]], ' ');
    s.push_back('\n');
  });
  fprintf(f, "CELL_TYPES %lld\n", (long long)nt);
  const std::string type = std::to_string(quadratic ? m.quadType : m.linearType) + "\n";
  ok &= write_rows(f, nt, [&](int64_t, std::string &s) { s.append(type); });
  fprintf(f, "POINT_DATA %lld\nFIELD FieldData %zu\n", (long long)nNodes, fields.size());
  for(const ExportField &fd : fields) {
    const int C = num.fieldComp[fd.field];
    const int W = C > 1 ? 3 : 1;  // vectors are written with three components
    const std::vector<int64_t> &vd = num.vdof[fd.field], &ed = num.edof[fd.field];
    fprintf(f, "%s %d %lld double\n", fd.name.c_str(), W, (long long)nNodes);
    ok &= write_rows(f, nNodes, [&](int64_t i, std::string &s) {
      for(int c = 0; c < W; ++c) {
        double v = 0.0;
        if(c < C) {
          if(i < nv) {
            v = zeroed(solution[vd[(size_t)i * C + c]]);
          } else {
            const int32_t e = edgeOrder[(size_t)(i - nv)];
            if(fd.degree == 2) {
              v = solution[ed[(size_t)e * C + c]];
            } else {
              const int32_t a = m.edgeV[2 * (size_t)e], b = m.edgeV[2 * (size_t)e + 1];
              v = 0.5 * solution[vd[(size_t)a * C + c]] + 0.5 * solution[vd[(size_t)b * C + c]];
            }
            // The reference's interpolant is a sum started from +0, so a
            // zero value is written unsigned.
            v += 0.0;
            if(C == 1) v = zeroed(v);
          }
        }
        put(s, v, precision, '\n');
      }
    });
  }
  if(!ok || ferror(f)) {
    set_error("write error on %s", path.c_str());
    return FE_READ_ERROR;
  }
  return FE_OK;
}

}  // namespace

int export_vtk(const Mesh2D &m, const Numbering &num, const double *solution,
               const std::vector<ExportField> &fields, int precision, const std::string &path)
{
  static const int triEdges[3] = {0, 1, 2};  // local edge k joins k and (k+1)%3, VTK's order
  MeshView v;
  v.nv = m.n_vertices(); v.ne = m.n_edges; v.ncell = m.n_triangles();
  v.nvpc = 3; v.nepc = 3;
  v.x = m.x.data(); v.y = m.y.data();
  v.cellV = m.tri.data(); v.cellE = m.tri_edges.data(); v.edgeV = m.edge_v.data();
  v.vtkEdge = triEdges;
  v.linearType = 5;   // VTK_TRIANGLE
  v.quadType = 22;    // VTK_QUADRATIC_TRIANGLE
  return write_vtk(v, num, solution, fields, precision, path);
}

int export_vtk3d(const Mesh3D &m, const Numbering &num, const double *solution,
                 const std::vector<ExportField> &fields, int precision, const std::string &path)
{
  // VTK edge slots (0,1) (1,2) (0,2) (0,3) (1,3) (2,3) in TET_EDGES terms:
  // (1,0) is edge 2, (2,1) edge 1, (0,2) edge 0, (3,0) edge 4, (1,3) edge 3, (3,2) edge 5.
  static const int tetEdges[6] = {2, 1, 0, 4, 3, 5};
  MeshView v;
  v.nv = m.n_vertices(); v.ne = m.n_edges; v.ncell = m.n_tets();
  v.nvpc = 4; v.nepc = 6;
  v.x = m.x.data(); v.y = m.y.data(); v.z = m.z.data();
  v.cellV = m.tet.data(); v.cellE = m.tet_edges.data(); v.edgeV = m.edge_v.data();
  v.vtkEdge = tetEdges;
  v.linearType = 10;  // VTK_TETRA
  v.quadType = 24;    // VTK_QUADRATIC_TETRA
  return write_vtk(v, num, solution, fields, precision, path);
}

}  // namespace feng
