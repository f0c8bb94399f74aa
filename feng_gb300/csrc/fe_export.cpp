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

int export_vtk(const Mesh2D &m, const Numbering &num, const double *solution,
               const std::vector<ExportField> &fields, int precision, const std::string &path)
{
  if(!solution) { set_error("null solution"); return FE_INVALID_ARG; }
  if(precision < 1 || precision > 17) {
    set_error("precision %d outside 1..17", precision);
    return FE_INVALID_ARG;
  }
  if(fields.empty()) { set_error("no field to export"); return FE_INVALID_ARG; }
  const int64_t nv = m.n_vertices(), nt = m.n_triangles(), ne = m.n_edges;
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
      const int64_t a = m.edge_v[2 * (size_t)e], b = m.edge_v[2 * (size_t)e + 1];
      return (std::min(a, b) << 32) | std::max(a, b);
    };
    std::sort(edgeOrder.begin(), edgeOrder.end(), [&](int32_t p, int32_t q) { return key(p) < key(q); });
    edgeNode.resize((size_t)ne);
    for(int64_t k = 0; k < ne; ++k) edgeNode[(size_t)edgeOrder[(size_t)k]] = nv + k;
  }
  const int64_t nNodes = nv + (quadratic ? ne : 0);
  const int nodesPerCell = quadratic ? 6 : 3;

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
    double x, y;
    if(i < nv) {
      x = m.x[(size_t)i];
      y = m.y[(size_t)i];
    } else {
      const int32_t e = edgeOrder[(size_t)(i - nv)];
      const int32_t a = m.edge_v[2 * (size_t)e], b = m.edge_v[2 * (size_t)e + 1];
      x = (m.x[a] + m.x[b]) / 2.;
      y = (m.y[a] + m.y[b]) / 2.;
    }
    put(s, x, precision, ' ');
    put(s, y, precision, ' ');
    put(s, 0.0, precision, '\n');
  });
  fprintf(f, "CELLS %lld %lld\n", (long long)nt, (long long)nt * (nodesPerCell + 1));
  ok &= write_rows(f, nt, [&](int64_t t, std::string &s) {
    put_int(s, nodesPerCell, ' ');
    for(int j = 0; j < 3; ++j) put_int(s, m.tri[3 * (size_t)t + j], ' ');
    if(quadratic)
      for(int k = 0; k < 3; ++k) put_int(s, edgeNode[(size_t)m.tri_edges[3 * (size_t)t + k]], ' ');
    s.push_back('\n');
  });
  fprintf(f, "CELL_TYPES %lld\n", (long long)nt);
  ok &= write_rows(f, nt, [&](int64_t, std::string &s) { s.append(quadratic ? "22\n" : "5\n"); });
  fprintf(f, "POINT_DATA %lld\nFIELD FieldData %zu\n", (long long)nNodes, fields.size());
  for(const ExportField &fd : fields) {
    const int C = num.fieldComp[fd.field];
    const int W = C > 1 ? 3 : 1;  // 2-vectors are written with three components
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
              const int32_t a = m.edge_v[2 * (size_t)e], b = m.edge_v[2 * (size_t)e + 1];
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

}  // namespace feng
