#include "fe_mesh.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <fstream>
#include <map>
#include <sstream>
#include <unordered_map>

#include "fe_common.h"
#include "fe_msh.h"

namespace feng {

int Mesh2D::build_topology()
{
  const int64_t nt = n_triangles();
  const int64_t nv = n_vertices();
  tri_edges.assign(nt * 3, -1);
  edge_v.clear();
  n_edges = 0;
  // Per-vertex list of (neighbour with larger index, edge id).
  std::vector<std::vector<std::pair<int32_t, int32_t>>> adj(nv);
  for(int64_t t = 0; t < nt; ++t) {
    for(int k = 0; k < 3; ++k) {
      int32_t a = tri[3 * t + k], b = tri[3 * t + (k + 1) % 3];
      if(a < 0 || b < 0 || a >= nv || b >= nv) {
        set_error("triangle %lld references vertex out of range", (long long)t);
        return FE_INVALID_ARG;
      }
      int32_t lo = std::min(a, b), hi = std::max(a, b);
      int32_t id = -1;
      for(auto &p : adj[lo])
        if(p.first == hi) { id = p.second; break; }
      if(id < 0) {
        id = n_edges++;
        adj[lo].push_back({hi, id});
        edge_v.push_back(a);
        edge_v.push_back(b);
      }
      tri_edges[3 * t + k] = id;
    }
  }
  const int64_t nb = n_boundary();
  bnd_edges.assign(nb, -1);
  for(int64_t i = 0; i < nb; ++i) {
    int32_t a = bnd[2 * i], b = bnd[2 * i + 1];
    int32_t lo = std::min(a, b), hi = std::max(a, b);
    int32_t id = -1;
    for(auto &p : adj[lo])
      if(p.first == hi) { id = p.second; break; }
    if(id < 0) {
      set_error("boundary line (%d,%d) is not an edge of the triangulation", a, b);
      return FE_INVALID_ARG;
    }
    if(edge_v[2 * id] != a) {
      set_error("boundary line (%d,%d) is oriented against its triangle", a, b);
      return FE_INVALID_ARG;
    }
    bnd_edges[i] = id;
  }
  return FE_OK;
}

int mesh_generate_square(Mesh2D &m, int n, double x0, double x1, double y0, double y1,
                         double jitter, uint64_t seed)
{
  if(n < 1 || !(x1 > x0) || !(y1 > y0) || jitter < 0 || jitter >= 0.5) {
    set_error("invalid square mesh parameters (n=%d, jitter=%g)", n, jitter);
    return FE_INVALID_ARG;
  }
  const int nv1 = n + 1;
  const double hx = (x1 - x0) / n, hy = (y1 - y0) / n;
  m = Mesh2D();
  m.x.resize((size_t)nv1 * nv1);
  m.y.resize((size_t)nv1 * nv1);
  SplitMix64 rng(seed);
  for(int j = 0; j <= n; ++j) {
    for(int i = 0; i <= n; ++i) {
      size_t v = (size_t)j * nv1 + i;
      // Exact endpoints on the boundary, no rounding drift from x0 + i*h.
      double x = (i == n) ? x1 : x0 + i * hx;
      double y = (j == n) ? y1 : y0 + j * hy;
      if(i > 0 && i < n && j > 0 && j < n && jitter > 0) {
        // Two draws per interior vertex, x first, in row-major order.
        x += jitter * hx * rng.uniform_pm1();
        y += jitter * hy * rng.uniform_pm1();
      }
      m.x[v] = x;
      m.y[v] = y;
    }
  }
  m.tri.reserve((size_t)n * n * 6);
  for(int j = 0; j < n; ++j) {
    for(int i = 0; i < n; ++i) {
      int32_t v00 = j * nv1 + i, v10 = v00 + 1, v01 = v00 + nv1, v11 = v01 + 1;
      m.tri.insert(m.tri.end(), {v00, v10, v11, v00, v11, v01});
    }
  }
  // Counter-clockwise boundary loop: bottom, right, top, left.
  for(int i = 0; i < n; ++i) m.bnd.insert(m.bnd.end(), {i, i + 1});
  for(int j = 0; j < n; ++j) m.bnd.insert(m.bnd.end(), {j * nv1 + n, (j + 1) * nv1 + n});
  for(int i = n; i > 0; --i) m.bnd.insert(m.bnd.end(), {n * nv1 + i, n * nv1 + i - 1});
  for(int j = n; j > 0; --j) m.bnd.insert(m.bnd.end(), {j * nv1, (j - 1) * nv1});
  m.point = 0;
  return m.build_topology();
}

int mesh_write_msh41(const Mesh2D &m, const std::string &path)
{
  FILE *f = fopen(path.c_str(), "w");
  if(!f) {
    set_error("cannot open %s for writing", path.c_str());
    return FE_READ_ERROR;
  }
  const int64_t nv = m.n_vertices(), nt = m.n_triangles(), nb = m.n_boundary();
  double xmin = 1e300, xmax = -1e300, ymin = 1e300, ymax = -1e300;
  for(int64_t v = 0; v < nv; ++v) {
    xmin = std::min(xmin, m.x[v]); xmax = std::max(xmax, m.x[v]);
    ymin = std::min(ymin, m.y[v]); ymax = std::max(ymax, m.y[v]);
  }
  const bool hasPoint = m.point >= 0;
  fprintf(f, "$MeshFormat\n4.1 0 8\n$EndMeshFormat\n");
  fprintf(f, "$PhysicalNames\n%d\n", hasPoint ? 3 : 2);
  if(hasPoint) fprintf(f, "0 1 \"PointPression\"\n");
  fprintf(f, "1 2 \"Bord\"\n2 3 \"Domaine\"\n$EndPhysicalNames\n");
  fprintf(f, "$Entities\n%d 1 1 0\n", hasPoint ? 1 : 0);
  if(hasPoint) fprintf(f, "1 %.17g %.17g 0 1 1\n", m.x[m.point], m.y[m.point]);
  fprintf(f, "1 %.17g %.17g 0 %.17g %.17g 0 1 2 0\n", xmin, ymin, xmax, ymax);
  fprintf(f, "1 %.17g %.17g 0 %.17g %.17g 0 1 3 1 1\n", xmin, ymin, xmax, ymax);
  fprintf(f, "$EndEntities\n");
  // All nodes live in the surface block.
  fprintf(f, "$Nodes\n1 %lld 1 %lld\n2 1 0 %lld\n", (long long)nv, (long long)nv, (long long)nv);
  for(int64_t v = 0; v < nv; ++v) fprintf(f, "%lld\n", (long long)v + 1);
  for(int64_t v = 0; v < nv; ++v) fprintf(f, "%.17g %.17g 0\n", m.x[v], m.y[v]);
  fprintf(f, "$EndNodes\n");
  const int64_t ne = (hasPoint ? 1 : 0) + nb + nt;
  fprintf(f, "$Elements\n%d %lld 1 %lld\n", hasPoint ? 3 : 2, (long long)ne, (long long)ne);
  int64_t tag = 1;
  if(hasPoint) fprintf(f, "0 1 15 1\n%lld %d\n", (long long)tag++, m.point + 1);
  fprintf(f, "1 1 1 %lld\n", (long long)nb);
  for(int64_t i = 0; i < nb; ++i)
    fprintf(f, "%lld %d %d\n", (long long)tag++, m.bnd[2 * i] + 1, m.bnd[2 * i + 1] + 1);
  fprintf(f, "2 1 2 %lld\n", (long long)nt);
  for(int64_t t = 0; t < nt; ++t)
    fprintf(f, "%lld %d %d %d\n", (long long)tag++, m.tri[3 * t] + 1, m.tri[3 * t + 1] + 1,
            m.tri[3 * t + 2] + 1);
  fprintf(f, "$EndElements\n");
  int rc = ferror(f) ? FE_READ_ERROR : FE_OK;
  fclose(f);
  if(rc) set_error("write error on %s", path.c_str());
  return rc;
}

int mesh_read_msh41(Mesh2D &m, const std::string &path, const MeshGroups &groups)
{
  MshData d;
  FE_TRY(read_msh41(path, d));
  m = Mesh2D();
  m.x = std::move(d.x);
  m.y = std::move(d.y);
  // Element blocks keyed like the reference's entity map (dim, entity tag);
  // blocks of one entity appended in file order.
  std::map<std::pair<int, int>, std::vector<int32_t>> blocks;
  for(const MshBlock &b : d.blocks) {
    auto &blk = blocks[{b.dim, b.tag}];
    blk.insert(blk.end(), b.nodes.begin(), b.nodes.end());
  }
  // Edge tags follow triangle file order; connectivity follows entity-key
  // order.  For files with a single surface entity both coincide.
  for(auto &kv : blocks) {
    const int dim = kv.first.first;
    const std::string name = d.name_of(dim, kv.first.second);
    const bool isBoundary =
        std::find(groups.boundary.begin(), groups.boundary.end(), name) != groups.boundary.end();
    if(dim == 2 && name == groups.domain) m.tri.insert(m.tri.end(), kv.second.begin(), kv.second.end());
    else if(dim == 1 && isBoundary) m.bnd.insert(m.bnd.end(), kv.second.begin(), kv.second.end());
    else if(dim == 0 && !groups.point.empty() && name == groups.point && !kv.second.empty())
      m.point = kv.second[0];
  }
  if(m.tri.empty()) {
    set_error("no \"%s\" triangles in %s", groups.domain.c_str(), path.c_str());
    return FE_READ_ERROR;
  }
  return m.build_topology();
}

}  // namespace feng
