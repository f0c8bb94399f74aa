#include "fe_mesh3d.h"

#include <algorithm>
#include <cmath>
#include <cstdio>

#include "fe_common.h"
#include "fe_msh.h"

namespace feng {

const int TET_FACES[4][3] = {{0, 2, 1}, {0, 1, 3}, {0, 3, 2}, {3, 1, 2}};
const int TET_EDGES[6][2] = {{0, 2}, {2, 1}, {1, 0}, {1, 3}, {3, 0}, {3, 2}};

int Mesh3D::build_topology()
{
  const int64_t nv = n_vertices(), nt = n_tets(), nb = n_boundary();
  for(int32_t v : tet)
    if(v < 0 || v >= nv) { set_error("tetrahedron vertex out of range"); return FE_INVALID_ARG; }
  for(int32_t v : bnd)
    if(v < 0 || v >= nv) { set_error("boundary triangle vertex out of range"); return FE_INVALID_ARG; }
  // Edges of each vertex to higher-numbered neighbours: (neighbour, edge id).
  std::vector<std::vector<std::pair<int32_t, int32_t>>> adj((size_t)nv);
  edge_v.clear();
  auto find = [&](int32_t a, int32_t b) {
    const int32_t lo = std::min(a, b), hi = std::max(a, b);
    for(const auto &p : adj[(size_t)lo])
      if(p.first == hi) return p.second;
    return (int32_t)-1;
  };
  auto add = [&](int32_t a, int32_t b) {
    int32_t e = find(a, b);
    if(e < 0) {
      e = (int32_t)(edge_v.size() / 2);
      adj[(size_t)std::min(a, b)].push_back({std::max(a, b), e});
      edge_v.push_back(a);
      edge_v.push_back(b);
    }
    return e;
  };
  bnd_edges.assign(nb * 3, -1);
  for(int64_t i = 0; i < nb; ++i)
    for(int k = 0; k < 3; ++k) bnd_edges[3 * i + k] = add(bnd[3 * i + k], bnd[3 * i + (k + 1) % 3]);
  const int64_t nBndEdges = (int64_t)edge_v.size() / 2;
  for(int64_t t = 0; t < nt; ++t)
    for(int f = 0; f < 4; ++f) {
      const int32_t v[3] = {tet[4 * t + TET_FACES[f][0]], tet[4 * t + TET_FACES[f][1]], tet[4 * t + TET_FACES[f][2]]};
      for(int k = 0; k < 3; ++k) add(v[k], v[(k + 1) % 3]);
    }
  n_edges = (int64_t)edge_v.size() / 2;
  tet_edges.assign(nt * 6, -1);
  for(int64_t t = 0; t < nt; ++t)
    for(int k = 0; k < 6; ++k)
      tet_edges[6 * t + k] = find(tet[4 * t + TET_EDGES[k][0]], tet[4 * t + TET_EDGES[k][1]]);
  // Every boundary edge must belong to a tetrahedron: edges only the
  // boundary created and no tetrahedron met mean a stray boundary triangle.
  std::vector<uint8_t> used((size_t)n_edges, 0);
  for(int32_t e : tet_edges) used[e] = 1;
  for(int64_t e = 0; e < nBndEdges; ++e)
    if(!used[e]) { set_error("boundary triangle edge %lld is not an edge of the tetrahedra", (long long)e); return FE_INVALID_ARG; }
  return FE_OK;
}

namespace {

double tet_det(const Mesh3D &m, int32_t a, int32_t b, int32_t c, int32_t d)
{
  const double ux = m.x[b] - m.x[a], uy = m.y[b] - m.y[a], uz = m.z[b] - m.z[a];
  const double vx = m.x[c] - m.x[a], vy = m.y[c] - m.y[a], vz = m.z[c] - m.z[a];
  const double wx = m.x[d] - m.x[a], wy = m.y[d] - m.y[a], wz = m.z[d] - m.z[a];
  return ux * (vy * wz - vz * wy) - uy * (vx * wz - vz * wx) + uz * (vx * wy - vy * wx);
}

}  // namespace

int mesh3d_generate_cube(Mesh3D &m, int n, const double box[6], double jitter, uint64_t seed)
{
  if(n < 1 || n > 1000 || !(box[1] > box[0]) || !(box[3] > box[2]) || !(box[5] > box[4]) || jitter < 0 ||
     jitter >= 0.25) {
    set_error("invalid cube mesh parameters (n=%d, jitter=%g)", n, jitter);
    return FE_INVALID_ARG;
  }
  m = Mesh3D();
  const int64_t n1 = n + 1;
  const double h[3] = {(box[1] - box[0]) / n, (box[3] - box[2]) / n, (box[5] - box[4]) / n};
  auto vid = [&](int64_t i, int64_t j, int64_t k) { return (int32_t)((k * n1 + j) * n1 + i); };
  m.x.resize(n1 * n1 * n1);
  m.y.resize(n1 * n1 * n1);
  m.z.resize(n1 * n1 * n1);
  SplitMix64 rng(seed);
  for(int64_t k = 0; k <= n; ++k)
    for(int64_t j = 0; j <= n; ++j)
      for(int64_t i = 0; i <= n; ++i) {
        // Exact end points on the boundary.
        double x = i == n ? box[1] : box[0] + i * h[0];
        double y = j == n ? box[3] : box[2] + j * h[1];
        double z = k == n ? box[5] : box[4] + k * h[2];
        if(i > 0 && i < n && j > 0 && j < n && k > 0 && k < n && jitter > 0) {
          x += jitter * h[0] * rng.uniform_pm1();
          y += jitter * h[1] * rng.uniform_pm1();
          z += jitter * h[2] * rng.uniform_pm1();
        }
        const int32_t v = vid(i, j, k);
        m.x[v] = x;
        m.y[v] = y;
        m.z[v] = z;
      }
  // Kuhn split: axis orderings and their parity.
  static const int order[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
  static const bool odd[6] = {false, true, true, false, false, true};
  m.tet.reserve((size_t)n * n * n * 24);
  for(int64_t k = 0; k < n; ++k)
    for(int64_t j = 0; j < n; ++j)
      for(int64_t i = 0; i < n; ++i)
        for(int p = 0; p < 6; ++p) {
          int64_t c[3] = {i, j, k};
          int32_t v[4];
          v[0] = vid(c[0], c[1], c[2]);
          ++c[order[p][0]];
          v[1] = vid(c[0], c[1], c[2]);
          ++c[order[p][1]];
          v[2] = vid(c[0], c[1], c[2]);
          v[3] = vid(i + 1, j + 1, k + 1);
          if(odd[p]) std::swap(v[2], v[3]);
          m.tet.insert(m.tet.end(), v, v + 4);
        }
  for(int64_t t = 0; t < m.n_tets(); ++t) {
    const int32_t *v = &m.tet[4 * t];
    if(!(tet_det(m, v[0], v[1], v[2], v[3]) > 0)) {
      set_error("tetrahedron %lld has a non-positive volume (jitter too large)", (long long)t);
      return FE_INVALID_ARG;
    }
  }
  // Boundary squares, two triangles each, cut from the lowest to the highest
  // corner as the tetrahedra cut them; outward orientation.
  for(int axis = 0; axis < 3; ++axis)
    for(int side = 0; side < 2; ++side) {
      const int a1 = (axis + 1) % 3, a2 = (axis + 2) % 3;
      const int u = std::min(a1, a2), w = std::max(a1, a2);  // in-plane axes, lower first
      for(int64_t q = 0; q < n; ++q)
        for(int64_t p = 0; p < n; ++p) {
          int64_t c[3];
          c[axis] = side ? n : 0;
          auto corner = [&](int du, int dw) {
            c[u] = p + du;
            c[w] = q + dw;
            return vid(c[0], c[1], c[2]);
          };
          const int32_t lo = corner(0, 0), b = corner(1, 0), d = corner(0, 1), hi = corner(1, 1);
          int32_t t1[3] = {lo, b, hi}, t2[3] = {lo, hi, d};
          // (e_u x e_w) points along +axis when (u, w, axis) is a cyclic order.
          const bool cyclic = (u + 1) % 3 == w;
          const bool flip = cyclic != (side == 1);
          if(flip) {
            std::swap(t1[1], t1[2]);
            std::swap(t2[1], t2[2]);
          }
          m.bnd.insert(m.bnd.end(), t1, t1 + 3);
          m.bnd.insert(m.bnd.end(), t2, t2 + 3);
        }
    }
  return m.build_topology();
}

int mesh3d_write_msh41(const Mesh3D &m, const std::string &path)
{
  FILE *f = fopen(path.c_str(), "w");
  if(!f) {
    set_error("cannot open %s for writing", path.c_str());
    return FE_READ_ERROR;
  }
  const int64_t nv = m.n_vertices(), nt = m.n_tets(), nb = m.n_boundary();
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  for(int64_t v = 0; v < nv; ++v) {
    const double p[3] = {m.x[v], m.y[v], m.z[v]};
    for(int d = 0; d < 3; ++d) { lo[d] = std::min(lo[d], p[d]); hi[d] = std::max(hi[d], p[d]); }
  }
  fprintf(f, "$MeshFormat\n4.1 0 8\n$EndMeshFormat\n");
  fprintf(f, "$PhysicalNames\n2\n2 1 \"Bord\"\n3 2 \"Domaine\"\n$EndPhysicalNames\n");
  fprintf(f, "$Entities\n0 0 1 1\n");
  fprintf(f, "1 %.17g %.17g %.17g %.17g %.17g %.17g 1 1 0\n", lo[0], lo[1], lo[2], hi[0], hi[1], hi[2]);
  fprintf(f, "1 %.17g %.17g %.17g %.17g %.17g %.17g 1 2 1 1\n", lo[0], lo[1], lo[2], hi[0], hi[1], hi[2]);
  fprintf(f, "$EndEntities\n");
  fprintf(f, "$Nodes\n1 %lld 1 %lld\n3 1 0 %lld\n", (long long)nv, (long long)nv, (long long)nv);
  for(int64_t v = 0; v < nv; ++v) fprintf(f, "%lld\n", (long long)v + 1);
  for(int64_t v = 0; v < nv; ++v) fprintf(f, "%.17g %.17g %.17g\n", m.x[v], m.y[v], m.z[v]);
  fprintf(f, "$EndNodes\n");
  fprintf(f, "$Elements\n2 %lld 1 %lld\n", (long long)(nb + nt), (long long)(nb + nt));
  int64_t tag = 1;
  fprintf(f, "2 1 2 %lld\n", (long long)nb);
  for(int64_t i = 0; i < nb; ++i)
    fprintf(f, "%lld %d %d %d\n", (long long)tag++, m.bnd[3 * i] + 1, m.bnd[3 * i + 1] + 1, m.bnd[3 * i + 2] + 1);
  fprintf(f, "3 1 4 %lld\n", (long long)nt);
  for(int64_t t = 0; t < nt; ++t)
    fprintf(f, "%lld %d %d %d %d\n", (long long)tag++, m.tet[4 * t] + 1, m.tet[4 * t + 1] + 1,
            m.tet[4 * t + 2] + 1, m.tet[4 * t + 3] + 1);
  fprintf(f, "$EndElements\n");
  const int rc = ferror(f) ? FE_READ_ERROR : FE_OK;
  fclose(f);
  if(rc) set_error("write error on %s", path.c_str());
  return rc;
}

int mesh3d_read_msh41(Mesh3D &m, const std::string &path, const std::string &domain,
                      const std::vector<std::string> &boundary)
{
  MshData d;
  FE_TRY(read_msh41(path, d));
  m = Mesh3D();
  m.x = std::move(d.x);
  m.y = std::move(d.y);
  m.z = std::move(d.z);
  bool seenTets = false;
  for(const MshBlock &b : d.blocks) {
    const std::string name = d.name_of(b.dim, b.tag);
    if(b.dim == 3 && b.type == 4 && name == domain) {
      m.tet.insert(m.tet.end(), b.nodes.begin(), b.nodes.end());
      seenTets = true;
    } else if(b.dim == 2 && b.type == 2 &&
              std::find(boundary.begin(), boundary.end(), name) != boundary.end()) {
      if(seenTets) {
        set_error("boundary triangles follow tetrahedra in %s; they must precede them", path.c_str());
        return FE_READ_ERROR;
      }
      m.bnd.insert(m.bnd.end(), b.nodes.begin(), b.nodes.end());
    }
  }
  if(m.tet.empty()) {
    set_error("no \"%s\" tetrahedra in %s", domain.c_str(), path.c_str());
    return FE_READ_ERROR;
  }
  return m.build_topology();
}

}  // namespace feng
