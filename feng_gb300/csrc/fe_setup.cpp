#include "fe_setup.h"

#include <algorithm>
#include <cstring>

#include "fe_common.h"

namespace feng {

namespace {
enum Code : int8_t { NONE = 0, UNKNOWN = 1, ESSENTIAL = 2 };
}

// DOF numbering, restating feMetaNumber (feNumber.cpp:677-835):
//  * every space marks the entities it touches UNKNOWN, then every essential
//    space marks its entities ESSENTIAL;
//  * fields are numbered in order of first appearance; within a field the
//    unknown DOFs come vertex by vertex, then element by element (boundary
//    lines carry "element" DOFs that alias the edge under them,
//    feSpace_1D.cpp:490-532 and feNumber.cpp:384-403), then edge by edge;
//  * all essential DOFs follow all unknown DOFs, in the same sequence.
int build_numbering(const Mesh2D &m, const std::vector<SpaceDesc> &spaces, Numbering &num)
{
  const int64_t nv = m.n_vertices(), ne = m.n_edges, nb = m.n_boundary();
  if(m.tri_edges.size() != (size_t)m.n_triangles() * 3) {
    set_error("mesh topology not built");
    return FE_INVALID_ARG;
  }
  int nFields = 0;
  for(const auto &s : spaces) nFields = std::max(nFields, s.field + 1);
  num = Numbering();
  num.nFields = nFields;
  num.fieldComp.assign(nFields, 0);
  for(const auto &s : spaces) {
    if(s.ncomp < 1 || s.ncomp > 2 || s.degree < 0 || s.degree > 2) {
      set_error("unsupported space (degree %d, %d components)", s.degree, s.ncomp);
      return FE_INVALID_ARG;
    }
    if(s.cnc == CNC_POINT && m.point < 0) {
      set_error("space on \"PointPression\" but the mesh has no such point");
      return FE_INVALID_ARG;
    }
    num.fieldComp[s.field] = std::max(num.fieldComp[s.field], s.ncomp);
  }

  struct FieldCodes {
    std::vector<int8_t> v, e, l;  // vertex, edge, boundary-line ("element") codes
    std::vector<int8_t> nv, ne, nl;  // DOFs per entity
  };
  std::vector<FieldCodes> fc(nFields);
  for(int f = 0; f < nFields; ++f) {
    fc[f].v.assign(nv, NONE); fc[f].e.assign(ne, NONE); fc[f].l.assign(nb, NONE);
    fc[f].nv.assign(nv, 0); fc[f].ne.assign(ne, 0); fc[f].nl.assign(nb, 0);
  }
  auto mark = [&](const SpaceDesc &s, int8_t code) {
    FieldCodes &F = fc[s.field];
    const int c = s.ncomp;
    if(s.cnc == CNC_DOMAIN) {
      for(int64_t t = 0; t < m.n_triangles(); ++t) {
        if(s.degree >= 1)
          for(int k = 0; k < 3; ++k) { int32_t v = m.tri[3 * t + k]; F.v[v] = code; F.nv[v] = c; }
        if(s.degree == 2)
          for(int k = 0; k < 3; ++k) { int32_t e = m.tri_edges[3 * t + k]; F.e[e] = code; F.ne[e] = c; }
      }
    } else if(s.cnc == CNC_BOUNDARY) {
      for(int64_t i = 0; i < nb; ++i) {
        if(s.degree >= 1)
          for(int k = 0; k < 2; ++k) { int32_t v = m.bnd[2 * i + k]; F.v[v] = code; F.nv[v] = c; }
        if(s.degree == 2) {
          F.l[i] = code; F.nl[i] = c;
          int32_t e = m.bnd_edges[i]; F.e[e] = code; F.ne[e] = c;
        }
      }
    } else {
      F.v[m.point] = code; F.nv[m.point] = c;
    }
  };
  for(const auto &s : spaces) mark(s, UNKNOWN);
  for(const auto &s : spaces)
    if(s.essential) mark(s, ESSENTIAL);

  num.vdof.assign(nFields, {});
  num.edof.assign(nFields, {});
  for(int f = 0; f < nFields; ++f) {
    num.vdof[f].assign(nv * num.fieldComp[f], -1);
    num.edof[f].assign(ne * num.fieldComp[f], -1);
  }
  int64_t g = 0;
  for(int pass = 0; pass < 2; ++pass) {
    const int8_t want = pass == 0 ? UNKNOWN : ESSENTIAL;
    for(int f = 0; f < nFields; ++f) {
      const int C = num.fieldComp[f];
      FieldCodes &F = fc[f];
      for(int64_t v = 0; v < nv; ++v)
        if(F.v[v] == want)
          for(int c = 0; c < F.nv[v]; ++c) num.vdof[f][v * C + c] = g++;
      for(int64_t i = 0; i < nb; ++i)
        if(F.l[i] == want) {
          int32_t e = m.bnd_edges[i];
          for(int c = 0; c < F.nl[i]; ++c) num.edof[f][(int64_t)e * C + c] = g++;
          F.e[e] = NONE;  // numbered through the line element
        }
      for(int64_t e = 0; e < ne; ++e)
        if(F.e[e] == want)
          for(int c = 0; c < F.ne[e]; ++c) num.edof[f][e * C + c] = g++;
    }
    if(pass == 0) num.nInc = g;
  }
  num.nDofs = g;

  num.dof_x.assign(g, 0.); num.dof_y.assign(g, 0.);
  num.dof_field.assign(g, -1); num.dof_comp.assign(g, -1); num.dof_is_vertex.assign(g, 0);
  for(int f = 0; f < nFields; ++f) {
    const int C = num.fieldComp[f];
    for(int64_t v = 0; v < nv; ++v)
      for(int c = 0; c < C; ++c) {
        int64_t d = num.vdof[f][v * C + c];
        if(d < 0) continue;
        num.dof_x[d] = m.x[v]; num.dof_y[d] = m.y[v];
        num.dof_field[d] = f; num.dof_comp[d] = c; num.dof_is_vertex[d] = 1;
      }
    for(int64_t e = 0; e < ne; ++e)
      for(int c = 0; c < C; ++c) {
        int64_t d = num.edof[f][e * C + c];
        if(d < 0) continue;
        int32_t a = m.edge_v[2 * e], b = m.edge_v[2 * e + 1];
        num.dof_x[d] = 0.5 * (m.x[a] + m.x[b]); num.dof_y[d] = 0.5 * (m.y[a] + m.y[b]);
        num.dof_field[d] = f; num.dof_comp[d] = c; num.dof_is_vertex[d] = 0;
      }
  }
  return FE_OK;
}

int build_element_tables(const Mesh2D &m, const Numbering &num, int type, int fieldU, int fieldP,
                         ElementTables &et)
{
  const int64_t nt = m.n_triangles();
  et = ElementTables();
  et.type = type;
  et.nElm = nt;
  if(type == ELEM_P2) {
    if(fieldU < 0 || fieldU >= num.nFields || num.fieldComp[fieldU] != 1) {
      set_error("ELEM_P2 needs a scalar field");
      return FE_INVALID_ARG;
    }
    et.nloc = 6;
    et.adr.resize(nt * 6);
    for(int64_t t = 0; t < nt; ++t) {
      for(int k = 0; k < 3; ++k) et.adr[6 * t + k] = num.vdof[fieldU][m.tri[3 * t + k]];
      for(int k = 0; k < 3; ++k) et.adr[6 * t + 3 + k] = num.edof[fieldU][m.tri_edges[3 * t + k]];
    }
    et.mask.assign(36, 1);
  } else if(type == ELEM_TAYLOR_HOOD) {
    if(fieldU < 0 || fieldP < 0 || fieldU >= num.nFields || fieldP >= num.nFields ||
       num.fieldComp[fieldU] != 2 || num.fieldComp[fieldP] != 1) {
      set_error("ELEM_TAYLOR_HOOD needs a 2-component velocity and a scalar pressure field");
      return FE_INVALID_ARG;
    }
    et.nloc = 15;
    et.adr.resize(nt * 15);
    for(int64_t t = 0; t < nt; ++t) {
      int64_t *a = &et.adr[15 * t];
      for(int k = 0; k < 3; ++k)
        for(int c = 0; c < 2; ++c) a[2 * k + c] = num.vdof[fieldU][2 * (int64_t)m.tri[3 * t + k] + c];
      for(int k = 0; k < 3; ++k)
        for(int c = 0; c < 2; ++c)
          a[6 + 2 * k + c] = num.edof[fieldU][2 * (int64_t)m.tri_edges[3 * t + k] + c];
      for(int k = 0; k < 3; ++k) a[12 + k] = num.vdof[fieldP][m.tri[3 * t + k]];
    }
    // Velocity rows couple to velocity and pressure columns, pressure rows to
    // velocity columns; the pressure-pressure block holds no form.
    et.mask.assign(225, 0);
    for(int i = 0; i < 15; ++i)
      for(int j = 0; j < 15; ++j) et.mask[i * 15 + j] = (i < 12 || j < 12) ? 1 : 0;
  } else {
    set_error("unknown element type %d", type);
    return FE_INVALID_ARG;
  }
  for(int64_t a : et.adr)
    if(a < 0) {
      set_error("element references a DOF that no space numbered");
      return FE_INVALID_ARG;
    }
  return FE_OK;
}

// Greedy vertex-sharing coloring in rounds, restating feCncGeo::colorElements
// algorithm 1 (feCncGeo.cpp:752-790): each round walks the uncolored elements
// in index order, takes an element whose uncolored vertex-neighbours were not
// taken earlier in the round, and blocks those neighbours.
int color_by_vertices(const int32_t *ev, int nvpe, int64_t ne, int64_t nv, int maxColors, Coloring &col)
{
  std::vector<int64_t> vstart(nv + 1, 0);
  for(int64_t i = 0; i < ne * nvpe; ++i) vstart[ev[i] + 1]++;
  for(int64_t v = 0; v < nv; ++v) vstart[v + 1] += vstart[v];
  std::vector<int32_t> velm(ne * nvpe);
  std::vector<int64_t> fill(vstart.begin(), vstart.end() - 1);
  for(int64_t t = 0; t < ne; ++t)
    for(int k = 0; k < nvpe; ++k) velm[fill[ev[nvpe * t + k]]++] = (int32_t)t;

  col = Coloring();
  col.elm_color.assign(ne, -1);
  std::vector<int8_t> blocked(ne, 0);
  int64_t done = 0;
  col.offsets.push_back(0);
  while(done < ne) {
    const int c = col.nColors;
    for(int64_t k = 0; k < ne; ++k) {
      if(col.elm_color[k] != -1 || blocked[k]) continue;
      for(int j = 0; j < nvpe; ++j) {
        int32_t v = ev[nvpe * k + j];
        for(int64_t p = vstart[v]; p < vstart[v + 1]; ++p) {
          int32_t o = velm[p];
          if(o != k && col.elm_color[o] == -1) blocked[o] = 1;
        }
      }
    }
    for(int64_t k = 0; k < ne; ++k) {
      if(col.elm_color[k] != -1) continue;
      if(blocked[k]) { blocked[k] = 0; continue; }
      col.elm_color[k] = c;
      col.elements.push_back((int32_t)k);
      ++done;
    }
    col.nColors++;
    col.offsets.push_back((int64_t)col.elements.size());
    if(col.nColors > maxColors) {
      set_error("coloring did not terminate");
      return FE_ERROR;
    }
  }
  return FE_OK;
}

int color_elements(const Mesh2D &m, Coloring &col)
{
  return color_by_vertices(m.tri.data(), 3, m.n_triangles(), m.n_vertices(), 64, col);
}

int validate_coloring(const Mesh2D &m, const Coloring &col)
{
  const int64_t nt = m.n_triangles(), nv = m.n_vertices();
  if((int64_t)col.elements.size() != nt || (int64_t)col.offsets.size() != col.nColors + 1 ||
     col.offsets.back() != nt) {
    set_error("coloring does not cover every element exactly once");
    return FE_BAD_COLORING;
  }
  std::vector<int8_t> seen(nt, 0);
  std::vector<int32_t> stamp(nv, -1);
  for(int c = 0; c < col.nColors; ++c) {
    for(int64_t p = col.offsets[c]; p < col.offsets[c + 1]; ++p) {
      int32_t t = col.elements[p];
      if(t < 0 || t >= nt || seen[t]) {
        set_error("element %d listed twice or out of range in the coloring", t);
        return FE_BAD_COLORING;
      }
      seen[t] = 1;
      for(int k = 0; k < 3; ++k) {
        int32_t v = m.tri[3 * t + k];
        if(stamp[v] == c) {
          set_error("two elements of color %d share vertex %d", c, v);
          return FE_BAD_COLORING;
        }
        stamp[v] = c;
      }
    }
  }
  return FE_OK;
}

// Sparsity pattern, restating feEZCompressedRowStorage
// (feCompressedRowStorage.cpp:15-135): the diagonal of every unknown row, plus
// every (adrI, adrJ) pair of every matrix form with both DOFs unknown, sorted
// and made unique row by row.  Rows are gathered here through the DOF-to-element
// adjacency, row by row in parallel, which yields the same sets.
int build_csr_pattern(const ElementTables &et, int64_t nInc, CSRPattern &pat)
{
  const int nl = et.nloc;
  const int64_t nt = et.nElm;
  // Unknown DOF -> (element, local index) adjacency, elements in order.
  std::vector<int64_t> dptr(nInc + 1, 0);
  for(int64_t t = 0; t < nt; ++t)
    for(int i = 0; i < nl; ++i)
      if(et.adr[t * nl + i] < nInc) ++dptr[et.adr[t * nl + i] + 1];
  for(int64_t r = 0; r < nInc; ++r) dptr[r + 1] += dptr[r];
  std::vector<int64_t> adj(dptr[nInc]);
  {
    std::vector<int64_t> fill(dptr.begin(), dptr.end() - 1);
    for(int64_t t = 0; t < nt; ++t)
      for(int i = 0; i < nl; ++i) {
        const int64_t d = et.adr[t * nl + i];
        if(d < nInc) adj[fill[d]++] = t * nl + i;
      }
  }
  // Row r: its diagonal and the coupled unknown DOFs of the elements that
  // hold it, sorted and unique.  Consecutive rows are built in chunks on the
  // host threads, each chunk into its own array, then copied into place, so
  // the scratch memory is the size of the pattern.  A per-thread stamp
  // (last row that took each column) drops repeated columns while gathering,
  // so only the unique columns are sorted.
  constexpr int64_t kRows = 1 << 12;
  const int64_t nChunks = (nInc + kRows - 1) / kRows;
  std::vector<std::vector<int32_t>> part((size_t)nChunks);
  pat = CSRPattern();
  pat.n = nInc;
  pat.ia.assign(nInc + 1, 0);
  parallel_for(
      nChunks,
      [&](int64_t c0, int64_t c1) {
        std::vector<int32_t> row;
        std::vector<int32_t> stamp((size_t)nInc, -1);
        for(int64_t c = c0; c < c1; ++c) {
          std::vector<int32_t> &out = part[(size_t)c];
          const int64_t rEnd = std::min(nInc, (c + 1) * kRows);
          for(int64_t r = c * kRows; r < rEnd; ++r) {
            row.clear();
            row.push_back((int32_t)r);
            stamp[(size_t)r] = (int32_t)r;
            for(int64_t k = dptr[r]; k < dptr[r + 1]; ++k) {
              const int64_t t = adj[k] / nl;
              const int i = (int)(adj[k] - t * nl);
              const int64_t *a = &et.adr[t * nl];
              for(int j = 0; j < nl; ++j) {
                const int64_t col = a[j];
                if(et.mask[i * nl + j] && col < nInc && stamp[(size_t)col] != (int32_t)r) {
                  stamp[(size_t)col] = (int32_t)r;
                  row.push_back((int32_t)col);
                }
              }
            }
            std::sort(row.begin(), row.end());
            pat.ia[r + 1] = (int64_t)row.size();
            out.insert(out.end(), row.begin(), row.end());
          }
        }
      },
      1);
  for(int64_t r = 0; r < nInc; ++r) pat.ia[r + 1] += pat.ia[r];
  if(pat.ia[nInc] >= (int64_t)INT32_MAX) {
    set_error("more than 2^31 nonzeros: 32-bit scatter map does not fit");
    return FE_INVALID_ARG;
  }
  pat.ja.resize(pat.ia[nInc]);
  parallel_for(
      nChunks,
      [&](int64_t c0, int64_t c1) {
        for(int64_t c = c0; c < c1; ++c) {
          std::copy(part[(size_t)c].begin(), part[(size_t)c].end(), pat.ja.begin() + pat.ia[c * kRows]);
          std::vector<int32_t>().swap(part[(size_t)c]);
        }
      },
      1);
  return FE_OK;
}

int build_scatter_map(const ElementTables &et, const Coloring &col, const CSRPattern &pat,
                      int64_t nInc, std::vector<int32_t> &map)
{
  const int nl = et.nloc;
  const int64_t nt = et.nElm;
  map.assign((size_t)nl * nl * nt, -1);
  std::atomic<int> missing{0};
  int64_t missI = 0, missJ = 0;
  parallel_for(nt, [&](int64_t p0, int64_t p1) {
    for(int64_t p = p0; p < p1; ++p) {
      const int32_t t = col.elements[p];
      const int64_t *a = &et.adr[(int64_t)t * nl];
      for(int i = 0; i < nl; ++i) {
        if(a[i] >= nInc) continue;
        const int32_t *rb = pat.ja.data() + pat.ia[a[i]];
        const int32_t *re = pat.ja.data() + pat.ia[a[i] + 1];
        for(int j = 0; j < nl; ++j) {
          if(!et.mask[i * nl + j] || a[j] >= nInc) continue;
          const int32_t *f = std::lower_bound(rb, re, (int32_t)a[j]);
          if(f == re || *f != a[j]) {
            if(missing.exchange(1) == 0) {
              missI = a[i];
              missJ = a[j];
            }
            continue;
          }
          map[(size_t)(i * nl + j) * nt + p] = (int32_t)(f - pat.ja.data());
        }
      }
    }
  });
  if(missing.load()) {
    set_error("pattern misses (%lld,%lld)", (long long)missI, (long long)missJ);
    return FE_ERROR;
  }
  return FE_OK;
}

}  // namespace feng
