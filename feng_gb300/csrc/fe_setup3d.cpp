// Host set-up on tetrahedral meshes: DOF numbering, element DOF tables and
// coloring, with the conventions of the triangle set-up (fe_setup.cpp).
#include <algorithm>

#include "fe_common.h"
#include "fe_setup.h"

namespace feng {

namespace {
constexpr int8_t NONE = 0, UNKNOWN = 1, ESSENTIAL = 2;
}

int build_numbering3d(const Mesh3D &m, const std::vector<SpaceDesc> &spaces, Numbering &num)
{
  const int64_t nv = m.n_vertices(), ne = m.n_edges, nt = m.n_tets(), nb = m.n_boundary();
  if(m.tet_edges.size() != (size_t)nt * 6 || m.bnd_edges.size() != (size_t)nb * 3) {
    set_error("mesh topology not built");
    return FE_INVALID_ARG;
  }
  int nFields = 0;
  for(const auto &s : spaces) nFields = std::max(nFields, s.field + 1);
  num = Numbering();
  num.nFields = nFields;
  num.fieldComp.assign(nFields, 0);
  for(const auto &s : spaces) {
    if(s.ncomp < 1 || s.ncomp > 3 || s.degree < 1 || s.degree > 2) {
      set_error("unsupported space on tetrahedra (degree %d, %d components)", s.degree, s.ncomp);
      return FE_INVALID_ARG;
    }
    if(s.cnc != CNC_DOMAIN && s.cnc != CNC_BOUNDARY) {
      set_error("tetrahedral meshes have no \"PointPression\" group");
      return FE_INVALID_ARG;
    }
    num.fieldComp[s.field] = std::max(num.fieldComp[s.field], s.ncomp);
  }
  std::vector<std::vector<int8_t>> vcode(nFields, std::vector<int8_t>(nv, NONE));
  std::vector<std::vector<int8_t>> ecode(nFields, std::vector<int8_t>(ne, NONE));
  auto mark = [&](const SpaceDesc &s, int8_t code) {
    std::vector<int8_t> &V = vcode[s.field], &E = ecode[s.field];
    if(s.cnc == CNC_DOMAIN) {
      for(int64_t i = 0; i < nt * 4; ++i) V[m.tet[i]] = code;
      if(s.degree == 2)
        for(int64_t i = 0; i < nt * 6; ++i) E[m.tet_edges[i]] = code;
    } else {
      for(int64_t i = 0; i < nb * 3; ++i) V[m.bnd[i]] = code;
      if(s.degree == 2)
        for(int64_t i = 0; i < nb * 3; ++i) E[m.bnd_edges[i]] = code;
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
      for(int64_t v = 0; v < nv; ++v)
        if(vcode[f][v] == want)
          for(int c = 0; c < C; ++c) num.vdof[f][v * C + c] = g++;
      for(int64_t e = 0; e < ne; ++e)
        if(ecode[f][e] == want)
          for(int c = 0; c < C; ++c) num.edof[f][e * C + c] = g++;
    }
    if(pass == 0) num.nInc = g;
  }
  num.nDofs = g;

  num.dof_x.assign(g, 0.); num.dof_y.assign(g, 0.); num.dof_z.assign(g, 0.);
  num.dof_field.assign(g, -1); num.dof_comp.assign(g, -1); num.dof_is_vertex.assign(g, 0);
  for(int f = 0; f < nFields; ++f) {
    const int C = num.fieldComp[f];
    for(int64_t v = 0; v < nv; ++v)
      for(int c = 0; c < C; ++c) {
        const int64_t d = num.vdof[f][v * C + c];
        if(d < 0) continue;
        num.dof_x[d] = m.x[v]; num.dof_y[d] = m.y[v]; num.dof_z[d] = m.z[v];
        num.dof_field[d] = f; num.dof_comp[d] = c; num.dof_is_vertex[d] = 1;
      }
    for(int64_t e = 0; e < ne; ++e)
      for(int c = 0; c < C; ++c) {
        const int64_t d = num.edof[f][e * C + c];
        if(d < 0) continue;
        const int32_t a = m.edge_v[2 * e], b = m.edge_v[2 * e + 1];
        num.dof_x[d] = 0.5 * (m.x[a] + m.x[b]);
        num.dof_y[d] = 0.5 * (m.y[a] + m.y[b]);
        num.dof_z[d] = 0.5 * (m.z[a] + m.z[b]);
        num.dof_field[d] = f; num.dof_comp[d] = c; num.dof_is_vertex[d] = 0;
      }
  }
  return FE_OK;
}

int build_element_tables3d(const Mesh3D &m, const Numbering &num, int type, int fieldU, int fieldP,
                           ElementTables &et)
{
  const int64_t nt = m.n_tets();
  et = ElementTables();
  et.type = type;
  et.nElm = nt;
  auto has = [&](int f, int C) { return f >= 0 && f < num.nFields && num.fieldComp[f] == C; };
  if(type == ELEM_TET_P2) {
    if(!has(fieldU, 1)) { set_error("ELEM_TET_P2 needs a scalar field"); return FE_INVALID_ARG; }
    et.nloc = 10;
    et.adr.resize(nt * 10);
    for(int64_t t = 0; t < nt; ++t) {
      int64_t *a = &et.adr[10 * t];
      for(int k = 0; k < 4; ++k) a[k] = num.vdof[fieldU][m.tet[4 * t + k]];
      for(int k = 0; k < 6; ++k) a[4 + k] = num.edof[fieldU][m.tet_edges[6 * t + k]];
    }
    et.mask.assign(100, 1);
  } else if(type == ELEM_TET_TAYLOR_HOOD) {
    if(!has(fieldU, 3) || !has(fieldP, 1)) {
      set_error("ELEM_TET_TAYLOR_HOOD needs a 3-component velocity and a scalar pressure field");
      return FE_INVALID_ARG;
    }
    et.nloc = 34;
    et.adr.resize(nt * 34);
    for(int64_t t = 0; t < nt; ++t) {
      int64_t *a = &et.adr[34 * t];
      for(int k = 0; k < 4; ++k)
        for(int c = 0; c < 3; ++c) a[3 * k + c] = num.vdof[fieldU][3 * (int64_t)m.tet[4 * t + k] + c];
      for(int k = 0; k < 6; ++k)
        for(int c = 0; c < 3; ++c)
          a[12 + 3 * k + c] = num.edof[fieldU][3 * (int64_t)m.tet_edges[6 * t + k] + c];
      for(int k = 0; k < 4; ++k) a[30 + k] = num.vdof[fieldP][m.tet[4 * t + k]];
    }
    // Velocity rows couple to velocity and pressure columns, pressure rows
    // to velocity columns only (no pressure-pressure form).
    et.mask.assign(34 * 34, 0);
    for(int i = 0; i < 34; ++i)
      for(int j = 0; j < 34; ++j) et.mask[i * 34 + j] = (i < 30 || j < 30) ? 1 : 0;
  } else {
    set_error("unknown tetrahedral element type %d", type);
    return FE_INVALID_ARG;
  }
  for(int64_t v : et.adr)
    if(v < 0) { set_error("an element DOF is not numbered (space missing on \"Domaine\")"); return FE_INVALID_ARG; }
  return FE_OK;
}

int color_elements3d(const Mesh3D &m, Coloring &col)
{
  return color_by_vertices(m.tet.data(), 4, m.n_tets(), m.n_vertices(), 256, col);
}

}  // namespace feng
