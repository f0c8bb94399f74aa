// extern "C" entry points declared in include/feng_cuda.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstring>
#include <memory>
#include <new>
#include <string>

#include "../../include/feng_cuda.h"
#include "fe_common.h"
#include "fe_export.h"
#include "fe_mesh.h"
#include "fe_mesh3d.h"
#include "fe_setup.h"
#include "fe_system.h"
#include "fe_transient.h"

namespace feng {
namespace {
thread_local std::string g_err;
}
void set_error(const char *fmt, ...)
{
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
}
const char *last_error() { return g_err.c_str(); }
std::atomic<long long> g_launches{0};
thread_local int g_capturing = 0;
}  // namespace feng

using namespace feng;

struct fe_mesh {
  Mesh2D m;
};

struct fe_mesh3d {
  Mesh3D m;
};

struct fe_cuda_system {
  SystemCUDA sys;
  double *saved = nullptr;
  cudaEvent_t ev[8] = {};
  ~fe_cuda_system()
  {
    cudaFree(saved);
    for(auto e : ev)
      if(e) cudaEventDestroy(e);
  }
};

struct fe_setup {
  bool tets = false;                  // built on a tetrahedral mesh
  std::vector<SpaceDesc> spaces;
  int64_t nVertices = 0, nEdges = 0;  // of the mesh the setup was built on
  Numbering num;
  ElementTables et;
  Coloring col;
  CSRPattern pat;
  int patternOnDevice = 0;            // the pattern was built on the device
  std::vector<int32_t> blockOfRow;
  std::vector<double> elemXY;
  QuadRule quad;
};

#define GUARD_BEGIN try {
#define GUARD_END                                  \
  }                                                \
  catch(const std::bad_alloc &) {                  \
    set_error("host allocation failed");           \
    return FE_CUDA_ERROR;                          \
  }                                                \
  catch(...) {                                     \
    set_error("unexpected exception");             \
    return FE_CUDA_ERROR;                          \
  }

static int check_options(const fe_cuda_options *o)
{
  if(!o) {
    set_error("null options");
    return FE_INVALID_ARG;
  }
  if(o->krylov < 0 || o->krylov > 1 || o->precond < 0 || o->precond > 3 || o->precision < 0 ||
     o->precision > 1 || o->restart < 1 || o->restart > 128 || o->max_iter < 1 ||
     !(o->rel_tol >= 0) || !(o->abs_tol >= 0) || o->pc_block_rows < 0) {
    set_error("invalid linear solver options");
    return FE_INVALID_ARG;
  }
  return FE_OK;
}

static SystemOptions to_sys_options(const fe_cuda_options *o)
{
  SystemOptions so;
  so.kry.method = o->krylov;
  so.kry.restart = o->restart;
  so.kry.maxIter = o->max_iter;
  so.kry.rtol = o->rel_tol;
  so.kry.atol = o->abs_tol;
  so.kry.dtol = o->div_tol > 0 ? o->div_tol : 1e6;
  so.kry.precond = o->precond;
  so.pcBlockRows = o->pc_block_rows;
  so.precision = o->precision;
  so.mgInner = o->mg_inner;
  so.mgSmooth = o->mg_smooth > 0 ? o->mg_smooth : 1;
  so.kry.gsPasses = o->gs_passes == 2 || o->gs_passes == 3 ? o->gs_passes : 1;
  return so;
}

static void to_forms(const fe_form_desc *forms, int n, std::vector<FormDesc> &out)
{
  out.resize(n);
  for(int i = 0; i < n; ++i) {
    out[i].kind = forms[i].kind;
    out[i].coeff = forms[i].coeff;
    out[i].coeff2 = forms[i].coeff2;
    out[i].source = forms[i].source;
    for(int k = 0; k < 4; ++k) out[i].params[k] = forms[i].params[k];
  }
}

extern "C" {

const char *fe_cuda_last_error(void) { return last_error(); }
int fe_cuda_version(void) { return 1; }

int fe_cuda_device_count(int *count)
{
  int c = 0;
  cudaError_t e = cudaGetDeviceCount(&c);
  if(count) *count = (e == cudaSuccess) ? c : 0;
  if(e != cudaSuccess) {
    cudaGetLastError();
    set_error("cudaGetDeviceCount: %s", cudaGetErrorString(e));
    return FE_CUDA_DEVICE_FAIL;
  }
  return FE_OK;
}

int fe_mesh_generate_square(int n, double x0, double x1, double y0, double y1, double jitter,
                            uint64_t seed, fe_mesh **out)
{
  GUARD_BEGIN
  if(!out) { set_error("null output"); return FE_INVALID_ARG; }
  auto *m = new fe_mesh();
  int s = mesh_generate_square(m->m, n, x0, x1, y0, y1, jitter, seed);
  if(s) { delete m; return s; }
  *out = m;
  return FE_OK;
  GUARD_END
}

int fe_mesh_read_msh(const char *path, fe_mesh **out)
{
  GUARD_BEGIN
  if(!out || !path) { set_error("null argument"); return FE_INVALID_ARG; }
  auto *m = new fe_mesh();
  int s = mesh_read_msh41(m->m, path);
  if(s) { delete m; return s; }
  *out = m;
  return FE_OK;
  GUARD_END
}

int fe_mesh_read_msh_groups(const char *path, const char *domain, const char *const *boundary,
                            int n_boundary, const char *point, fe_mesh **out)
{
  GUARD_BEGIN
  if(!out || !path || !domain || n_boundary < 0 || (n_boundary > 0 && !boundary)) {
    set_error("null argument");
    return FE_INVALID_ARG;
  }
  MeshGroups g;
  g.domain = domain;
  g.boundary.clear();
  for(int i = 0; i < n_boundary; ++i) {
    if(!boundary[i]) { set_error("null boundary group name"); return FE_INVALID_ARG; }
    g.boundary.push_back(boundary[i]);
  }
  g.point = point ? point : "";
  auto *m = new fe_mesh();
  int s = mesh_read_msh41(m->m, path, g);
  if(s) { delete m; return s; }
  *out = m;
  return FE_OK;
  GUARD_END
}

int fe_mesh_from_arrays(int64_t nv, const double *x, const double *y, int64_t nt, const int32_t *tri,
                        int64_t nb, const int32_t *bnd, int32_t point, fe_mesh **out)
{
  GUARD_BEGIN
  if(!out || !x || !y || !tri || nv <= 0 || nt <= 0 || nb < 0 || (nb > 0 && !bnd)) {
    set_error("null or empty argument");
    return FE_INVALID_ARG;
  }
  for(int64_t i = 0; i < 3 * nt; ++i)
    if(tri[i] < 0 || tri[i] >= nv) { set_error("triangle vertex %d out of range", tri[i]); return FE_INVALID_ARG; }
  for(int64_t i = 0; i < 2 * nb; ++i)
    if(bnd[i] < 0 || bnd[i] >= nv) { set_error("boundary vertex %d out of range", bnd[i]); return FE_INVALID_ARG; }
  if(point < -1 || point >= nv) { set_error("point vertex %d out of range", point); return FE_INVALID_ARG; }
  auto *m = new fe_mesh();
  m->m.x.assign(x, x + nv);
  m->m.y.assign(y, y + nv);
  m->m.tri.assign(tri, tri + 3 * nt);
  m->m.bnd.assign(bnd, bnd + 2 * nb);
  m->m.point = point;
  int s = m->m.build_topology();
  if(s) { delete m; return s; }
  *out = m;
  return FE_OK;
  GUARD_END
}

int fe_mesh_write_msh(const fe_mesh *m, const char *path)
{
  GUARD_BEGIN
  if(!m || !path) { set_error("null argument"); return FE_INVALID_ARG; }
  return mesh_write_msh41(m->m, path);
  GUARD_END
}

int fe_mesh_sizes(const fe_mesh *m, int64_t *nv, int64_t *nt, int64_t *ne, int64_t *nb)
{
  if(!m) { set_error("null mesh"); return FE_INVALID_ARG; }
  if(nv) *nv = m->m.n_vertices();
  if(nt) *nt = m->m.n_triangles();
  if(ne) *ne = m->m.n_edges;
  if(nb) *nb = m->m.n_boundary();
  return FE_OK;
}

int fe_mesh_arrays(const fe_mesh *m, double *x, double *y, int32_t *tri, int32_t *tri_edges,
                   int32_t *bnd, int32_t *point)
{
  if(!m) { set_error("null mesh"); return FE_INVALID_ARG; }
  const Mesh2D &M = m->m;
  if(x) std::copy(M.x.begin(), M.x.end(), x);
  if(y) std::copy(M.y.begin(), M.y.end(), y);
  if(tri) std::copy(M.tri.begin(), M.tri.end(), tri);
  if(tri_edges) std::copy(M.tri_edges.begin(), M.tri_edges.end(), tri_edges);
  if(bnd) std::copy(M.bnd.begin(), M.bnd.end(), bnd);
  if(point) *point = M.point;
  return FE_OK;
}

void fe_mesh_destroy(fe_mesh *m) { delete m; }

int fe_mesh3d_generate_cube(int n, const double *box, double jitter, uint64_t seed, fe_mesh3d **out)
{
  GUARD_BEGIN
  if(!out || !box) { set_error("null argument"); return FE_INVALID_ARG; }
  std::unique_ptr<fe_mesh3d> m(new fe_mesh3d());
  FE_TRY(mesh3d_generate_cube(m->m, n, box, jitter, seed));
  *out = m.release();
  return FE_OK;
  GUARD_END
}

int fe_mesh3d_read_msh(const char *path, fe_mesh3d **out)
{
  GUARD_BEGIN
  if(!out || !path) { set_error("null argument"); return FE_INVALID_ARG; }
  std::unique_ptr<fe_mesh3d> m(new fe_mesh3d());
  FE_TRY(mesh3d_read_msh41(m->m, path));
  *out = m.release();
  return FE_OK;
  GUARD_END
}

int fe_mesh3d_from_arrays(int64_t nv, const double *x, const double *y, const double *z, int64_t nt,
                          const int32_t *tet, int64_t nb, const int32_t *bnd, fe_mesh3d **out)
{
  GUARD_BEGIN
  if(!out || nv <= 0 || nt <= 0 || nb < 0 || !x || !y || !z || !tet || (nb > 0 && !bnd)) {
    set_error("invalid arguments");
    return FE_INVALID_ARG;
  }
  std::unique_ptr<fe_mesh3d> m(new fe_mesh3d());
  m->m.x.assign(x, x + nv);
  m->m.y.assign(y, y + nv);
  m->m.z.assign(z, z + nv);
  m->m.tet.assign(tet, tet + 4 * nt);
  if(nb > 0) m->m.bnd.assign(bnd, bnd + 3 * nb);
  FE_TRY(m->m.build_topology());
  *out = m.release();
  return FE_OK;
  GUARD_END
}

int fe_mesh3d_write_msh(const fe_mesh3d *m, const char *path)
{
  GUARD_BEGIN
  if(!m || !path) { set_error("null argument"); return FE_INVALID_ARG; }
  return mesh3d_write_msh41(m->m, path);
  GUARD_END
}

int fe_mesh3d_sizes(const fe_mesh3d *m, int64_t *nv, int64_t *nt, int64_t *nb)
{
  if(!m) { set_error("null mesh"); return FE_INVALID_ARG; }
  if(nv) *nv = m->m.n_vertices();
  if(nt) *nt = m->m.n_tets();
  if(nb) *nb = m->m.n_boundary();
  return FE_OK;
}

int fe_mesh3d_arrays(const fe_mesh3d *m, double *x, double *y, double *z, int32_t *tet, int32_t *bnd)
{
  if(!m) { set_error("null mesh"); return FE_INVALID_ARG; }
  const Mesh3D &M = m->m;
  if(x) std::copy(M.x.begin(), M.x.end(), x);
  if(y) std::copy(M.y.begin(), M.y.end(), y);
  if(z) std::copy(M.z.begin(), M.z.end(), z);
  if(tet) std::copy(M.tet.begin(), M.tet.end(), tet);
  if(bnd) std::copy(M.bnd.begin(), M.bnd.end(), bnd);
  return FE_OK;
}

void fe_mesh3d_destroy(fe_mesh3d *m) { delete m; }

static int to_spaces(const fe_space_desc *spaces, int n, std::vector<SpaceDesc> &out)
{
  if(!spaces || n <= 0) { set_error("no spaces"); return FE_INVALID_ARG; }
  out.resize(n);
  for(int i = 0; i < n; ++i) {
    out[i] = {spaces[i].field, spaces[i].degree, spaces[i].ncomp, spaces[i].cnc, spaces[i].essential};
    if(out[i].field < 0 || out[i].field > 7 || out[i].cnc < 0 || out[i].cnc > 2) {
      set_error("invalid space %d", i);
      return FE_INVALID_ARG;
    }
  }
  return FE_OK;
}

// Block-Jacobi partition: unknowns grouped by the smallest mesh vertex
// they touch, in contiguous vertex ranges, so a block holds the velocity and
// pressure unknowns of one patch (velocity rows first, as numbered).
// Saddle-point rows (the pressure field, whose diagonal no form fills) get a
// nonzero ILU(0) pivot only through eliminated velocity unknowns of the same
// block: a pressure row with no velocity unknown in its block (next to
// essential velocities at a block border) joins the block of its first
// coupled velocity unknown.
static void block_partition(const Numbering &num, const CSRPattern &pat, const int32_t *edge_v, int64_t nEdges,
                            int64_t nv, int pc_block_rows, bool saddle, int fieldU, int fieldP,
                            std::vector<int32_t> &blockOfRow)
{
  const int64_t nInc = num.nInc;
  const int64_t nb = pc_block_rows > 0 ? std::max<int64_t>(1, nInc / pc_block_rows) : 1;
  std::vector<int64_t> key(num.nDofs, 0);
  for(int f = 0; f < num.nFields; ++f) {
    const int C = num.fieldComp[f];
    for(int64_t v = 0; v < nv; ++v)
      for(int c = 0; c < C; ++c) {
        int64_t d = num.vdof[f][v * C + c];
        if(d >= 0) key[d] = v;
      }
    for(int64_t e = 0; e < nEdges; ++e)
      for(int c = 0; c < C; ++c) {
        int64_t d = num.edof[f][e * C + c];
        if(d >= 0) key[d] = std::min(edge_v[2 * e], edge_v[2 * e + 1]);
      }
  }
  blockOfRow.resize(nInc);
  for(int64_t i = 0; i < nInc; ++i) blockOfRow[i] = (int32_t)((key[i] * nb) / nv);
  if(saddle && nb > 1) {
    for(int64_t i = 0; i < nInc; ++i) {
      if(num.dof_field[i] != fieldP) continue;
      int64_t firstU = -1;
      bool inBlock = false;
      for(int64_t k = pat.ia[i]; k < pat.ia[i + 1]; ++k) {
        const int32_t j = pat.ja[k];
        if(num.dof_field[j] != fieldU) continue;
        if(firstU < 0) firstU = j;
        if(blockOfRow[j] == blockOfRow[i]) { inBlock = true; break; }
      }
      if(!inBlock && firstU >= 0) blockOfRow[i] = blockOfRow[firstU];
    }
  }
}

int fe_setup_create(const fe_mesh *m, const fe_space_desc *spaces, int nspaces, int elem_type,
                    int quad_degree, int pc_block_rows, fe_setup **out)
{
  GUARD_BEGIN
  if(!m || !out) { set_error("null argument"); return FE_INVALID_ARG; }
  if(pc_block_rows < 0) { set_error("negative block size"); return FE_INVALID_ARG; }
  std::vector<SpaceDesc> sp;
  FE_TRY(to_spaces(spaces, nspaces, sp));
  std::unique_ptr<fe_setup> S(new fe_setup());
  const Mesh2D &M = m->m;
  FE_TRY(build_numbering(M, sp, S->num));
  S->spaces = sp;
  S->nVertices = M.n_vertices();
  S->nEdges = M.n_edges;
  // The element's fields: the P2 space on the domain, and for Taylor-Hood the
  // P1 space on the domain.
  int fieldU = -1, fieldP = -1;
  for(const SpaceDesc &d : sp) {
    if(d.cnc != CNC_DOMAIN) continue;
    if(d.degree == 2 && fieldU < 0) fieldU = d.field;
    if(d.degree == 1 && fieldP < 0) fieldP = d.field;
  }
  FE_TRY(build_element_tables(M, S->num, elem_type, fieldU,
                              elem_type == ELEM_TAYLOR_HOOD ? fieldP : -1, S->et));
  FE_TRY(color_elements(M, S->col));
  FE_TRY(build_csr_pattern_auto(S->et, S->num.nInc, S->pat, &S->patternOnDevice));
  FE_TRY(triangle_rule(quad_degree, S->quad));
  block_partition(S->num, S->pat, M.edge_v.data(), M.n_edges, M.n_vertices(), pc_block_rows,
                  elem_type == ELEM_TAYLOR_HOOD, fieldU, fieldP, S->blockOfRow);
  S->elemXY.resize(M.n_triangles() * 6);
  for(int64_t t = 0; t < M.n_triangles(); ++t)
    for(int k = 0; k < 3; ++k) {
      S->elemXY[6 * t + 2 * k] = M.x[M.tri[3 * t + k]];
      S->elemXY[6 * t + 2 * k + 1] = M.y[M.tri[3 * t + k]];
    }
  *out = S.release();
  return FE_OK;
  GUARD_END
}

int fe_setup3d_create(const fe_mesh3d *m, const fe_space_desc *spaces, int nspaces, int elem_type,
                      int pc_block_rows, fe_setup **out)
{
  GUARD_BEGIN
  if(!m || !out) { set_error("null argument"); return FE_INVALID_ARG; }
  if(pc_block_rows < 0) { set_error("negative block size"); return FE_INVALID_ARG; }
  if(elem_type != ELEM_TET_P2 && elem_type != ELEM_TET_TAYLOR_HOOD) {
    set_error("element type %d is not a tetrahedral type", elem_type);
    return FE_INVALID_ARG;
  }
  std::vector<SpaceDesc> sp;
  FE_TRY(to_spaces(spaces, nspaces, sp));
  std::unique_ptr<fe_setup> S(new fe_setup());
  const Mesh3D &M = m->m;
  S->tets = true;
  FE_TRY(build_numbering3d(M, sp, S->num));
  S->spaces = sp;
  S->nVertices = M.n_vertices();
  S->nEdges = M.n_edges;
  int fieldU = -1, fieldP = -1;
  for(const SpaceDesc &d : sp) {
    if(d.cnc != CNC_DOMAIN) continue;
    if(d.degree == 2 && fieldU < 0) fieldU = d.field;
    if(d.degree == 1 && fieldP < 0) fieldP = d.field;
  }
  FE_TRY(build_element_tables3d(M, S->num, elem_type, fieldU, elem_type == ELEM_TET_TAYLOR_HOOD ? fieldP : -1,
                                S->et));
  FE_TRY(color_elements3d(M, S->col));
  FE_TRY(build_csr_pattern_auto(S->et, S->num.nInc, S->pat, &S->patternOnDevice));
  block_partition(S->num, S->pat, M.edge_v.data(), M.n_edges, M.n_vertices(), pc_block_rows,
                  elem_type == ELEM_TET_TAYLOR_HOOD, fieldU, fieldP, S->blockOfRow);
  // vertex coordinates per tetrahedron: x0 y0 z0 ... x3 y3 z3
  S->elemXY.resize(M.n_tets() * 12);
  for(int64_t t = 0; t < M.n_tets(); ++t)
    for(int k = 0; k < 4; ++k) {
      const int32_t v = M.tet[4 * t + k];
      S->elemXY[12 * t + 3 * k] = M.x[v];
      S->elemXY[12 * t + 3 * k + 1] = M.y[v];
      S->elemXY[12 * t + 3 * k + 2] = M.z[v];
    }
  *out = S.release();
  return FE_OK;
  GUARD_END
}

int fe_setup_set_quadrature(fe_setup *s, int nq, const double *rule)
{
  GUARD_BEGIN
  if(!s || nq < 1 || !rule) { set_error("null argument or empty rule"); return FE_INVALID_ARG; }
  const int d = s->tets ? 3 : 2;
  QuadRule q;
  q.degree = s->quad.degree;
  for(int k = 0; k < nq; ++k) {
    q.r.push_back(rule[(d + 1) * k]);
    q.s.push_back(rule[(d + 1) * k + 1]);
    if(s->tets) q.t.push_back(rule[(d + 1) * k + 2]);
    q.w.push_back(rule[(d + 1) * k + d]);
  }
  s->quad = q;
  return FE_OK;
  GUARD_END
}

int fe_setup_get_dof_z(const fe_setup *s, double *z)
{
  if(!s) { set_error("null setup"); return FE_INVALID_ARG; }
  if(!s->tets) { set_error("a triangle set-up has no z coordinates"); return FE_INVALID_ARG; }
  if(z) std::copy(s->num.dof_z.begin(), s->num.dof_z.end(), z);
  return FE_OK;
}

void fe_setup_destroy(fe_setup *s) { delete s; }

int fe_setup_sizes(const fe_setup *s, int64_t *n_inc, int64_t *n_dofs, int64_t *nnz,
                   int64_t *n_elm, int *n_colors, int *nloc)
{
  if(!s) { set_error("null setup"); return FE_INVALID_ARG; }
  if(n_inc) *n_inc = s->num.nInc;
  if(n_dofs) *n_dofs = s->num.nDofs;
  if(nnz) *nnz = s->pat.nnz();
  if(n_elm) *n_elm = s->et.nElm;
  if(n_colors) *n_colors = s->col.nColors;
  if(nloc) *nloc = s->et.nloc;
  return FE_OK;
}

int fe_setup_get_pattern(const fe_setup *s, int64_t *ia, int32_t *ja)
{
  if(!s) { set_error("null setup"); return FE_INVALID_ARG; }
  if(ia) std::copy(s->pat.ia.begin(), s->pat.ia.end(), ia);
  if(ja) std::copy(s->pat.ja.begin(), s->pat.ja.end(), ja);
  return FE_OK;
}

int fe_setup_get_coloring(const fe_setup *s, int64_t *offsets, int32_t *elements)
{
  if(!s) { set_error("null setup"); return FE_INVALID_ARG; }
  if(offsets) std::copy(s->col.offsets.begin(), s->col.offsets.end(), offsets);
  if(elements) std::copy(s->col.elements.begin(), s->col.elements.end(), elements);
  return FE_OK;
}

int fe_setup_get_element_dofs(const fe_setup *s, int64_t *adr)
{
  if(!s) { set_error("null setup"); return FE_INVALID_ARG; }
  if(adr) std::copy(s->et.adr.begin(), s->et.adr.end(), adr);
  return FE_OK;
}

int fe_setup_get_dof_info(const fe_setup *s, double *x, double *y, int32_t *field, int32_t *comp,
                          int32_t *is_vertex)
{
  if(!s) { set_error("null setup"); return FE_INVALID_ARG; }
  const Numbering &n = s->num;
  if(x) std::copy(n.dof_x.begin(), n.dof_x.end(), x);
  if(y) std::copy(n.dof_y.begin(), n.dof_y.end(), y);
  if(field) std::copy(n.dof_field.begin(), n.dof_field.end(), field);
  if(comp) std::copy(n.dof_comp.begin(), n.dof_comp.end(), comp);
  if(is_vertex)
    for(size_t i = 0; i < n.dof_is_vertex.size(); ++i) is_vertex[i] = n.dof_is_vertex[i];
  return FE_OK;
}

int fe_setup_get_blocks(const fe_setup *s, int32_t *block_of_row)
{
  if(!s) { set_error("null setup"); return FE_INVALID_ARG; }
  if(block_of_row) std::copy(s->blockOfRow.begin(), s->blockOfRow.end(), block_of_row);
  return FE_OK;
}

int fe_tet_quadrature_rule(int degree, int *n, double *r, double *s, double *t, double *w)
{
  GUARD_BEGIN
  if(!n) { set_error("null argument"); return FE_INVALID_ARG; }
  QuadRule q;
  FE_TRY(tet_rule(degree, q));
  *n = q.n();
  if(r) std::copy(q.r.begin(), q.r.end(), r);
  if(s) std::copy(q.s.begin(), q.s.end(), s);
  if(t) std::copy(q.t.begin(), q.t.end(), t);
  if(w) std::copy(q.w.begin(), q.w.end(), w);
  return FE_OK;
  GUARD_END
}

int fe_quadrature_rule(int degree, int *n, double *r, double *s, double *w)
{
  GUARD_BEGIN
  QuadRule q;
  FE_TRY(triangle_rule(degree, q));
  if(n) *n = q.n();
  for(int k = 0; k < q.n(); ++k) {
    if(r) r[k] = q.r[k];
    if(s) s[k] = q.s[k];
    if(w) w[k] = q.w[k];
  }
  return FE_OK;
  GUARD_END
}

int fe_cuda_system_create(const fe_setup *setup, const fe_form_desc *forms, int nforms,
                          const fe_cuda_options *opt, fe_cuda_system **out)
{
  GUARD_BEGIN
  if(!setup || !out || (!forms && nforms > 0)) { set_error("null argument"); return FE_INVALID_ARG; }
  FE_TRY(check_options(opt));
  if(setup->tets) {
    // tetrahedra: the set-up's own rule when one was given
    // (fe_setup_set_quadrature), else the rule of the options' degree
  } else if(opt->quad_degree != setup->quad.degree) {
    set_error("options ask for quadrature degree %d, the set-up was built with %d",
              opt->quad_degree, setup->quad.degree);
    return FE_INVALID_ARG;
  }
  std::unique_ptr<fe_cuda_system> S(new fe_cuda_system());
  SystemTables T;
  T.elemType = setup->et.type;
  T.nElm = setup->et.nElm;
  T.nloc = setup->et.nloc;
  T.nInc = setup->num.nInc;
  T.nDofs = setup->num.nDofs;
  T.adr = setup->et.adr.data();
  T.elemXY = setup->elemXY.data();
  T.coloring = &setup->col;
  T.pattern = &setup->pat;
  // The set-up's partition targets its own block size; a different size in
  // the options re-partitions by contiguous index ranges.
  T.blockOfRow = &setup->blockOfRow;
  T.quad = setup->quad;
  if(setup->tets && setup->quad.n() == 0) FE_TRY(tet_rule(opt->quad_degree, T.quad));
  std::vector<FormDesc> fd;
  to_forms(forms, nforms, fd);
  FE_TRY(S->sys.init(T, fd.data(), nforms, to_sys_options(opt)));
  *out = S.release();
  return FE_OK;
  GUARD_END
}

int fe_cuda_system_create_from_tables(int elem_type, int64_t n_elm, const int64_t *adr,
                                      const double *elem_xy, int64_t n_inc, int64_t n_dofs,
                                      int n_colors, const int64_t *color_offsets,
                                      const int32_t *color_elements, const int64_t *ia,
                                      const int32_t *ja, const int32_t *block_of_row,
                                      const fe_form_desc *forms, int nforms,
                                      const fe_cuda_options *opt, fe_cuda_system **out)
{
  return fe_cuda_system_create_from_tables_rule(elem_type, n_elm, adr, elem_xy, n_inc, n_dofs, n_colors,
                                                color_offsets, color_elements, ia, ja, block_of_row, forms, nforms,
                                                opt, 0, nullptr, out);
}

int fe_cuda_system_create_from_tables_rule(int elem_type, int64_t n_elm, const int64_t *adr,
                                           const double *elem_xy, int64_t n_inc, int64_t n_dofs,
                                           int n_colors, const int64_t *color_offsets,
                                           const int32_t *color_elements, const int64_t *ia,
                                           const int32_t *ja, const int32_t *block_of_row,
                                           const fe_form_desc *forms, int nforms,
                                           const fe_cuda_options *opt, int nq, const double *rule,
                                           fe_cuda_system **out)
{
  GUARD_BEGIN
  if(!out || !adr || !elem_xy || (!forms && nforms > 0) || (nq > 0 && !rule) || nq < 0) {
    set_error("null argument or negative rule size");
    return FE_INVALID_ARG;
  }
  FE_TRY(check_options(opt));
  std::unique_ptr<fe_cuda_system> S(new fe_cuda_system());
  const bool tet = elem_type == ELEM_TET_P2 || elem_type == ELEM_TET_TAYLOR_HOOD;
  const int nloc = elem_type == ELEM_P2 ? 6 : elem_type == ELEM_TAYLOR_HOOD ? 15 : elem_type == ELEM_TET_P2 ? 10
                 : elem_type == ELEM_TET_TAYLOR_HOOD ? 34 : 0;
  if(!nloc) { set_error("unknown element type %d", elem_type); return FE_INVALID_ARG; }
  SystemTables T;
  T.elemType = elem_type;
  T.nElm = n_elm;
  T.nloc = nloc;
  T.nInc = n_inc;
  T.nDofs = n_dofs;
  T.adr = adr;
  T.elemXY = elem_xy;
  Coloring col;
  if(color_offsets && color_elements && n_colors > 0) {
    if(n_colors > MAX_COLORS) { set_error("at most %d colors", MAX_COLORS); return FE_BAD_COLORING; }
    col.nColors = n_colors;
    col.offsets.assign(color_offsets, color_offsets + n_colors + 1);
    col.elements.assign(color_elements, color_elements + n_elm);
    if(col.offsets[0] != 0 || col.offsets[n_colors] != n_elm) { set_error("color offsets do not cover the elements"); return FE_BAD_COLORING; }
    T.coloring = &col;
  }
  CSRPattern pat;
  if(ia && ja) {
    pat.n = n_inc;
    pat.ia.assign(ia, ia + n_inc + 1);
    if(pat.ia[0] != 0 || pat.ia[n_inc] < n_inc) { set_error("invalid CSR row pointers"); return FE_INVALID_ARG; }
    for(int64_t r = 0; r < n_inc; ++r)
      if(pat.ia[r + 1] < pat.ia[r]) { set_error("CSR row pointers decrease at row %lld", (long long)r); return FE_INVALID_ARG; }
    pat.ja.assign(ja, ja + pat.ia[n_inc]);
    for(int64_t r = 0; r < n_inc; ++r)
      for(int64_t k = pat.ia[r]; k < pat.ia[r + 1]; ++k)
        if(pat.ja[k] < 0 || pat.ja[k] >= n_inc || (k > pat.ia[r] && pat.ja[k] <= pat.ja[k - 1])) {
          set_error("CSR columns of row %lld are out of range or not strictly ascending", (long long)r);
          return FE_INVALID_ARG;
        }
    T.pattern = &pat;
  }
  std::vector<int32_t> blocks;
  if(block_of_row) {
    blocks.assign(block_of_row, block_of_row + n_inc);
    for(int32_t b : blocks)
      if(b < 0) { set_error("negative block id"); return FE_INVALID_ARG; }
    T.blockOfRow = &blocks;
  }
  if(nq > 0) {
    // the caller's rule, rows (r, s, [t,] w): the reference's own values
    // (feSpace::getRQuadraturePoints etc.) reproduce its sums exactly
    const int d = tet ? 3 : 2;
    T.quad = QuadRule();
    T.quad.degree = opt->quad_degree;
    for(int k = 0; k < nq; ++k) {
      T.quad.r.push_back(rule[(d + 1) * k]);
      T.quad.s.push_back(rule[(d + 1) * k + 1]);
      if(tet) T.quad.t.push_back(rule[(d + 1) * k + 2]);
      T.quad.w.push_back(rule[(d + 1) * k + d]);
    }
  } else if(tet) {
    FE_TRY(tet_rule(opt->quad_degree, T.quad));
  } else {
    FE_TRY(triangle_rule(opt->quad_degree, T.quad));
  }
  std::vector<FormDesc> fd;
  to_forms(forms, nforms, fd);
  // init range-checks the DOF ids and validates the coloring before use
  FE_TRY(S->sys.init(T, fd.data(), nforms, to_sys_options(opt)));
  *out = S.release();
  return FE_OK;
  GUARD_END
}

void fe_cuda_system_destroy(fe_cuda_system *s) { delete s; }

int fe_cuda_system_sizes(const fe_cuda_system *s, int64_t *n_inc, int64_t *n_dofs, int64_t *nnz,
                         int64_t *n_elm, int *n_colors)
{
  if(!s) { set_error("null system"); return FE_INVALID_ARG; }
  if(n_inc) *n_inc = s->sys.nInc();
  if(n_dofs) *n_dofs = s->sys.nDofs();
  if(nnz) *nnz = s->sys.nnz();
  if(n_elm) *n_elm = s->sys.nElm();
  if(n_colors) *n_colors = s->sys.nColors();
  return FE_OK;
}

int fe_cuda_get_pattern(const fe_cuda_system *s, int64_t *ia, int32_t *ja)
{
  if(!s) { set_error("null system"); return FE_INVALID_ARG; }
  const CSRPattern &p = s->sys.pattern();
  if(ia) std::copy(p.ia.begin(), p.ia.end(), ia);
  if(ja) std::copy(p.ja.begin(), p.ja.end(), ja);
  return FE_OK;
}

int fe_cuda_get_coloring(const fe_cuda_system *s, int64_t *offsets, int32_t *elements)
{
  if(!s) { set_error("null system"); return FE_INVALID_ARG; }
  const Coloring &c = s->sys.coloring();
  if(offsets) std::copy(c.offsets.begin(), c.offsets.end(), offsets);
  if(elements) std::copy(c.elements.begin(), c.elements.end(), elements);
  return FE_OK;
}

int fe_cuda_validate_coloring(const fe_cuda_system *s)
{
  if(!s) { set_error("null system"); return FE_INVALID_ARG; }
  return s->sys.validateColoring();
}

int fe_cuda_set_solution(fe_cuda_system *s, const double *u, const double *udot)
{
  if(!s) { set_error("null system"); return FE_INVALID_ARG; }
  return s->sys.setSolution(u, udot);
}

int fe_cuda_get_solution(const fe_cuda_system *s, double *u)
{
  if(!s || !u) { set_error("null argument"); return FE_INVALID_ARG; }
  return s->sys.getSolution(u);
}

int fe_cuda_norm_points(fe_cuda_system *s, int *nq, double *x, double *y)
{
  if(!s || !nq) { set_error("null argument"); return FE_INVALID_ARG; }
  return s->sys.normPoints(nq, x, y);
}

int fe_cuda_l2_error(fe_cuda_system *s, int field, const double *exact, double *error)
{
  if(!s || !exact || !error) { set_error("null argument"); return FE_INVALID_ARG; }
  return s->sys.l2Error(field, exact, error);
}

int fe_cuda_set_time(fe_cuda_system *s, double t, double c0)
{
  if(!s) { set_error("null system"); return FE_INVALID_ARG; }
  s->sys.setTime(t, c0);
  return FE_OK;
}

int fe_cuda_set_bdf(fe_cuda_system *s, int order, const double *cn, const double *hist1,
                    const double *hist2)
{
  if(!s || !cn) { set_error("null argument"); return FE_INVALID_ARG; }
  const double *h[3] = {nullptr, hist1, hist2};
  return s->sys.setBDF(order, cn, h);
}

int fe_cuda_compute_soldot(fe_cuda_system *s)
{
  if(!s) { set_error("null system"); return FE_INVALID_ARG; }
  return s->sys.computeSolDot();
}

int fe_cuda_set_to_zero(fe_cuda_system *s) { return s ? s->sys.setToZero() : FE_INVALID_ARG; }
int fe_cuda_set_matrix_to_zero(fe_cuda_system *s) { return s ? s->sys.setMatrixToZero() : FE_INVALID_ARG; }
int fe_cuda_set_residual_to_zero(fe_cuda_system *s) { return s ? s->sys.setResidualToZero() : FE_INVALID_ARG; }
int fe_cuda_assemble_residuals(fe_cuda_system *s) { return s ? s->sys.assembleResiduals() : FE_INVALID_ARG; }
int fe_cuda_assemble_matrices(fe_cuda_system *s) { return s ? s->sys.assembleMatrices() : FE_INVALID_ARG; }

int fe_cuda_get_rhs_max_norm(fe_cuda_system *s, double *norm)
{
  if(!s || !norm) { set_error("null argument"); return FE_INVALID_ARG; }
  return s->sys.getRHSMaxNorm(norm);
}

int fe_cuda_set_tolerances(fe_cuda_system *s, double rel_tol, double abs_tol, int max_iter)
{
  if(!s || !(rel_tol >= 0) || !(abs_tol >= 0) || max_iter < 1) {
    set_error("invalid tolerances");
    return FE_INVALID_ARG;
  }
  s->sys.krylov().opt.rtol = rel_tol;
  s->sys.krylov().opt.atol = abs_tol;
  s->sys.krylov().opt.maxIter = max_iter;
  return FE_OK;
}

int fe_cuda_solve(fe_cuda_system *s, double *norm_dx, double *norm_rhs, double *norm_axb, int *n_iter)
{
  if(!s) { set_error("null system"); return FE_INVALID_ARG; }
  return s->sys.solve(norm_dx, norm_rhs, norm_axb, n_iter);
}

int fe_cuda_correct_solution(fe_cuda_system *s) { return s ? s->sys.correctSolution() : FE_INVALID_ARG; }

int fe_cuda_get_matrix(const fe_cuda_system *s, double *values)
{
  if(!s || !values) { set_error("null argument"); return FE_INVALID_ARG; }
  return s->sys.getMatrix(values);
}

int fe_cuda_get_rhs(const fe_cuda_system *s, double *rhs)
{
  if(!s || !rhs) { set_error("null argument"); return FE_INVALID_ARG; }
  return s->sys.getRHS(rhs);
}

int fe_cuda_apply_preconditioner(fe_cuda_system *s, const double *r, double *z)
{
  GUARD_BEGIN
  if(!s || !r || !z) { set_error("null argument"); return FE_INVALID_ARG; }
  return s->sys.applyPreconditioner(r, z);
  GUARD_END
}

int fe_cuda_get_du(const fe_cuda_system *s, double *du)
{
  if(!s || !du) { set_error("null argument"); return FE_INVALID_ARG; }
  return s->sys.getDu(du);
}

int fe_setup_set_pattern_mode(int mode)
{
  return set_pattern_mode(mode);
}

int fe_setup_pattern_on_device(const fe_setup *s, int *on_device)
{
  if(!s || !on_device) { set_error("null argument"); return FE_INVALID_ARG; }
  *on_device = s->patternOnDevice;
  return FE_OK;
}

int fe_cuda_jacobian_route(const fe_cuda_system *s, int *route)
{
  if(!s || !route) { set_error("null argument"); return FE_INVALID_ARG; }
  *route = s->sys.jacobianRoute();
  return FE_OK;
}

int fe_cuda_get_du_max_norm(fe_cuda_system *s, double *norm)
{
  GUARD_BEGIN
  if(!s || !norm) { set_error("null argument"); return FE_INVALID_ARG; }
  *norm = s->sys.krylov().norminf(s->sys.dDu());
  if(!std::isfinite(*norm)) {
    set_error("non-finite Newton correction");
    return FE_NONFINITE;
  }
  return FE_OK;
  GUARD_END
}

int fe_cuda_newton(fe_cuda_system *s, const fe_newton_options *o, fe_newton_stats *st)
{
  GUARD_BEGIN
  if(!s || !o) { set_error("null argument"); return FE_INVALID_ARG; }
  NewtonOptions no;
  no.tolResidual = o->tol_residual;
  no.tolCorrection = o->tol_correction;
  no.tolDivergence = o->tol_divergence;
  no.maxIter = o->max_iter;
  no.recomputeEvery = o->recompute_every > 0 ? o->recompute_every : 3;
  no.residualDecrease = o->residual_decrease;
  no.stationary = o->stationary;
  no.relResidual = o->rel_residual;
  no.linearRtolMin = o->linear_rtol_min;
  no.residualScale = o->residual_scale;
  NewtonStats ns;
  const PhaseTimes before = s->sys.times;
  int r = newton_solve(s->sys, no, ns);
  if(st) {
    st->iterations = ns.iterations;
    st->krylov_iterations = ns.krylovIterations;
    st->matrix_assemblies = ns.matrixAssemblies;
    st->status = ns.status;
    st->residual0 = ns.residual0;
    st->residual = ns.residual;
    st->correction = ns.correction;
    st->residual_ms = s->sys.times.residual_ms - before.residual_ms;
    st->matrix_ms = s->sys.times.matrix_ms - before.matrix_ms;
    st->factor_ms = s->sys.times.factor_ms - before.factor_ms;
    st->solve_ms = s->sys.times.solve_ms - before.solve_ms;
  }
  return r;
  GUARD_END
}

int fe_cuda_get_times(const fe_cuda_system *s, double *residual_ms, double *matrix_ms,
                      double *factor_ms, double *solve_ms)
{
  if(!s) { set_error("null system"); return FE_INVALID_ARG; }
  if(residual_ms) *residual_ms = s->sys.times.residual_ms;
  if(matrix_ms) *matrix_ms = s->sys.times.matrix_ms;
  if(factor_ms) *factor_ms = s->sys.times.factor_ms;
  if(solve_ms) *solve_ms = s->sys.times.solve_ms;
  return FE_OK;
}

int fe_cuda_reset_times(fe_cuda_system *s)
{
  if(!s) { set_error("null system"); return FE_INVALID_ARG; }
  s->sys.times = PhaseTimes();
  return FE_OK;
}

int fe_cuda_smoother_bytes(fe_cuda_system *s, int64_t *bytes)
{
  GUARD_BEGIN
  if(!s || !bytes) { set_error("null argument"); return FE_INVALID_ARG; }
  // One step also computes the figure; run it on the system stream.
  const int r = s->sys.krylov().smootherStep(bytes);
  if(r != FE_OK) return r;
  if(cudaStreamSynchronize(s->sys.stream()) != cudaSuccess) {
    set_error("fe_cuda_smoother_bytes: device error");
    return FE_CUDA_DEVICE_FAIL;
  }
  return FE_OK;
  GUARD_END
}

int fe_cuda_phase_bytes(fe_cuda_system *s, int which, int64_t *bytes)
{
  GUARD_BEGIN
  if(!s || !bytes) { set_error("null argument"); return FE_INVALID_ARG; }
  if(which == 4) return fe_cuda_smoother_bytes(s, bytes);
  if(which < 5 || which > 9) { set_error("no byte count for phase %d", which); return FE_INVALID_ARG; }
  Krylov &k = s->sys.krylov();
  const int mode = which == 5 || which == 7 ? 0 : which == 6 || which == 8 ? 4 : 6;
  const int r = k.gsStep(mode, std::max(1, k.opt.restart / 2), bytes);
  if(r != FE_OK) return r;
  if(cudaStreamSynchronize(s->sys.stream()) != cudaSuccess) {
    set_error("fe_cuda_phase_bytes: device error");
    return FE_CUDA_DEVICE_FAIL;
  }
  return FE_OK;
  GUARD_END
}

int fe_cuda_bench_phase(fe_cuda_system *s, int which, int reps, int64_t flush_bytes, double *avg_ms)
{
  if(!s || !avg_ms || flush_bytes < 0) { set_error("invalid argument"); return FE_INVALID_ARG; }
  return s->sys.benchPhase(which, reps, (size_t)flush_bytes, avg_ms);
}

int fe_cuda_save_solution(fe_cuda_system *s)
{
  if(!s) { set_error("null system"); return FE_INVALID_ARG; }
  const size_t bytes = sizeof(double) * s->sys.nDofs();
  if(!s->saved && cudaMalloc(&s->saved, bytes) != cudaSuccess) {
    set_error("device allocation failed");
    return FE_CUDA_DEVICE_FAIL;
  }
  if(cudaMemcpyAsync(s->saved, s->sys.dU(), bytes, cudaMemcpyDeviceToDevice, s->sys.stream()) != cudaSuccess) {
    set_error("device copy failed");
    return FE_CUDA_DEVICE_FAIL;
  }
  return FE_OK;
}

int fe_cuda_restore_solution(fe_cuda_system *s)
{
  if(!s || !s->saved) { set_error("no saved solution"); return FE_INVALID_ARG; }
  if(cudaMemcpyAsync(s->sys.dU(), s->saved, sizeof(double) * s->sys.nDofs(), cudaMemcpyDeviceToDevice,
                     s->sys.stream()) != cudaSuccess) {
    set_error("device copy failed");
    return FE_CUDA_DEVICE_FAIL;
  }
  return FE_OK;
}

int fe_cuda_event_record(fe_cuda_system *s, int slot)
{
  if(!s || slot < 0 || slot > 7) { set_error("invalid event slot"); return FE_INVALID_ARG; }
  if(!s->ev[slot] && cudaEventCreate(&s->ev[slot]) != cudaSuccess) {
    set_error("event creation failed");
    return FE_CUDA_DEVICE_FAIL;
  }
  if(cudaEventRecord(s->ev[slot], s->sys.stream()) != cudaSuccess) {
    set_error("event record failed");
    return FE_CUDA_DEVICE_FAIL;
  }
  return FE_OK;
}

int fe_cuda_event_elapsed(fe_cuda_system *s, int slot0, int slot1, double *ms)
{
  if(!s || !ms || slot0 < 0 || slot0 > 7 || slot1 < 0 || slot1 > 7 || !s->ev[slot0] || !s->ev[slot1]) {
    set_error("invalid event slots");
    return FE_INVALID_ARG;
  }
  float f = 0.f;
  if(cudaEventSynchronize(s->ev[slot1]) != cudaSuccess ||
     cudaEventElapsedTime(&f, s->ev[slot0], s->ev[slot1]) != cudaSuccess) {
    set_error("event timing failed");
    return FE_CUDA_DEVICE_FAIL;
  }
  *ms = f;
  return FE_OK;
}

int fe_cuda_set_device(int device)
{
  if(cudaSetDevice(device) != cudaSuccess) {
    cudaGetLastError();
    set_error("cudaSetDevice(%d) failed", device);
    return FE_CUDA_DEVICE_FAIL;
  }
  return FE_OK;
}

int fe_cuda_launch_count(int64_t *count)
{
  if(!count) { set_error("null argument"); return FE_INVALID_ARG; }
  *count = g_launches.load();
  return FE_OK;
}

int fe_cuda_synchronize(fe_cuda_system *s)
{
  if(!s) { set_error("null system"); return FE_INVALID_ARG; }
  cudaError_t e = cudaStreamSynchronize(s->sys.stream());
  if(e != cudaSuccess) {
    set_error("stream synchronize: %s", cudaGetErrorString(e));
    return FE_CUDA_DEVICE_FAIL;
  }
  return FE_OK;
}

}  // extern "C"

// ---- BDF2 time integration with extrapolated / learned initial guesses ------

struct fe_transient {
  fe_cuda_system *sys = nullptr;
  Transient tr;
};

static NewtonOptions newton_options_of(const fe_newton_options *o)
{
  NewtonOptions no;
  no.tolResidual = o->tol_residual;
  no.tolCorrection = o->tol_correction;
  no.tolDivergence = o->tol_divergence;
  no.maxIter = o->max_iter;
  no.recomputeEvery = o->recompute_every > 0 ? o->recompute_every : 3;
  no.residualDecrease = o->residual_decrease;
  no.stationary = 0;
  no.relResidual = o->rel_residual;
  no.linearRtolMin = o->linear_rtol_min;
  no.residualScale = 0.0;  // set per step by the integrator
  return no;
}

extern "C" int fe_cuda_transient_create(fe_cuda_system *s, const fe_transient_options *o,
                                        const fe_newton_options *n, fe_transient **out)
{
  GUARD_BEGIN
  if(!s || !o || !n || !out) { set_error("null argument"); return FE_INVALID_ARG; }
  TransientOptions to;
  to.dt = o->dt;
  to.t0 = o->t0;
  to.guess = o->guess;
  to.trainFrom = o->train_from;
  to.useFrom = o->use_from;
  to.trainIters = o->train_iters;
  to.batch = o->batch;
  to.lr = o->lr;
  to.seed = o->seed;
  auto *t = new fe_transient();
  t->sys = s;
  const int r = t->tr.init(&s->sys, to, newton_options_of(n));
  if(r != FE_OK) {
    delete t;
    return r;
  }
  *out = t;
  return FE_OK;
  GUARD_END
}

extern "C" int fe_cuda_transient_steps(fe_transient *t, int nsteps, fe_step_stats *stats)
{
  GUARD_BEGIN
  if(!t || nsteps < 0) { set_error("null handle or negative step count"); return FE_INVALID_ARG; }
  for(int k = 0; k < nsteps; ++k) {
    StepStats st;
    const int r = t->tr.step(st);
    if(stats) {
      fe_step_stats &o = stats[k];
      o.step = st.step;
      o.newton_iterations = st.newtonIterations;
      o.krylov_iterations = st.krylovIterations;
      o.status = r != FE_OK ? r : st.status;
      o.guess_used = st.guessUsed;
      o.t = st.t;
      o.residual_ref = st.residualRef;
      o.residual_guess = st.residualGuess;
      o.residual_extrap = st.residualExtrap;
      o.residual = st.residual;
      o.step_ms = st.stepMs;
      o.guess_ms = st.guessMs;
      o.train_ms = st.trainMs;
      o.train_loss = st.trainLoss;
      o.guess_scale = st.guessScale;
    }
    if(r != FE_OK) return r;
  }
  return FE_OK;
  GUARD_END
}

extern "C" int fe_cuda_transient_get_network(const fe_transient *t, float *params)
{
  GUARD_BEGIN
  if(!t || !params) { set_error("null argument"); return FE_INVALID_ARG; }
  return t->tr.getNetwork(params);
  GUARD_END
}

extern "C" int fe_cuda_transient_set_network(fe_transient *t, const float *params)
{
  GUARD_BEGIN
  if(!t || !params) { set_error("null argument"); return FE_INVALID_ARG; }
  return t->tr.setNetwork(params);
  GUARD_END
}

extern "C" void fe_cuda_transient_destroy(fe_transient *t) { delete t; }

// ---- partially essential components and periodicity (feLinearSystem::
// constrainEssentialComponents / applyPeriodicity) -----------------------------

extern "C" int fe_cuda_set_constrained_rows(fe_cuda_system *s, const int64_t *rows, int64_t n)
{
  GUARD_BEGIN
  if(!s || (n > 0 && !rows) || n < 0) { set_error("null argument or negative count"); return FE_INVALID_ARG; }
  return s->sys.setConstrainedRows(rows, n);
  GUARD_END
}

extern "C" int fe_cuda_constrain_essential_components(fe_cuda_system *s)
{
  GUARD_BEGIN
  if(!s) { set_error("null argument"); return FE_INVALID_ARG; }
  return s->sys.constrainEssentialComponents();
  GUARD_END
}

extern "C" int fe_cuda_set_periodic_pairs(fe_cuda_system *s, const int64_t *master, const int64_t *slave, int64_t n)
{
  GUARD_BEGIN
  if(!s || (n > 0 && (!master || !slave)) || n < 0) { set_error("null argument or negative count"); return FE_INVALID_ARG; }
  return s->sys.setPeriodicPairs(master, slave, n);
  GUARD_END
}

extern "C" int fe_cuda_apply_periodicity(fe_cuda_system *s)
{
  GUARD_BEGIN
  if(!s) { set_error("null argument"); return FE_INVALID_ARG; }
  return s->sys.applyPeriodicity();
  GUARD_END
}

// Fields to export: those with a space on the domain, in the order of their
// first domain space, filtered by `required`, then reversed: the reference
// fills an unordered_map in space order and writes in its iteration order,
// which for the two fields of this path is the reverse.
static int export_fields(const fe_setup *s, const char *const *field_names, int n_field_names,
                         const char *const *required, int n_required, std::vector<ExportField> &fields)
{
  if(!field_names || n_required < 0 || (n_required > 0 && !required)) {
    set_error("null argument");
    return FE_INVALID_ARG;
  }
  if(n_field_names != s->num.nFields) {
    set_error("%d field names for %d fields", n_field_names, s->num.nFields);
    return FE_INVALID_ARG;
  }
  for(int f = 0; f < n_field_names; ++f)
    if(!field_names[f]) { set_error("null field name"); return FE_INVALID_ARG; }
  for(int i = 0; i < n_required; ++i) {
    if(!required[i]) { set_error("null field name"); return FE_INVALID_ARG; }
    bool known = false;
    for(int f = 0; f < n_field_names; ++f) known |= std::string(required[i]) == field_names[f];
    if(!known) { set_error("no field named \"%s\"", required[i]); return FE_INVALID_ARG; }
  }
  fields.clear();
  for(const SpaceDesc &d : s->spaces) {
    if(d.cnc != CNC_DOMAIN) continue;
    bool seen = false;
    for(const ExportField &e : fields) seen |= e.field == d.field;
    if(seen) continue;
    bool wanted = n_required == 0;
    for(int i = 0; i < n_required; ++i) wanted |= std::string(required[i]) == field_names[d.field];
    if(wanted) fields.push_back({d.field, field_names[d.field], d.degree});
  }
  std::reverse(fields.begin(), fields.end());
  return FE_OK;
}

int fe_export_vtk(const fe_mesh *m, const fe_setup *s, const double *solution,
                  const char *const *field_names, int n_field_names, const char *const *required,
                  int n_required, int precision, const char *path)
{
  GUARD_BEGIN
  if(!m || !s || !solution || !path) { set_error("null argument"); return FE_INVALID_ARG; }
  if(s->tets || m->m.n_vertices() != s->nVertices || m->m.n_edges != s->nEdges) {
    set_error("the setup was not built on this mesh");
    return FE_INVALID_ARG;
  }
  std::vector<ExportField> fields;
  FE_TRY(export_fields(s, field_names, n_field_names, required, n_required, fields));
  return export_vtk(m->m, s->num, solution, fields, precision == 0 ? 6 : precision, path);
  GUARD_END
}

int fe_export_vtk3d(const fe_mesh3d *m, const fe_setup *s, const double *solution,
                    const char *const *field_names, int n_field_names, const char *const *required,
                    int n_required, int precision, const char *path)
{
  GUARD_BEGIN
  if(!m || !s || !solution || !path) { set_error("null argument"); return FE_INVALID_ARG; }
  if(!s->tets || m->m.n_vertices() != s->nVertices || m->m.n_edges != s->nEdges) {
    set_error("the setup was not built on this mesh");
    return FE_INVALID_ARG;
  }
  std::vector<ExportField> fields;
  FE_TRY(export_fields(s, field_names, n_field_names, required, n_required, fields));
  return export_vtk3d(m->m, s->num, solution, fields, precision == 0 ? 6 : precision, path);
  GUARD_END
}
