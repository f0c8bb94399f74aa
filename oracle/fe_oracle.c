/* CPU oracle: see fe_oracle.h.  TEST INFRASTRUCTURE ONLY (checker and CPU
 * baseline); the product never links or calls it. */
#include "fe_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define PI 3.14159265358979323846

/* P2 Lagrange functions on the reference triangle (feSpace_2D.cpp:536-566,
 * 727-737) and P1 (feSpace_2D.cpp:118-131). */
static void p2(double r, double s, double L[6], double dr[6], double ds[6])
{
  L[0] = (1. - r - s) * (1. - 2. * r - 2. * s);
  L[1] = r * (2. * r - 1.);
  L[2] = s * (2. * s - 1.);
  L[3] = 4. * r * (1. - r - s);
  L[4] = 4. * r * s;
  L[5] = 4. * s * (1. - r - s);
  dr[0] = 4. * (r + s) - 3.; dr[1] = 4. * r - 1.; dr[2] = 0.;
  dr[3] = 4. * (1. - 2. * r - s); dr[4] = 4. * s; dr[5] = -4. * s;
  ds[0] = 4. * (r + s) - 3.; ds[1] = 0.; ds[2] = 4. * s - 1.;
  ds[3] = -4. * r; ds[4] = 4. * r; ds[5] = 4. * (1. - r - 2. * s);
}

static void source(int kind, const double *p, double x, double y, double f[2])
{
  f[0] = f[1] = 0.;
  if(kind == 1 || kind == 4) {
    f[0] = p[0] * sin(PI * x) * sin(PI * y);
  } else if(kind == 2) {
    /* manufactured NS source, tests/withLinearSolver/navier_stokes.cpp:33-51 */
    const double mdpdx0 = -2. * x * y * y, mdpdx1 = -2. * x * x * y;
    const double lap0 = 12. * (x * x * y * y * y * y + x * x * x * x * y * y);
    const double lap1 = -4. / 5. * (6. * x * y * y * y * y * y + 20. * x * x * x * y * y * y);
    const double u0 = x * x * x * x * y * y * y * y, u1 = -4. / 5. * x * x * x * y * y * y * y * y;
    const double g00 = 4. * x * x * x * y * y * y * y, g01 = -12. * x * x * y * y * y * y * y / 5.;
    const double g10 = 4. * x * x * x * x * y * y * y, g11 = -4. * x * x * x * y * y * y * y;
    const double c0 = u0 * g00 + u1 * g10, c1 = u0 * g01 + u1 * g11;
    f[0] = -(-c0 + mdpdx0 + lap0);
    f[1] = -(-c1 + mdpdx1 + lap1);
  } else if(kind == 3) {
    f[0] = p[0];
    f[1] = p[1];
  }
}

typedef struct geo {
  double x[3], y[3], jac, drdx[2], drdy[2];
} geo;

/* feCncGeo::computeElementTransformation for P1 triangles (feCncGeo.cpp:651-670). */
static void element_geo(const double *xy, geo *g)
{
  for(int k = 0; k < 3; ++k) { g->x[k] = xy[2 * k]; g->y[k] = xy[2 * k + 1]; }
  const double dxdr0 = g->x[1] - g->x[0], dxdr1 = g->y[1] - g->y[0];
  const double dxds0 = g->x[2] - g->x[0], dxds1 = g->y[2] - g->y[0];
  g->jac = dxdr0 * dxds1 - dxdr1 * dxds0;
  g->drdx[0] = dxds1 / g->jac;
  g->drdx[1] = -dxdr1 / g->jac;
  g->drdy[0] = -dxds0 / g->jac;
  g->drdy[1] = dxdr0 / g->jac;
}

/* Vector P2 function i = 2a+c at a node: value and gradient tensor
 * g[m*2+n] = d/dx_m (phi_n) (feSpace.cpp:735-755). */
static void vec_phi(int i, const double L[6], const double gx[6], const double gy[6], double phi[2],
                    double g[4])
{
  const int a = i / 2, c = i % 2;
  phi[0] = c == 0 ? L[a] : 0.;
  phi[1] = c == 1 ? L[a] : 0.;
  g[0] = c == 0 ? gx[a] : 0.;
  g[1] = c == 1 ? gx[a] : 0.;
  g[2] = c == 0 ? gy[a] : 0.;
  g[3] = c == 1 ? gy[a] : 0.;
}

/* Local residual Be (and matrix Ae when Ae != NULL) of the fused forms. */
static void element_system(const fo_problem *p, const geo *G, const double *ue, const double *ude,
                           double c0, double *Be, double *Ae)
{
  const fo_forms *f = &p->forms;
  const int nl = p->nloc;
  for(int i = 0; i < nl; ++i) {
    Be[i] = 0.;
    if(Ae)
      for(int j = 0; j < nl; ++j) Ae[i * nl + j] = 0.;
  }
  for(int k = 0; k < p->nq; ++k) {
    double L[6], dr[6], ds[6], gx[6], gy[6];
    p2(p->qr[k], p->qs[k], L, dr, ds);
    const double psi[3] = {1. - p->qr[k] - p->qs[k], p->qr[k], p->qs[k]};
    const double jac = G->jac, w = p->qw[k];
    for(int a = 0; a < 6; ++a) {
      gx[a] = dr[a] * G->drdx[0] + ds[a] * G->drdx[1];
      gy[a] = dr[a] * G->drdy[0] + ds[a] * G->drdy[1];
    }
    const double px = G->x[0] * psi[0] + G->x[1] * psi[1] + G->x[2] * psi[2];
    const double py = G->y[0] * psi[0] + G->y[1] * psi[1] + G->y[2] * psi[2];
    double S[2];
    source(f->src_kind, f->src_param, px, py, S);

    if(p->elem_type == 1) {
      if(f->has_diff) {
        double gu[2] = {0., 0.};
        for(int b = 0; b < 6; ++b) { gu[0] += ue[b] * gx[b]; gu[1] += ue[b] * gy[b]; }
        for(int a = 0; a < 6; ++a) {
          Be[a] -= f->diff * gx[a] * gu[0] * jac * w;
          Be[a] -= f->diff * gy[a] * gu[1] * jac * w;
          if(Ae)
            for(int b = 0; b < 6; ++b) {
              Ae[a * 6 + b] += f->diff * gx[a] * gx[b] * jac * w;
              Ae[a * 6 + b] += f->diff * gy[a] * gy[b] * jac * w;
            }
        }
      }
      if(f->src_kind)
        for(int a = 0; a < 6; ++a) Be[a] -= L[a] * f->src_coeff * S[0] * jac * w;
      continue;
    }

    /* Taylor-Hood: velocity at the node, its gradient, pressure, udot */
    double u[2] = {0., 0.}, gu[4] = {0., 0., 0., 0.}, ud[2] = {0., 0.}, pp = 0.;
    for(int b = 0; b < 6; ++b) {
      const double ux = ue[2 * b], uy = ue[2 * b + 1];
      u[0] += ux * L[b]; u[1] += uy * L[b];
      gu[0] += ux * gx[b]; gu[1] += uy * gx[b];
      gu[2] += ux * gy[b]; gu[3] += uy * gy[b];
      if(f->has_mass) { ud[0] += ude[2 * b] * L[b]; ud[1] += ude[2 * b + 1] * L[b]; }
    }
    for(int j = 0; j < 3; ++j) pp += ue[12 + j] * psi[j];
    const double div_u = gu[0] + gu[3];
    const double udg[2] = {u[0] * gu[0] + u[1] * gu[2], u[0] * gu[1] + u[1] * gu[3]};
    const double sym[4] = {2. * gu[0], gu[1] + gu[2], gu[2] + gu[1], 2. * gu[3]};
    for(int i = 0; i < 12; ++i) {
      double phi_i[2], g_i[4];
      vec_phi(i, L, gx, gy, phi_i, g_i);
      const double div_i = g_i[0] + g_i[3];
      if(f->has_conv) Be[i] -= f->conv * (phi_i[0] * udg[0] + phi_i[1] * udg[1]) * jac * w;
      if(f->has_sigma) {
        const double dco = g_i[0] * sym[0] + g_i[1] * sym[1] + g_i[2] * sym[2] + g_i[3] * sym[3];
        Be[i] -= f->sigma * (pp * div_i - f->mu * dco) * jac * w;
      }
      if(f->has_mass) Be[i] -= f->mass * (ud[0] * phi_i[0] + ud[1] * phi_i[1]) * jac * w;
      if(f->src_kind) Be[i] -= f->src_coeff * (S[0] * phi_i[0] + S[1] * phi_i[1]) * jac * w;
      if(Ae) {
        for(int j = 0; j < 12; ++j) {
          double phi_j[2], g_j[4];
          vec_phi(j, L, gx, gy, phi_j, g_j);
          double v = 0.;
          if(f->has_conv) {
            const double r1 = u[0] * (g_j[0] * phi_i[0] + g_j[1] * phi_i[1]) +
                              u[1] * (g_j[2] * phi_i[0] + g_j[3] * phi_i[1]);
            const double r2 = phi_j[0] * (gu[0] * phi_i[0] + gu[1] * phi_i[1]) +
                              phi_j[1] * (gu[2] * phi_i[0] + gu[3] * phi_i[1]);
            Ae[i * 15 + j] += f->conv * (r1 + r2) * jac * w;
          }
          if(f->has_sigma) {
            const double dc = g_i[0] * g_j[0] + g_i[1] * g_j[1] + g_i[2] * g_j[2] + g_i[3] * g_j[3];
            const double dct = g_i[0] * g_j[0] + g_i[1] * g_j[2] + g_i[2] * g_j[1] + g_i[3] * g_j[3];
            Ae[i * 15 + j] += -f->sigma * f->mu * (dc + dct) * jac * w;
          }
          if(f->has_mass)
            Ae[i * 15 + j] += f->mass * c0 * (phi_i[0] * phi_j[0] + phi_i[1] * phi_j[1]) * jac * w;
          (void)v;
        }
        if(f->has_sigma)
          for(int j = 0; j < 3; ++j) Ae[i * 15 + 12 + j] += f->sigma * psi[j] * div_i * jac * w;
      }
    }
    if(f->has_divu)
      for(int j = 0; j < 3; ++j) {
        Be[12 + j] -= f->divu * div_u * psi[j] * jac * w;
        if(Ae)
          for(int i = 0; i < 12; ++i) {
            double phi_i[2], g_i[4];
            vec_phi(i, L, gx, gy, phi_i, g_i);
            Ae[(12 + j) * 15 + i] += f->divu * psi[j] * (g_i[0] + g_i[3]) * jac * w;
          }
      }
  }
}

static void gather(const fo_problem *p, int64_t e, const double *u, double *ue)
{
  for(int i = 0; i < p->nloc; ++i) ue[i] = u ? u[p->adr[e * p->nloc + i]] : 0.;
}

int fo_assemble_residual(const fo_problem *p, const double *u, const double *udot, double *rhs,
                         int64_t elem_begin, int64_t elem_end, int nthreads)
{
  const int nl = p->nloc;
  for(int c = 0; c < p->n_colors; ++c) {
    int64_t b = p->color_offsets[c], e = p->color_offsets[c + 1];
    if(b < elem_begin) b = elem_begin;
    if(e > elem_end) e = elem_end;
    if(e <= b) continue;
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 64)
    for(int64_t q = b; q < e; ++q) {
      const int64_t el = p->color_elements[q];
      double ue[15], ude[15], Be[15];
      geo G;
      element_geo(p->elem_xy + 6 * el, &G);
      gather(p, el, u, ue);
      gather(p, el, udot, ude);
      element_system(p, &G, ue, ude, 0., Be, NULL);
      for(int i = 0; i < nl; ++i) {
        const int64_t d = p->adr[el * nl + i];
        if(d < p->n_inc) rhs[d] += Be[i];
      }
    }
  }
  return 0;
}


int fo_assemble_matrix(const fo_problem *p, const double *u, double c0, double *values,
                       int64_t elem_begin, int64_t elem_end, int nthreads)
{
  const int nl = p->nloc;
  for(int c = 0; c < p->n_colors; ++c) {
    int64_t b = p->color_offsets[c], e = p->color_offsets[c + 1];
    if(b < elem_begin) b = elem_begin;
    if(e > elem_end) e = elem_end;
    if(e <= b) continue;
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 64)
    for(int64_t q = b; q < e; ++q) {
      const int64_t el = p->color_elements[q];
      double ue[15], Be[15], Ae[225];
      geo G;
      element_geo(p->elem_xy + 6 * el, &G);
      gather(p, el, u, ue);
      element_system(p, &G, ue, ue, c0, Be, Ae);
      /* MKL-style scatter: keep unknown rows/columns, visit them in
       * increasing global order and scan the CSR row linearly from the last
       * match (feLinearSystemMklPardiso.cpp:574-660). */
      const int64_t *adr = p->adr + el * nl;
      int ri[15], cj[15], nr = 0, nc = 0;
      for(int i = 0; i < nl; ++i)
        if(adr[i] < p->n_inc) ri[nr++] = i;
      for(int j = 0; j < nl; ++j)
        if(adr[j] < p->n_inc) cj[nc++] = j;
      for(int x = 1; x < nr; ++x)
        for(int y = x; y > 0 && adr[ri[y - 1]] > adr[ri[y]]; --y) { int t = ri[y]; ri[y] = ri[y - 1]; ri[y - 1] = t; }
      for(int x = 1; x < nc; ++x)
        for(int y = x; y > 0 && adr[cj[y - 1]] > adr[cj[y]]; --y) { int t = cj[y]; cj[y] = cj[y - 1]; cj[y - 1] = t; }
      for(int x = 0; x < nr; ++x) {
        const int i = ri[x];
        const int64_t beg = p->ia[adr[i]], num = p->ia[adr[i] + 1] - beg;
        int64_t start = 0;
        for(int y = 0; y < nc; ++y) {
          const int j = cj[y];
          /* the pressure-pressure block holds no form */
          if(p->elem_type == 2 && i >= 12 && j >= 12) continue;
          for(int64_t J = start; J < num; ++J)
            if(p->ja[beg + J] == adr[j]) {
              values[beg + J] += Ae[i * nl + j];
              start = J;
              break;
            }
        }
      }
    }
  }
  return 0;
}

void fo_spmv(int64_t n, const int64_t *ia, const int32_t *ja, const double *a, const double *x,
             double *y, int nthreads)
{
#pragma omp parallel for num_threads(nthreads) schedule(static)
  for(int64_t i = 0; i < n; ++i) {
    double s = 0.;
    for(int64_t k = ia[i]; k < ia[i + 1]; ++k) s += a[k] * x[ja[k]];
    y[i] = s;
  }
}

/* ---------------------------------------------------------------------------
 * Preconditioners
 * ------------------------------------------------------------------------- */
struct fo_precond {
  int kind;
  int64_t n;
  const int64_t *ia;
  const int32_t *ja;
  /* ILU restricted to a row subset (block-diagonal part among 'active' rows) */
  int64_t nb;
  int64_t *bstart;   /* [nb+1] into perm */
  int32_t *perm;     /* active rows by block, ascending */
  int64_t *lia;      /* [n+1] */
  int32_t *lja;      /* local entries: global column */
  int64_t *src;      /* position in the full CSR */
  int64_t *ldiag;    /* [n] */
  double *f;         /* factor values */
  double *dinv;      /* Jacobi */
  /* Schur */
  const int32_t *isp;
  double *pscale;    /* viscosity / lumped mass for pressure rows */
  double *tmp;
  const double *A;   /* current matrix values (for the G z_p product) */
  fo_spmg *spmg;     /* kinds 4, 5 */
};

fo_precond *fo_precond_from_spmg(fo_spmg *S)
{
  fo_precond *pc = calloc(1, sizeof(fo_precond));
  pc->kind = 4;
  pc->spmg = S;
  return pc;
}

fo_precond *fo_precond_create(int kind, int64_t n, const int64_t *ia, const int32_t *ja,
                              const int32_t *block_of_row, const int32_t *is_pressure,
                              const double *pmass_lumped, double viscosity)
{
  fo_precond *pc = calloc(1, sizeof(fo_precond));
  pc->kind = kind;
  pc->n = n;
  pc->ia = ia;
  pc->ja = ja;
  pc->isp = is_pressure;
  if(kind == 2) pc->dinv = malloc(sizeof(double) * n);
  if(kind == 1 || kind == 3) {
    int64_t nb = 1;
    if(block_of_row)
      for(int64_t i = 0; i < n; ++i)
        if(block_of_row[i] + 1 > nb) nb = block_of_row[i] + 1;
    pc->nb = nb;
    pc->bstart = calloc(nb + 1, sizeof(int64_t));
    pc->perm = malloc(sizeof(int32_t) * n);
    int64_t cnt = 0;
    for(int64_t i = 0; i < n; ++i) {
      if(kind == 3 && is_pressure[i]) continue;
      pc->bstart[(block_of_row ? block_of_row[i] : 0) + 1]++;
      cnt++;
    }
    for(int64_t b = 0; b < nb; ++b) pc->bstart[b + 1] += pc->bstart[b];
    int64_t *fill = malloc(sizeof(int64_t) * nb);
    for(int64_t b = 0; b < nb; ++b) fill[b] = pc->bstart[b];
    for(int64_t i = 0; i < n; ++i) {
      if(kind == 3 && is_pressure[i]) continue;
      pc->perm[fill[block_of_row ? block_of_row[i] : 0]++] = (int32_t)i;
    }
    free(fill);
    pc->lia = calloc(n + 1, sizeof(int64_t));
    pc->ldiag = malloc(sizeof(int64_t) * n);
    int64_t nnz = ia[n];
    pc->lja = malloc(sizeof(int32_t) * nnz);
    pc->src = malloc(sizeof(int64_t) * nnz);
    int64_t pos = 0;
    for(int64_t i = 0; i < n; ++i) {
      pc->ldiag[i] = -1;
      const int active = !(kind == 3 && is_pressure[i]);
      const int32_t bi = block_of_row ? block_of_row[i] : 0;
      if(active)
        for(int64_t k = ia[i]; k < ia[i + 1]; ++k) {
          const int32_t j = ja[k];
          if(kind == 3 && is_pressure[j]) continue;
          if((block_of_row ? block_of_row[j] : 0) != bi) continue;
          if(j == i) pc->ldiag[i] = pos;
          pc->lja[pos] = j;
          pc->src[pos] = k;
          pos++;
        }
      pc->lia[i + 1] = pos;
    }
    pc->f = malloc(sizeof(double) * (pos > 0 ? pos : 1));
  }
  if(kind == 3) {
    pc->pscale = malloc(sizeof(double) * n);
    for(int64_t i = 0; i < n; ++i) pc->pscale[i] = is_pressure[i] ? viscosity / pmass_lumped[i] : 0.;
    pc->tmp = malloc(sizeof(double) * n);
  }
  return pc;
}

int fo_precond_factor(fo_precond *pc, const double *a)
{
  pc->A = a;
  if(pc->kind == 4) return fo_spmg_factor(pc->spmg, a);
  if(pc->kind == 2) {
    for(int64_t i = 0; i < pc->n; ++i) {
      double d = 0.;
      for(int64_t k = pc->ia[i]; k < pc->ia[i + 1]; ++k)
        if(pc->ja[k] == i) d = a[k];
      if(d == 0.) return -6;
      pc->dinv[i] = 1. / d;
    }
    return 0;
  }
  if(pc->kind != 1 && pc->kind != 3) return 0;
  int bad = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(| : bad)
  for(int64_t b = 0; b < pc->nb; ++b) {
    for(int64_t q = pc->bstart[b]; q < pc->bstart[b + 1]; ++q) {
      const int32_t i = pc->perm[q];
      const int64_t rb = pc->lia[i], re = pc->lia[i + 1], rd = pc->ldiag[i];
      for(int64_t k = rb; k < re; ++k) pc->f[k] = a[pc->src[k]];
      if(rd < 0) { bad = 1; break; }
      for(int64_t kk = rb; kk < rd; ++kk) {
        const int32_t kr = pc->lja[kk];
        const double piv = pc->f[pc->ldiag[kr]];
        if(piv == 0.) { bad = 1; break; }
        const double lik = pc->f[kk] / piv;
        pc->f[kk] = lik;
        int64_t p2 = pc->ldiag[kr] + 1;
        const int64_t pe = pc->lia[kr + 1];
        for(int64_t jj = kk + 1; jj < re && p2 < pe; ++jj) {
          const int32_t col = pc->lja[jj];
          while(p2 < pe && pc->lja[p2] < col) ++p2;
          if(p2 < pe && pc->lja[p2] == col) pc->f[jj] -= lik * pc->f[p2];
        }
      }
      if(bad || pc->f[rd] == 0. || !isfinite(pc->f[rd])) { bad = 1; break; }
    }
  }
  return bad ? -6 : 0;
}

static void ilu_apply(fo_precond *pc, const double *r, double *z)
{
#pragma omp parallel for schedule(dynamic, 1)
  for(int64_t b = 0; b < pc->nb; ++b) {
    const int64_t qb = pc->bstart[b], qe = pc->bstart[b + 1];
    for(int64_t q = qb; q < qe; ++q) {
      const int32_t i = pc->perm[q];
      double s = r[i];
      for(int64_t k = pc->lia[i]; k < pc->ldiag[i]; ++k) s -= pc->f[k] * z[pc->lja[k]];
      z[i] = s;
    }
    for(int64_t q = qe - 1; q >= qb; --q) {
      const int32_t i = pc->perm[q];
      double s = z[i];
      for(int64_t k = pc->ldiag[i] + 1; k < pc->lia[i + 1]; ++k) s -= pc->f[k] * z[pc->lja[k]];
      z[i] = s / pc->f[pc->ldiag[i]];
    }
  }
}

void fo_precond_apply(fo_precond *pc, const double *r, double *z)
{
  const int64_t n = pc->n;
  if(pc->kind == 4) {
    fo_spmg_apply(pc->spmg, r, z);
  } else if(pc->kind == 0) {
    memcpy(z, r, sizeof(double) * n);
  } else if(pc->kind == 2) {
    for(int64_t i = 0; i < n; ++i) z[i] = r[i] * pc->dinv[i];
  } else if(pc->kind == 1) {
    ilu_apply(pc, r, z);
  } else {
    /* block upper-triangular: z_p = S^-1 r_p with S ~ M_p / viscosity,
     * z_u = A_uu^-1 (r_u - A_up z_p) */
    for(int64_t i = 0; i < n; ++i) z[i] = pc->isp[i] ? pc->pscale[i] * r[i] : 0.;
    for(int64_t i = 0; i < n; ++i) {
      if(pc->isp[i]) continue;
      double s = r[i];
      for(int64_t k = pc->ia[i]; k < pc->ia[i + 1]; ++k)
        if(pc->isp[pc->ja[k]]) s -= pc->A[k] * z[pc->ja[k]];
      pc->tmp[i] = s;
    }
    ilu_apply(pc, pc->tmp, z);
  }
}

void fo_precond_destroy(fo_precond *pc)
{
  if(!pc) return;  /* a kind-4 object does not own its multigrid (fo_spmg_destroy) */
  free(pc->bstart); free(pc->perm); free(pc->lia); free(pc->lja); free(pc->src);
  free(pc->ldiag); free(pc->f); free(pc->dinv); free(pc->pscale); free(pc->tmp);
  free(pc);
}

/* ---------------------------------------------------------------------------
 * Krylov
 * ------------------------------------------------------------------------- */
#define FO_MAX_RESTART 200

static double dot(int64_t n, const double *x, const double *y, int nt)
{
  double s = 0.;
#pragma omp parallel for num_threads(nt) reduction(+ : s) schedule(static)
  for(int64_t i = 0; i < n; ++i) s += x[i] * y[i];
  return s;
}

int fo_krylov_solve(int method, int m, int max_iter, double rtol, double atol, int64_t n,
                    const int64_t *ia, const int32_t *ja, const double *a, fo_precond *pc,
                    const double *b, double *x, fo_krylov_stats *st, int nt)
{
  memset(st, 0, sizeof(*st));
  for(int64_t i = 0; i < n; ++i) x[i] = 0.;
  const double bn = sqrt(dot(n, b, b, nt));
  st->rnorm0 = bn;
  const double tol = fmax(rtol * bn, atol);
  if(bn <= atol) { st->converged = 1; st->rnorm = bn; return 0; }
  if(method == 0) {
    double *r = malloc(sizeof(double) * n), *z = malloc(sizeof(double) * n);
    double *p = malloc(sizeof(double) * n), *q = malloc(sizeof(double) * n);
    memcpy(r, b, sizeof(double) * n);
    fo_precond_apply(pc, r, z);
    memcpy(p, z, sizeof(double) * n);
    double rz = dot(n, r, z, nt), rr = bn * bn;
    int it = 0;
    while(it < max_iter && sqrt(rr) > tol) {
      fo_spmv(n, ia, ja, a, p, q, nt);
      const double alpha = rz / dot(n, p, q, nt);
#pragma omp parallel for num_threads(nt) schedule(static)
      for(int64_t i = 0; i < n; ++i) { x[i] += alpha * p[i]; r[i] -= alpha * q[i]; }
      rr = dot(n, r, r, nt);
      fo_precond_apply(pc, r, z);
      const double rzn = dot(n, r, z, nt);
      const double beta = rzn / rz;
      rz = rzn;
#pragma omp parallel for num_threads(nt) schedule(static)
      for(int64_t i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
      ++it;
    }
    st->iterations = it;
    st->rnorm = sqrt(rr);
    st->converged = st->rnorm <= tol;
    free(r); free(z); free(p); free(q);
    return st->converged ? 0 : -5;
  }
  /* FGMRES(m), right preconditioning, CGS2 Arnoldi */
  if(m < 1 || m > FO_MAX_RESTART) return -3;
  double *V = malloc(sizeof(double) * n * (m + 1)), *Z = malloc(sizeof(double) * n * m);
  double *w = malloc(sizeof(double) * n);
  double *H = calloc((size_t)(m + 1) * m, sizeof(double));
  double *cs = malloc(sizeof(double) * m), *sn = malloc(sizeof(double) * m);
  double *g = malloc(sizeof(double) * (m + 1)), *y = malloc(sizeof(double) * m);
  double *h = malloc(sizeof(double) * (m + 1));
  int total = 0;
  double est = bn;
  while(total < max_iter) {
    fo_spmv(n, ia, ja, a, x, w, nt);
#pragma omp parallel for num_threads(nt) schedule(static)
    for(int64_t i = 0; i < n; ++i) w[i] = b[i] - w[i];
    const double beta = sqrt(dot(n, w, w, nt));
    est = beta;
    if(beta <= tol) break;
#pragma omp parallel for num_threads(nt) schedule(static)
    for(int64_t i = 0; i < n; ++i) V[i] = w[i] / beta;
    for(int i = 0; i <= m; ++i) g[i] = 0.;
    g[0] = beta;
    int k = 0;
    for(int j = 0; j < m && total < max_iter; ++j) {
      fo_precond_apply(pc, V + (int64_t)j * n, Z + (int64_t)j * n);
      fo_spmv(n, ia, ja, a, Z + (int64_t)j * n, w, nt);
      for(int c = 0; c <= j; ++c) H[c * m + j] = 0.;
      for(int pass = 0; pass < 2; ++pass) {
        /* classical Gram-Schmidt: all products, then one update pass */
        for(int c = 0; c <= j; ++c) h[c] = 0.;
#pragma omp parallel num_threads(nt)
        {
          double hl[FO_MAX_RESTART + 1];
          for(int c = 0; c <= j; ++c) hl[c] = 0.;
#pragma omp for schedule(static)
          for(int64_t i = 0; i < n; ++i)
            for(int c = 0; c <= j; ++c) hl[c] += V[(int64_t)c * n + i] * w[i];
#pragma omp critical
          for(int c = 0; c <= j; ++c) h[c] += hl[c];
        }
        for(int c = 0; c <= j; ++c) H[c * m + j] += h[c];
#pragma omp parallel for num_threads(nt) schedule(static)
        for(int64_t i = 0; i < n; ++i) {
          double t = w[i];
          for(int c = 0; c <= j; ++c) t -= h[c] * V[(int64_t)c * n + i];
          w[i] = t;
        }
      }
      const double hn = sqrt(dot(n, w, w, nt));
      H[(j + 1) * m + j] = hn;
#pragma omp parallel for num_threads(nt) schedule(static)
      for(int64_t i = 0; i < n; ++i) V[(int64_t)(j + 1) * n + i] = hn > 0 ? w[i] / hn : 0.;
      for(int c = 0; c < j; ++c) {
        const double t = cs[c] * H[c * m + j] + sn[c] * H[(c + 1) * m + j];
        H[(c + 1) * m + j] = -sn[c] * H[c * m + j] + cs[c] * H[(c + 1) * m + j];
        H[c * m + j] = t;
      }
      const double aa = H[j * m + j], bb = H[(j + 1) * m + j], r = hypot(aa, bb);
      cs[j] = r > 0 ? aa / r : 1.;
      sn[j] = r > 0 ? bb / r : 0.;
      H[j * m + j] = r;
      H[(j + 1) * m + j] = 0.;
      g[j + 1] = -sn[j] * g[j];
      g[j] = cs[j] * g[j];
      est = fabs(g[j + 1]);
      ++total;
      k = j + 1;
      if(est <= tol || hn == 0.) break;
    }
    for(int i = k - 1; i >= 0; --i) {
      double s = g[i];
      for(int c = i + 1; c < k; ++c) s -= H[i * m + c] * y[c];
      y[i] = s / H[i * m + i];
    }
#pragma omp parallel for num_threads(nt) schedule(static)
    for(int64_t i = 0; i < n; ++i) {
      double t = x[i];
      for(int c = 0; c < k; ++c) t += y[c] * Z[(int64_t)c * n + i];
      x[i] = t;
    }
    if(est <= tol) break;
  }
  fo_spmv(n, ia, ja, a, x, w, nt);
#pragma omp parallel for num_threads(nt) schedule(static)
  for(int64_t i = 0; i < n; ++i) w[i] = b[i] - w[i];
  st->rnorm = sqrt(dot(n, w, w, nt));
  st->iterations = total;
  st->converged = est <= tol;
  free(V); free(Z); free(w); free(H); free(cs); free(sn); free(g); free(y); free(h);
  return st->converged ? 0 : -5;
}

/* ---- essential components and periodicity: restatement of
 * feLinearSystemMklPardiso::constrainEssentialComponents
 * (src/feLinearSystemMklPardiso.cpp:1082-1112: columns of every constrained
 * row zeroed, then the row zeroed with 1 on its diagonal, rhs 0) and
 * applyPeriodicity (:1119-1149: slave row = [1 at slave, -1 at master],
 * rhs 0).  Rows / pairs with an index >= n are ignored, as there. */
void fo_constrain(int64_t n, const int64_t *ia, const int32_t *ja, double *values, double *rhs,
                  const int64_t *rows, int64_t nrows)
{
  const int64_t nnz = ia[n];
  unsigned char *isc = calloc((size_t)n, 1);
  for(int64_t i = 0; i < nrows; ++i)
    if(rows[i] >= 0 && rows[i] < n) isc[rows[i]] = 1;
  for(int64_t k = 0; k < nnz; ++k)
    if(isc[ja[k]]) values[k] = 0.;
  for(int64_t r = 0; r < n; ++r) {
    if(!isc[r]) continue;
    for(int64_t k = ia[r]; k < ia[r + 1]; ++k) values[k] = ja[k] == r ? 1. : 0.;
    rhs[r] = 0.;
  }
  free(isc);
}

void fo_periodicity(int64_t n, const int64_t *ia, const int32_t *ja, double *values, double *rhs,
                    const int64_t *master, const int64_t *slave, int64_t npairs)
{
  for(int64_t p = 0; p < npairs; ++p) {
    const int64_t m = master[p], s = slave[p];
    if(m < 0 || s < 0 || m >= n || s >= n) continue;
    for(int64_t k = ia[s]; k < ia[s + 1]; ++k) values[k] = ja[k] == s ? 1. : (ja[k] == m ? -1. : 0.);
    rhs[s] = 0.;
  }
}

/* ---- element coloring: feCncGeo::colorElements algorithm 1
 * (src/feCncGeo.cpp:752-790).  Rounds over the uncolored elements in index
 * order: every uncolored element that is not yet blocked blocks its
 * uncolored vertex-neighbours; the elements left unblocked take the round's
 * color, the blocked ones are released for the next round. */
int fo_color_elements(const int32_t *ev, int nvpe, int64_t ne, int64_t nv, int32_t *color)
{
  int64_t *vs = calloc(nv + 1, sizeof(int64_t));
  for(int64_t i = 0; i < ne * nvpe; ++i) {
    if(ev[i] < 0 || ev[i] >= nv) { free(vs); return -3; }
    vs[ev[i] + 1]++;
  }
  for(int64_t v = 0; v < nv; ++v) vs[v + 1] += vs[v];
  int32_t *ve = malloc(sizeof(int32_t) * (ne * nvpe > 0 ? ne * nvpe : 1));
  int64_t *pos = malloc(sizeof(int64_t) * (nv > 0 ? nv : 1));
  memcpy(pos, vs, sizeof(int64_t) * nv);
  for(int64_t t = 0; t < ne; ++t)
    for(int k = 0; k < nvpe; ++k) ve[pos[ev[nvpe * t + k]]++] = (int32_t)t;
  free(pos);
  unsigned char *blk = calloc(ne > 0 ? ne : 1, 1);
  for(int64_t t = 0; t < ne; ++t) color[t] = -1;
  int64_t left = ne;
  int nc = 0;
  while(left > 0) {
    if(nc >= 64) { nc = -1; break; }
    for(int64_t t = 0; t < ne; ++t) {
      if(color[t] >= 0 || blk[t]) continue;
      for(int k = 0; k < nvpe; ++k) {
        const int32_t v = ev[nvpe * t + k];
        for(int64_t p = vs[v]; p < vs[v + 1]; ++p)
          if(ve[p] != t && color[ve[p]] < 0) blk[ve[p]] = 1;
      }
    }
    for(int64_t t = 0; t < ne; ++t) {
      if(color[t] >= 0) continue;
      if(blk[t]) blk[t] = 0;
      else { color[t] = nc; --left; }
    }
    ++nc;
  }
  free(vs); free(ve); free(blk);
  return nc;
}

/* Thread count of the OpenMP regions that take none explicitly (the
 * multigrid of fe_oracle_mg.c). */
void fo_set_threads(int n)
{
  if(n > 0) omp_set_num_threads(n);
}
