/* CPU oracle: smoothed-aggregation multigrid and the block-triangular
 * saddle-point preconditioner.  TEST INFRASTRUCTURE ONLY: the CPU baseline
 * and the reference arm of bench.py solve with it; the product never calls it.
 *
 * The reference's solves are library calls (PETSc KSP, MKL Pardiso:
 * src/feLinearSystemPETSc.cpp:900-1031, src/feLinearSystemMklPardiso.cpp:893-965)
 * that cannot be built here, and the configurations' FGMRES + block-Jacobi
 * ILU(0) does not converge on the Navier-Stokes Jacobians.  A CPU Newton solve
 * that converges therefore needs a saddle-point preconditioner; this file
 * restates, from the published methods, the one the device path uses:
 *   - smoothed aggregation (Vanek, Mandel, Brezina, Computing 56, 1996):
 *     strength |a_ij| >= theta sqrt(|a_ii a_jj|), greedy three-pass
 *     aggregation (the threshold halved while fewer than half of the rows
 *     aggregate), tentative prolongator with unit-norm columns, one damped
 *     Jacobi smoothing step (omega = 4 / (3 rho(D^-1 A))) except on levels
 *     denser than 64 entries per row (plain aggregation there), Galerkin
 *     coarse operators, dense inverse of the coarsest level;
 *   - V-cycles with one degree-1 Chebyshev (weighted Jacobi) sweep before and
 *     after the coarse correction, weight 1 / (0.7 rho);
 *   - the block upper-triangular preconditioner of Elman, Silvester and
 *     Wathen (Finite Elements and Fast Iterative Solvers, 2nd ed., ch. 9):
 *     z_p = S^-1 r_p with S^-1 ~ -6 (s / (1.5 sigma c_div)) M_p^-1 (lumped
 *     pressure mass) and the constant pressure mode deflated, then
 *     z_u = (s K)^-1 (r_u - G z_p) per velocity component by one V-cycle on
 *     the scalar P2 stiffness K, s = diag(A_uu) sum / diag(K) sum.
 * All loops over rows run on OpenMP threads.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "fe_oracle.h"

typedef struct {
  int64_t n, m;
  int64_t *ia;
  int32_t *ja;
  double *a;
} csr_t;

static void csr_free(csr_t *A)
{
  free(A->ia); free(A->ja); free(A->a);
  memset(A, 0, sizeof(*A));
}

/* C = A B: symbolic then numeric row pass with a dense marker per thread;
 * columns of each row sorted. */
static int cmp_i32(const void *x, const void *y)
{
  const int32_t a = *(const int32_t *)x, b = *(const int32_t *)y;
  return (a > b) - (a < b);
}

static csr_t spgemm(const csr_t *A, const csr_t *B)
{
  csr_t C = {A->n, B->m, calloc(A->n + 1, sizeof(int64_t)), NULL, NULL};
#pragma omp parallel
  {
    int64_t *mark = malloc(sizeof(int64_t) * (B->m > 0 ? B->m : 1));
    for(int64_t j = 0; j < B->m; ++j) mark[j] = -1;
#pragma omp for schedule(dynamic, 256)
    for(int64_t i = 0; i < A->n; ++i) {
      int64_t c = 0;
      for(int64_t k = A->ia[i]; k < A->ia[i + 1]; ++k)
        for(int64_t l = B->ia[A->ja[k]]; l < B->ia[A->ja[k] + 1]; ++l)
          if(mark[B->ja[l]] != i) { mark[B->ja[l]] = i; ++c; }
      C.ia[i + 1] = c;
    }
    free(mark);
  }
  for(int64_t i = 0; i < A->n; ++i) C.ia[i + 1] += C.ia[i];
  C.ja = malloc(sizeof(int32_t) * (C.ia[A->n] > 0 ? C.ia[A->n] : 1));
  C.a = malloc(sizeof(double) * (C.ia[A->n] > 0 ? C.ia[A->n] : 1));
#pragma omp parallel
  {
    int64_t *mark = malloc(sizeof(int64_t) * (B->m > 0 ? B->m : 1));
    double *acc = malloc(sizeof(double) * (B->m > 0 ? B->m : 1));
    for(int64_t j = 0; j < B->m; ++j) mark[j] = -1;
#pragma omp for schedule(dynamic, 256)
    for(int64_t i = 0; i < A->n; ++i) {
      int64_t o = C.ia[i];
      for(int64_t k = A->ia[i]; k < A->ia[i + 1]; ++k) {
        const double av = A->a[k];
        for(int64_t l = B->ia[A->ja[k]]; l < B->ia[A->ja[k] + 1]; ++l) {
          const int32_t c = B->ja[l];
          if(mark[c] != i) { mark[c] = i; acc[c] = 0.; C.ja[o++] = c; }
          acc[c] += av * B->a[l];
        }
      }
      qsort(C.ja + C.ia[i], (size_t)(o - C.ia[i]), sizeof(int32_t), cmp_i32);
      for(int64_t p = C.ia[i]; p < o; ++p) C.a[p] = acc[C.ja[p]];
    }
    free(mark);
    free(acc);
  }
  return C;
}

static csr_t transpose(const csr_t *A)
{
  const int64_t nnz = A->ia[A->n];
  csr_t T = {A->m, A->n, calloc(A->m + 1, sizeof(int64_t)), malloc(sizeof(int32_t) * (nnz > 0 ? nnz : 1)),
             malloc(sizeof(double) * (nnz > 0 ? nnz : 1))};
  for(int64_t k = 0; k < nnz; ++k) T.ia[A->ja[k] + 1]++;
  for(int64_t i = 0; i < A->m; ++i) T.ia[i + 1] += T.ia[i];
  int64_t *fill = malloc(sizeof(int64_t) * (A->m > 0 ? A->m : 1));
  memcpy(fill, T.ia, sizeof(int64_t) * A->m);
  for(int64_t i = 0; i < A->n; ++i)
    for(int64_t k = A->ia[i]; k < A->ia[i + 1]; ++k) {
      const int64_t p = fill[A->ja[k]]++;
      T.ja[p] = (int32_t)i;
      T.a[p] = A->a[k];
    }
  free(fill);
  return T;
}

/* rho(D^-1 A) by 20 power iterations from x_i = 1 + 0.1 sin(0.37 i). */
static double spectral_radius(const csr_t *A, const double *dinv)
{
  double *x = malloc(sizeof(double) * A->n), *y = malloc(sizeof(double) * A->n);
  for(int64_t i = 0; i < A->n; ++i) x[i] = 1.0 + 0.1 * sin(0.37 * (double)i);
  double lam = 1.;
  for(int it = 0; it < 20; ++it) {
    double nrm = 0., xn = 0.;
#pragma omp parallel for reduction(+ : nrm, xn) schedule(static)
    for(int64_t i = 0; i < A->n; ++i) {
      double s = 0.;
      for(int64_t k = A->ia[i]; k < A->ia[i + 1]; ++k) s += A->a[k] * x[A->ja[k]];
      y[i] = dinv[i] * s;
      nrm += y[i] * y[i];
      xn += x[i] * x[i];
    }
    nrm = sqrt(nrm);
    lam = nrm / sqrt(xn > 1e-300 ? xn : 1e-300);
    if(nrm == 0.) break;
    for(int64_t i = 0; i < A->n; ++i) x[i] = y[i] / nrm;
  }
  free(x);
  free(y);
  return lam;
}

static int64_t aggregate(const csr_t *A, double theta, int32_t *agg)
{
  const int64_t n = A->n;
  double *diag = calloc(n, sizeof(double));
  for(int64_t i = 0; i < n; ++i)
    for(int64_t k = A->ia[i]; k < A->ia[i + 1]; ++k)
      if(A->ja[k] == i) diag[i] = fabs(A->a[k]);
#define STRONG(i, k) (A->ja[k] != (i) && fabs(A->a[k]) >= theta * sqrt(diag[i] * diag[A->ja[k]]))
  for(int64_t i = 0; i < n; ++i) agg[i] = -1;
  int64_t na = 0;
  /* pass 1: roots whose strong neighbourhood is free */
  for(int64_t i = 0; i < n; ++i) {
    if(agg[i] >= 0) continue;
    int ok = 1, any = 0;
    for(int64_t k = A->ia[i]; k < A->ia[i + 1]; ++k)
      if(STRONG(i, k)) {
        any = 1;
        if(agg[A->ja[k]] >= 0) { ok = 0; break; }
      }
    if(!ok) continue;
    agg[i] = (int32_t)na;
    if(any)
      for(int64_t k = A->ia[i]; k < A->ia[i + 1]; ++k)
        if(STRONG(i, k)) agg[A->ja[k]] = (int32_t)na;
    ++na;
  }
  /* pass 2: join the most strongly connected aggregate of pass 1 */
  int32_t *agg1 = malloc(sizeof(int32_t) * (n > 0 ? n : 1));
  memcpy(agg1, agg, sizeof(int32_t) * n);
  for(int64_t i = 0; i < n; ++i) {
    if(agg1[i] >= 0) continue;
    double best = -1.;
    int32_t pick = -1;
    for(int64_t k = A->ia[i]; k < A->ia[i + 1]; ++k)
      if(STRONG(i, k) && agg1[A->ja[k]] >= 0 && fabs(A->a[k]) > best) {
        best = fabs(A->a[k]);
        pick = agg1[A->ja[k]];
      }
    if(pick >= 0) agg[i] = pick;
  }
  /* pass 3: leftovers form aggregates with their free strong neighbours */
  for(int64_t i = 0; i < n; ++i) {
    if(agg[i] >= 0) continue;
    agg[i] = (int32_t)na;
    for(int64_t k = A->ia[i]; k < A->ia[i + 1]; ++k)
      if(STRONG(i, k) && agg[A->ja[k]] < 0) agg[A->ja[k]] = (int32_t)na;
    ++na;
  }
#undef STRONG
  free(agg1);
  free(diag);
  return na;
}

#define MG_MAX_LEVELS 12

struct fo_mg {
  int nl;
  csr_t A[MG_MAX_LEVELS], P[MG_MAX_LEVELS], R[MG_MAX_LEVELS];
  double *dinv[MG_MAX_LEVELS];
  double lmax[MG_MAX_LEVELS];
  double *x[MG_MAX_LEVELS], *b[MG_MAX_LEVELS], *t[MG_MAX_LEVELS];  /* work, 2 components */
  double *cinv;  /* dense inverse of the coarsest operator */
  int64_t nc;
  double diag_sum;
};

fo_mg *fo_mg_create(int64_t n, const int64_t *ia, const int32_t *ja, const double *a, double theta,
                    int64_t coarse_size)
{
  fo_mg *M = calloc(1, sizeof(fo_mg));
  csr_t A = {n, n, malloc(sizeof(int64_t) * (n + 1)), malloc(sizeof(int32_t) * (ia[n] > 0 ? ia[n] : 1)),
             malloc(sizeof(double) * (ia[n] > 0 ? ia[n] : 1))};
  memcpy(A.ia, ia, sizeof(int64_t) * (n + 1));
  memcpy(A.ja, ja, sizeof(int32_t) * ia[n]);
  memcpy(A.a, a, sizeof(double) * ia[n]);
  for(int64_t i = 0; i < n; ++i)
    for(int64_t k = ia[i]; k < ia[i + 1]; ++k)
      if(ja[k] == i) M->diag_sum += a[k];
  for(int lev = 0; lev < MG_MAX_LEVELS; ++lev) {
    M->A[lev] = A;
    M->nl = lev + 1;
    double *dinv = calloc(A.n, sizeof(double));
    for(int64_t i = 0; i < A.n; ++i)
      for(int64_t k = A.ia[i]; k < A.ia[i + 1]; ++k)
        if(A.ja[k] == i) dinv[i] = A.a[k] != 0. ? 1. / A.a[k] : 0.;
    for(int64_t i = 0; i < A.n; ++i)
      if(dinv[i] == 0. || !isfinite(dinv[i])) { free(dinv); fo_mg_destroy(M); return NULL; }
    M->dinv[lev] = dinv;
    M->lmax[lev] = spectral_radius(&A, dinv);
    M->x[lev] = calloc(2 * A.n, sizeof(double));
    M->b[lev] = calloc(2 * A.n, sizeof(double));
    M->t[lev] = calloc(2 * A.n, sizeof(double));
    if(A.n <= coarse_size || lev == MG_MAX_LEVELS - 1) break;
    int32_t *agg = malloc(sizeof(int32_t) * A.n);
    /* the threshold is halved while fewer than half of the rows aggregate */
    double th = theta;
    int64_t na = aggregate(&A, th, agg);
    for(int k = 0; k < 8 && 2 * na > A.n; ++k) {
      th *= 0.5;
      na = aggregate(&A, th, agg);
    }
    if(na >= A.n || na == 0) { free(agg); break; }
    int64_t *size = calloc(na, sizeof(int64_t));
    for(int64_t i = 0; i < A.n; ++i) size[agg[i]]++;
    csr_t T = {A.n, na, malloc(sizeof(int64_t) * (A.n + 1)), malloc(sizeof(int32_t) * A.n),
               malloc(sizeof(double) * A.n)};
    for(int64_t i = 0; i < A.n; ++i) {
      T.ia[i] = i;
      T.ja[i] = agg[i];
      T.a[i] = 1.0 / sqrt((double)size[agg[i]]);
    }
    T.ia[A.n] = A.n;
    free(size);
    free(agg);
    if(A.ia[A.n] > 64 * A.n) {
      /* plain aggregation on levels denser than 64 entries per row: P = T */
      M->P[lev] = T;
      M->R[lev] = transpose(&T);
      csr_t AP0 = spgemm(&A, &T);
      A = spgemm(&M->R[lev], &AP0);
      csr_free(&AP0);
      continue;
    }
    /* P = (I - omega D^-1 A) T */
    const double omega = 4.0 / (3.0 * M->lmax[lev]);
    csr_t AT = spgemm(&A, &T);
    csr_t P = {A.n, na, malloc(sizeof(int64_t) * (A.n + 1)), malloc(sizeof(int32_t) * (AT.ia[A.n] + A.n)),
               malloc(sizeof(double) * (AT.ia[A.n] + A.n))};
    int64_t o = 0;
    P.ia[0] = 0;
    for(int64_t i = 0; i < A.n; ++i) {
      const int32_t tc = T.ja[i];
      const double tv = T.a[i];
      int placed = 0;
      for(int64_t k = AT.ia[i]; k < AT.ia[i + 1]; ++k) {
        const int32_t c = AT.ja[k];
        double v = -omega * dinv[i] * AT.a[k];
        if(!placed && c > tc) { P.ja[o] = tc; P.a[o++] = tv; placed = 1; }
        if(c == tc) { v += tv; placed = 1; }
        P.ja[o] = c;
        P.a[o++] = v;
      }
      if(!placed) { P.ja[o] = tc; P.a[o++] = tv; }
      P.ia[i + 1] = o;
    }
    csr_free(&AT);
    csr_free(&T);
    M->P[lev] = P;
    M->R[lev] = transpose(&P);
    csr_t AP = spgemm(&A, &P);
    A = spgemm(&M->R[lev], &AP);
    csr_free(&AP);
  }
  /* dense inverse of the coarsest operator (Gauss-Jordan, partial pivoting) */
  const csr_t *C = &M->A[M->nl - 1];
  const int64_t nc = C->n;
  double *Mx = calloc(nc * nc, sizeof(double)), *I = calloc(nc * nc, sizeof(double));
  for(int64_t i = 0; i < nc; ++i) {
    for(int64_t k = C->ia[i]; k < C->ia[i + 1]; ++k) Mx[i * nc + C->ja[k]] = C->a[k];
    I[i * nc + i] = 1.;
  }
  for(int64_t c = 0; c < nc; ++c) {
    int64_t piv = c;
    for(int64_t r = c + 1; r < nc; ++r)
      if(fabs(Mx[r * nc + c]) > fabs(Mx[piv * nc + c])) piv = r;
    if(fabs(Mx[piv * nc + c]) < 1e-300) { free(Mx); free(I); fo_mg_destroy(M); return NULL; }
    if(piv != c)
      for(int64_t k = 0; k < nc; ++k) {
        double t = Mx[c * nc + k]; Mx[c * nc + k] = Mx[piv * nc + k]; Mx[piv * nc + k] = t;
        t = I[c * nc + k]; I[c * nc + k] = I[piv * nc + k]; I[piv * nc + k] = t;
      }
    const double inv = 1. / Mx[c * nc + c];
    for(int64_t k = 0; k < nc; ++k) { Mx[c * nc + k] *= inv; I[c * nc + k] *= inv; }
#pragma omp parallel for schedule(static)
    for(int64_t r = 0; r < nc; ++r) {
      if(r == c) continue;
      const double f = Mx[r * nc + c];
      if(f == 0.) continue;
      for(int64_t k = 0; k < nc; ++k) { Mx[r * nc + k] -= f * Mx[c * nc + k]; I[r * nc + k] -= f * I[c * nc + k]; }
    }
  }
  free(Mx);
  M->cinv = I;
  M->nc = nc;
  return M;
}

void fo_mg_destroy(fo_mg *M)
{
  if(!M) return;
  for(int l = 0; l < M->nl; ++l) {
    csr_free(&M->A[l]);
    csr_free(&M->P[l]);
    csr_free(&M->R[l]);
    free(M->dinv[l]); free(M->x[l]); free(M->b[l]); free(M->t[l]);
  }
  free(M->cinv);
  free(M);
}

int fo_mg_levels(const fo_mg *M) { return M->nl; }
double fo_mg_diag_sum(const fo_mg *M) { return M->diag_sum; }

/* One V-cycle on nv (1 or 2) interleaved right-hand sides, b[nv i + c]. */
static void vcycle(fo_mg *M, int l, const double *b, double *x, int nv)
{
  const csr_t *A = &M->A[l];
  const int64_t n = A->n;
  if(l == M->nl - 1) {
    const int64_t nc = M->nc;
#pragma omp parallel for schedule(static)
    for(int64_t i = 0; i < nc; ++i)
      for(int c = 0; c < nv; ++c) {
        double s = 0.;
        for(int64_t k = 0; k < nc; ++k) s += M->cinv[i * nc + k] * b[nv * k + c];
        x[nv * i + c] = s;
      }
    return;
  }
  const double it = 1.0 / (0.7 * M->lmax[l]);
  const double *dinv = M->dinv[l];
  double *res = M->t[l];
  /* pre-smoothing from zero, then the residual b - A x */
#pragma omp parallel for schedule(static)
  for(int64_t i = 0; i < n; ++i)
    for(int c = 0; c < nv; ++c) x[nv * i + c] = it * dinv[i] * b[nv * i + c];
#pragma omp parallel for schedule(static)
  for(int64_t i = 0; i < n; ++i)
    for(int c = 0; c < nv; ++c) {
      double s = b[nv * i + c];
      for(int64_t k = A->ia[i]; k < A->ia[i + 1]; ++k) s -= A->a[k] * x[nv * A->ja[k] + c];
      res[nv * i + c] = s;
    }
  const csr_t *R = &M->R[l], *P = &M->P[l];
  double *bc = M->b[l + 1], *xc = M->x[l + 1];
#pragma omp parallel for schedule(static)
  for(int64_t i = 0; i < R->n; ++i)
    for(int c = 0; c < nv; ++c) {
      double s = 0.;
      for(int64_t k = R->ia[i]; k < R->ia[i + 1]; ++k) s += R->a[k] * res[nv * R->ja[k] + c];
      bc[nv * i + c] = s;
    }
  vcycle(M, l + 1, bc, xc, nv);
  /* y = x + P xc (into res), then x = y + D^-1 (b - A y) / theta */
#pragma omp parallel for schedule(static)
  for(int64_t i = 0; i < n; ++i)
    for(int c = 0; c < nv; ++c) {
      double s = x[nv * i + c];
      for(int64_t k = P->ia[i]; k < P->ia[i + 1]; ++k) s += P->a[k] * xc[nv * P->ja[k] + c];
      res[nv * i + c] = s;
    }
#pragma omp parallel for schedule(static)
  for(int64_t i = 0; i < n; ++i)
    for(int c = 0; c < nv; ++c) {
      double s = b[nv * i + c];
      for(int64_t k = A->ia[i]; k < A->ia[i + 1]; ++k) s -= A->a[k] * res[nv * A->ja[k] + c];
      x[nv * i + c] = res[nv * i + c] + it * dinv[i] * s;
    }
}

void fo_mg_vcycle(fo_mg *M, const double *b, double *x, int nv) { vcycle(M, 0, b, x, nv); }

/* ---------------------------------------------------------------------------
 * Saddle-point (kind 4) and scalar (kind 5) multigrid preconditioners.
 * ------------------------------------------------------------------------- */
struct fo_spmg {
  int kind;
  int64_t n;             /* system rows */
  const int64_t *ia;
  const int32_t *ja;
  const double *A;       /* current values */
  fo_mg *mg;
  int64_t nn;            /* velocity nodes (or unknowns, kind 5) */
  int32_t *dofx, *dofy;  /* node -> row of each component */
  int64_t *diagx;        /* CSR position of the diagonal of the x rows */
  int64_t np;
  int32_t *prows;
  double *pmass, *pscale;
  int64_t *gia;          /* G block per velocity slot 2k+c: CSR positions of pressure columns */
  int64_t *gpos;
  int64_t *dia;          /* D block per pressure row: positions of velocity columns */
  int64_t *dpos;
  int32_t *slot;         /* row -> velocity slot (-1 otherwise) */
  double sigma, divu, s, cMc, cSc;
  double *bxy, *zxy;
};

fo_spmg *fo_spmg_create(int kind, int64_t n, const int64_t *ia, const int32_t *ja, int64_t nn,
                        const int64_t *kia, const int32_t *kja, const double *ka, const int32_t *dofx,
                        const int32_t *dofy, int64_t np, const int32_t *prows, const double *pmass,
                        double sigma, double divu)
{
  fo_spmg *S = calloc(1, sizeof(fo_spmg));
  S->kind = kind;
  S->n = n;
  S->ia = ia;
  S->ja = ja;
  S->nn = nn;
  S->sigma = sigma;
  S->divu = divu;
  S->mg = fo_mg_create(nn, kia, kja, ka, 0.08, 1200);
  if(!S->mg) { free(S); return NULL; }
  S->dofx = malloc(sizeof(int32_t) * nn);
  memcpy(S->dofx, dofx, sizeof(int32_t) * nn);
  if(kind == 4) {
    S->dofy = malloc(sizeof(int32_t) * nn);
    memcpy(S->dofy, dofy, sizeof(int32_t) * nn);
  }
  S->diagx = malloc(sizeof(int64_t) * nn);
  for(int64_t k = 0; k < nn; ++k) {
    S->diagx[k] = -1;
    for(int64_t e = ia[dofx[k]]; e < ia[dofx[k] + 1]; ++e)
      if(ja[e] == dofx[k]) S->diagx[k] = e;
  }
  S->bxy = calloc(2 * nn, sizeof(double));
  S->zxy = calloc(2 * nn, sizeof(double));
  if(kind == 4) {
    S->np = np;
    S->prows = malloc(sizeof(int32_t) * np);
    memcpy(S->prows, prows, sizeof(int32_t) * np);
    S->pmass = malloc(sizeof(double) * np);
    memcpy(S->pmass, pmass, sizeof(double) * np);
    S->pscale = malloc(sizeof(double) * np);
    S->cMc = 0.;
    for(int64_t k = 0; k < np; ++k) S->cMc += pmass[k];
    unsigned char *isp = calloc(n, 1);
    for(int64_t k = 0; k < np; ++k) isp[prows[k]] = 1;
    S->slot = malloc(sizeof(int32_t) * n);
    for(int64_t i = 0; i < n; ++i) S->slot[i] = -1;
    for(int64_t k = 0; k < nn; ++k) { S->slot[dofx[k]] = (int32_t)(2 * k); S->slot[dofy[k]] = (int32_t)(2 * k + 1); }
    S->gia = calloc(2 * nn + 1, sizeof(int64_t));
    for(int64_t q = 0; q < 2 * nn; ++q) {
      const int32_t d = (q & 1) ? dofy[q >> 1] : dofx[q >> 1];
      int64_t c = 0;
      for(int64_t e = ia[d]; e < ia[d + 1]; ++e) c += isp[ja[e]];
      S->gia[q + 1] = S->gia[q] + c;
    }
    S->gpos = malloc(sizeof(int64_t) * (S->gia[2 * nn] + 1));
    for(int64_t q = 0; q < 2 * nn; ++q) {
      const int32_t d = (q & 1) ? dofy[q >> 1] : dofx[q >> 1];
      int64_t o = S->gia[q];
      for(int64_t e = ia[d]; e < ia[d + 1]; ++e)
        if(isp[ja[e]]) S->gpos[o++] = e;
    }
    S->dia = calloc(np + 1, sizeof(int64_t));
    for(int64_t k = 0; k < np; ++k) {
      int64_t c = 0;
      for(int64_t e = ia[prows[k]]; e < ia[prows[k] + 1]; ++e) c += S->slot[ja[e]] >= 0;
      S->dia[k + 1] = S->dia[k] + c;
    }
    S->dpos = malloc(sizeof(int64_t) * (S->dia[np] + 1));
    for(int64_t k = 0; k < np; ++k) {
      int64_t o = S->dia[k];
      for(int64_t e = ia[prows[k]]; e < ia[prows[k] + 1]; ++e)
        if(S->slot[ja[e]] >= 0) S->dpos[o++] = e;
    }
    free(isp);
  }
  return S;
}

int fo_spmg_factor(fo_spmg *S, const double *a)
{
  S->A = a;
  double sum = 0.;
  for(int64_t k = 0; k < S->nn; ++k) {
    if(S->diagx[k] < 0) return -6;
    sum += a[S->diagx[k]];
  }
  if(!isfinite(sum) || sum == 0.) return -6;
  S->s = sum / fo_mg_diag_sum(S->mg);
  if(S->kind != 4) return 0;
  /* the device preconditioner's scaled viscous estimate (factor 6) */
  for(int64_t k = 0; k < S->np; ++k) S->pscale[k] = -6.0 * S->s / (1.5 * S->sigma * S->divu * S->pmass[k]);
  /* c^T S c = -(D^T c) . (s K)^-1 (G c), c = 1 on the pressure unknowns */
  const int64_t nn = S->nn;
  for(int64_t q = 0; q < 2 * nn; ++q) {
    double g = 0.;
    for(int64_t e = S->gia[q]; e < S->gia[q + 1]; ++e) g += a[S->gpos[e]];
    S->bxy[q] = g;
  }
  fo_mg_vcycle(S->mg, S->bxy, S->zxy, 2);
  double sum2 = 0.;
  for(int64_t k = 0; k < S->np; ++k) {
    double t = 0.;
    for(int64_t e = S->dia[k]; e < S->dia[k + 1]; ++e) t += a[S->dpos[e]] * S->zxy[S->slot[S->ja[S->dpos[e]]]];
    sum2 += t;
  }
  S->cSc = -sum2 / S->s;
  if(!isfinite(S->cSc)) S->cSc = 0.;
  return 0;
}

void fo_spmg_apply(fo_spmg *S, const double *r, double *z)
{
  const int64_t nn = S->nn;
  const double inv_s = 1.0 / S->s;
  if(S->kind == 5) {
    for(int64_t k = 0; k < nn; ++k) S->bxy[k] = r[S->dofx[k]];
    fo_mg_vcycle(S->mg, S->bxy, S->zxy, 1);
    for(int64_t k = 0; k < nn; ++k) z[S->dofx[k]] = S->zxy[k] * inv_s;
    return;
  }
  double cr = 0.;
  for(int64_t k = 0; k < S->np; ++k) cr += r[S->prows[k]];
  const double shift = S->cMc > 0 ? cr / S->cMc : 0., lift = S->cSc != 0. ? cr / S->cSc : 0.;
  for(int64_t k = 0; k < S->np; ++k)
    z[S->prows[k]] = S->pscale[k] * (r[S->prows[k]] - shift * S->pmass[k]) + lift;
  const double *a = S->A;
#pragma omp parallel for schedule(static)
  for(int64_t q = 0; q < 2 * nn; ++q) {
    const int32_t d = (q & 1) ? S->dofy[q >> 1] : S->dofx[q >> 1];
    double t = r[d];
    for(int64_t e = S->gia[q]; e < S->gia[q + 1]; ++e) t -= a[S->gpos[e]] * z[S->ja[S->gpos[e]]];
    S->bxy[q] = t;
  }
  fo_mg_vcycle(S->mg, S->bxy, S->zxy, 2);
#pragma omp parallel for schedule(static)
  for(int64_t k = 0; k < nn; ++k) {
    z[S->dofx[k]] = S->zxy[2 * k] * inv_s;
    z[S->dofy[k]] = S->zxy[2 * k + 1] * inv_s;
  }
}

void fo_spmg_destroy(fo_spmg *S)
{
  if(!S) return;
  fo_mg_destroy(S->mg);
  free(S->dofx); free(S->dofy); free(S->diagx); free(S->prows); free(S->pmass); free(S->pscale);
  free(S->gia); free(S->gpos); free(S->dia); free(S->dpos); free(S->slot); free(S->bxy); free(S->zxy);
  free(S);
}
