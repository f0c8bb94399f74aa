// Host set-up of the smoothed-aggregation hierarchy (see fe_amg.h).
#include <algorithm>
#include <cmath>
#include <numeric>

#include "fe_amg.h"
#include "fe_common.h"

namespace feng {

namespace {

// C = A * B (Gustavson's row-by-row product with a dense marker), rows in
// parallel: a symbolic pass for the row sizes, then the numeric pass; each
// row is formed exactly as a serial product would form it.
HostCSR spgemm(const HostCSR &A, const HostCSR &B)
{
  HostCSR C;
  C.n = A.n;
  C.m = B.m;
  C.ia.assign(A.n + 1, 0);
  parallel_for(A.n, [&](int64_t r0, int64_t r1) {
    std::vector<int64_t> marker(B.m, -1);
    for(int64_t i = r0; i < r1; ++i) {
      int64_t c = 0;
      for(int64_t k = A.ia[i]; k < A.ia[i + 1]; ++k) {
        const int32_t j = A.ja[k];
        for(int64_t l = B.ia[j]; l < B.ia[j + 1]; ++l)
          if(marker[B.ja[l]] != i) {
            marker[B.ja[l]] = i;
            ++c;
          }
      }
      C.ia[i + 1] = c;
    }
  }, 1024);
  for(int64_t i = 0; i < A.n; ++i) C.ia[i + 1] += C.ia[i];
  C.ja.resize(C.ia[A.n]);
  C.a.resize(C.ia[A.n]);
  parallel_for(A.n, [&](int64_t r0, int64_t r1) {
    std::vector<int64_t> marker(B.m, -1);
    std::vector<double> acc(B.m, 0.);
    std::vector<int32_t> cols;
    for(int64_t i = r0; i < r1; ++i) {
      cols.clear();
      for(int64_t k = A.ia[i]; k < A.ia[i + 1]; ++k) {
        const int32_t j = A.ja[k];
        const double av = A.a[k];
        for(int64_t l = B.ia[j]; l < B.ia[j + 1]; ++l) {
          const int32_t c = B.ja[l];
          if(marker[c] != i) {
            marker[c] = i;
            acc[c] = 0.;
            cols.push_back(c);
          }
          acc[c] += av * B.a[l];
        }
      }
      std::sort(cols.begin(), cols.end());
      int64_t o = C.ia[i];
      for(int32_t c : cols) {
        C.ja[o] = c;
        C.a[o++] = acc[c];
      }
    }
  }, 1024);
  return C;
}

HostCSR transpose(const HostCSR &A)
{
  HostCSR T;
  T.n = A.m;
  T.m = A.n;
  T.ia.assign(A.m + 1, 0);
  for(int32_t j : A.ja) T.ia[j + 1]++;
  for(int64_t i = 0; i < A.m; ++i) T.ia[i + 1] += T.ia[i];
  T.ja.resize(A.nnz());
  T.a.resize(A.nnz());
  std::vector<int64_t> fill(T.ia.begin(), T.ia.end() - 1);
  for(int64_t i = 0; i < A.n; ++i)
    for(int64_t k = A.ia[i]; k < A.ia[i + 1]; ++k) {
      const int64_t p = fill[A.ja[k]]++;
      T.ja[p] = (int32_t)i;
      T.a[p] = A.a[k];
    }
  return T;
}

std::vector<double> inv_diag(const HostCSR &A)
{
  std::vector<double> d(A.n, 0.);
  for(int64_t i = 0; i < A.n; ++i)
    for(int64_t k = A.ia[i]; k < A.ia[i + 1]; ++k)
      if(A.ja[k] == i) d[i] = A.a[k] != 0 ? 1. / A.a[k] : 0.;
  return d;
}

// Spectral radius of D^-1 A by power iteration (deterministic start).
double spectral_radius(const HostCSR &A, const std::vector<double> &dinv, int iters = 20)
{
  std::vector<double> x(A.n), y(A.n);
  for(int64_t i = 0; i < A.n; ++i) x[i] = 1.0 + 0.1 * std::sin(0.37 * (double)i);
  double lam = 1.;
  for(int it = 0; it < iters; ++it) {
    double nrm = 0.;
    for(int64_t i = 0; i < A.n; ++i) {
      double s = 0.;
      for(int64_t k = A.ia[i]; k < A.ia[i + 1]; ++k) s += A.a[k] * x[A.ja[k]];
      y[i] = dinv[i] * s;
      nrm += y[i] * y[i];
    }
    nrm = std::sqrt(nrm);
    double xn = 0.;
    for(double v : x) xn += v * v;
    lam = nrm / std::sqrt(std::max(xn, 1e-300));
    if(nrm == 0) break;
    for(int64_t i = 0; i < A.n; ++i) x[i] = y[i] / nrm;
  }
  return lam;
}

// Greedy aggregation over the strong-connection graph (three passes).
int64_t aggregate(const HostCSR &A, double theta, std::vector<int32_t> &agg)
{
  const int64_t n = A.n;
  std::vector<double> diag(n, 0.);
  for(int64_t i = 0; i < n; ++i)
    for(int64_t k = A.ia[i]; k < A.ia[i + 1]; ++k)
      if(A.ja[k] == i) diag[i] = std::fabs(A.a[k]);
  auto strong = [&](int64_t i, int64_t k) {
    const int32_t j = A.ja[k];
    return j != i && std::fabs(A.a[k]) >= theta * std::sqrt(diag[i] * diag[j]);
  };
  agg.assign(n, -1);
  int64_t na = 0;
  // pass 1: roots whose strong neighbourhood is still free
  for(int64_t i = 0; i < n; ++i) {
    if(agg[i] >= 0) continue;
    bool free = true, any = false;
    for(int64_t k = A.ia[i]; k < A.ia[i + 1]; ++k)
      if(strong(i, k)) {
        any = true;
        if(agg[A.ja[k]] >= 0) { free = false; break; }
      }
    if(!free) continue;
    agg[i] = (int32_t)na;
    if(any)
      for(int64_t k = A.ia[i]; k < A.ia[i + 1]; ++k)
        if(strong(i, k)) agg[A.ja[k]] = (int32_t)na;
    ++na;
  }
  // pass 2: join a neighbouring aggregate (strongest connection)
  std::vector<int32_t> agg1 = agg;
  for(int64_t i = 0; i < n; ++i) {
    if(agg1[i] >= 0) continue;
    double best = -1.;
    int32_t pick = -1;
    for(int64_t k = A.ia[i]; k < A.ia[i + 1]; ++k)
      if(strong(i, k) && agg1[A.ja[k]] >= 0 && std::fabs(A.a[k]) > best) {
        best = std::fabs(A.a[k]);
        pick = agg1[A.ja[k]];
      }
    if(pick >= 0) agg[i] = pick;
  }
  // pass 3: leftovers form their own aggregates
  for(int64_t i = 0; i < n; ++i) {
    if(agg[i] >= 0) continue;
    agg[i] = (int32_t)na;
    for(int64_t k = A.ia[i]; k < A.ia[i + 1]; ++k)
      if(strong(i, k) && agg[A.ja[k]] < 0) agg[A.ja[k]] = (int32_t)na;
    ++na;
  }
  return na;
}

}  // namespace

int amg_build(const HostCSR &A0, const AMGParams &p, AMGHierarchy &H)
{
  H = AMGHierarchy();
  HostCSR A = A0;
  for(int lev = 0; lev < p.maxLevels; ++lev) {
    AMGLevel L;
    L.A = A;
    L.dinv = inv_diag(A);
    for(double d : L.dinv)
      if(!(std::isfinite(d)) || d == 0.) {
        set_error("multigrid operator has a zero diagonal on level %d", lev);
        return FE_PC_FAILED;
      }
    L.lmax = spectral_radius(A, L.dinv);
    if(A.n <= p.coarseSize || lev == p.maxLevels - 1) {
      H.levels.push_back(std::move(L));
      break;
    }
    // Halve the strength threshold while fewer than half of the rows join a
    // neighbour's aggregate: on the Galerkin operators of three-dimensional
    // P2 systems (dense stencils of small entries) the first threshold keeps
    // nearly every row a singleton, the level barely shrinks and its
    // Galerkin product fills in (41 k -> 40 k rows, 189 -> 4,547 entries per
    // row for the 32^3 cube's shifted velocity operator).
    std::vector<int32_t> agg;
    double theta = p.theta;
    int64_t na = aggregate(A, theta, agg);
    for(int k = 0; k < 8 && 2 * na > A.n; ++k) {
      theta *= 0.5;
      na = aggregate(A, theta, agg);
    }
    if(na >= A.n || na == 0) {  // no coarsening possible
      H.levels.push_back(std::move(L));
      break;
    }
    // Tentative prolongator: constant per aggregate, unit-norm columns.
    std::vector<int64_t> size(na, 0);
    for(int32_t g : agg) size[g]++;
    HostCSR T;
    T.n = A.n;
    T.m = na;
    T.ia.resize(A.n + 1);
    T.ja.resize(A.n);
    T.a.resize(A.n);
    for(int64_t i = 0; i < A.n; ++i) {
      T.ia[i] = i;
      T.ja[i] = agg[i];
      T.a[i] = 1.0 / std::sqrt((double)size[agg[i]]);
    }
    T.ia[A.n] = A.n;
    if((double)A.nnz() > p.smoothMaxRow * (double)A.n) {
      // plain aggregation: P = T
      L.P = T;
      L.R = transpose(T);
      HostCSR AT = spgemm(A, T);
      A = spgemm(L.R, AT);
      H.levels.push_back(std::move(L));
      continue;
    }
    // Smoothed prolongator P = (I - omega D^-1 A) T, omega = 4 / (3 rho).
    const double omega = 4.0 / (3.0 * L.lmax);
    // filterSmoothing: the prolongator is smoothed with the filtered operator
    // (strong couplings kept, the weak ones lumped onto the diagonal), whose
    // sparser stencil keeps the next level sparse
    HostCSR AF;
    if(p.filterSmoothing) {
      std::vector<double> dg(A.n, 0.);
      for(int64_t i = 0; i < A.n; ++i)
        for(int64_t k = A.ia[i]; k < A.ia[i + 1]; ++k)
          if(A.ja[k] == i) dg[i] = std::fabs(A.a[k]);
      AF.n = A.n;
      AF.m = A.m;
      AF.ia.assign(A.n + 1, 0);
      for(int64_t i = 0; i < A.n; ++i) {
        double lump = 0.;
        int64_t dpos = -1;
        for(int64_t k = A.ia[i]; k < A.ia[i + 1]; ++k) {
          const int32_t j = A.ja[k];
          if(j == i) {
            dpos = (int64_t)AF.ja.size();
            AF.ja.push_back(j);
            AF.a.push_back(A.a[k]);
          } else if(std::fabs(A.a[k]) >= theta * std::sqrt(dg[i] * dg[j])) {
            AF.ja.push_back(j);
            AF.a.push_back(A.a[k]);
          } else {
            lump += A.a[k];
          }
        }
        if(dpos >= 0) AF.a[dpos] += lump;
        AF.ia[i + 1] = (int64_t)AF.ja.size();
      }
    }
    const HostCSR &AS = p.filterSmoothing ? AF : A;
    const std::vector<double> dinvS = p.filterSmoothing ? inv_diag(AF) : L.dinv;
    const double omegaS = p.filterSmoothing ? 4.0 / (3.0 * spectral_radius(AF, dinvS)) : omega;
    HostCSR AT = spgemm(AS, T);
    HostCSR P;
    P.n = A.n;
    P.m = na;
    P.ia.assign(A.n + 1, 0);
    for(int64_t i = 0; i < A.n; ++i) {
      // merge row i of T (single entry) with -omega dinv_i * row i of AT
      const int32_t tc = T.ja[i];
      const double tv = T.a[i];
      bool placed = false;
      for(int64_t k = AT.ia[i]; k < AT.ia[i + 1]; ++k) {
        const int32_t c = AT.ja[k];
        double v = -omegaS * dinvS[i] * AT.a[k];
        if(!placed && c > tc) {
          P.ja.push_back(tc);
          P.a.push_back(tv);
          placed = true;
        }
        if(c == tc) {
          v += tv;
          placed = true;
        }
        P.ja.push_back(c);
        P.a.push_back(v);
      }
      if(!placed) {
        P.ja.push_back(tc);
        P.a.push_back(tv);
      }
      P.ia[i + 1] = (int64_t)P.ja.size();
    }
    L.P = P;
    L.R = transpose(P);
    HostCSR AP = spgemm(A, P);
    A = spgemm(L.R, AP);
    H.levels.push_back(std::move(L));
  }
  // Dense inverse of the coarsest operator (Gauss-Jordan, partial pivoting).
  const HostCSR &Ac = H.levels.back().A;
  const int64_t nc = Ac.n;
  std::vector<double> M(nc * nc, 0.), I(nc * nc, 0.);
  for(int64_t i = 0; i < nc; ++i) {
    for(int64_t k = Ac.ia[i]; k < Ac.ia[i + 1]; ++k) M[i * nc + Ac.ja[k]] = Ac.a[k];
    I[i * nc + i] = 1.;
  }
  for(int64_t c = 0; c < nc; ++c) {
    int64_t piv = c;
    for(int64_t r = c + 1; r < nc; ++r)
      if(std::fabs(M[r * nc + c]) > std::fabs(M[piv * nc + c])) piv = r;
    if(std::fabs(M[piv * nc + c]) < 1e-300) {
      set_error("coarsest multigrid operator is singular");
      return FE_PC_FAILED;
    }
    if(piv != c)
      for(int64_t k = 0; k < nc; ++k) {
        std::swap(M[c * nc + k], M[piv * nc + k]);
        std::swap(I[c * nc + k], I[piv * nc + k]);
      }
    const double inv = 1. / M[c * nc + c];
    for(int64_t k = 0; k < nc; ++k) { M[c * nc + k] *= inv; I[c * nc + k] *= inv; }
    for(int64_t r = 0; r < nc; ++r) {
      if(r == c) continue;
      const double f = M[r * nc + c];
      if(f == 0.) continue;
      for(int64_t k = 0; k < nc; ++k) { M[r * nc + k] -= f * M[c * nc + k]; I[r * nc + k] -= f * I[c * nc + k]; }
    }
  }
  H.coarseInv = std::move(I);
  return FE_OK;
}

}  // namespace feng
