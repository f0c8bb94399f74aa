// Symmetric quadrature rules on the reference triangle (0,0)-(1,0)-(0,1),
// weights summing to the triangle area 1/2.
//
// The rules are the classical fully-symmetric ones (Dunavant, "High degree
// efficient symmetrical Gaussian quadrature rules for the triangle", IJNME
// 21, 1985) that feNG tabulates in getGQTPts (feQuadratureTri.cpp:874-...),
// laid out with the same orbit structure and point order, so element sums
// visit quadrature nodes in the same sequence:
//   centroid;  S21(a): (a,a) (a,1-2a) (1-2a,a);
//   S111(a,b): (a,b) (b,a) (a,c) (c,a) (b,c) (c,b) with c = 1-a-b.
// Instead of transcribing digits, each rule is computed here: its orbit
// parameters start from a few-digit approximation and are refined by
// Gauss-Newton on the moment equations  sum_q w_q r^i s^j = i! j! / (i+j+2)!
// for all i+j <= degree, in long double.  The refined rule is exact to
// rounding, which a unit test checks against the monomial integrals.
#include <algorithm>
#include <cmath>
#include <vector>

#include "fe_common.h"
#include "fe_setup.h"

namespace feng {

namespace {

enum OrbitKind { CENTROID, S21, S111 };
struct Orbit {
  OrbitKind kind;
  int nparam;  // number of point parameters (0, 1, 2); plus one weight
};

void expand(const std::vector<Orbit> &orb, const std::vector<long double> &th,
            std::vector<long double> &r, std::vector<long double> &s, std::vector<long double> &w)
{
  r.clear(); s.clear(); w.clear();
  size_t p = 0;
  for(const Orbit &o : orb) {
    if(o.kind == CENTROID) {
      long double wt = th[p++];
      r.push_back(1.0L / 3); s.push_back(1.0L / 3); w.push_back(wt);
    } else if(o.kind == S21) {
      long double a = th[p++], wt = th[p++], b = 1 - 2 * a;
      long double pr[3] = {a, a, b}, ps[3] = {a, b, a};
      for(int k = 0; k < 3; ++k) { r.push_back(pr[k]); s.push_back(ps[k]); w.push_back(wt); }
    } else {
      long double a = th[p++], b = th[p++], wt = th[p++], c = 1 - a - b;
      long double pr[6] = {a, b, a, c, b, c}, ps[6] = {b, a, c, a, c, b};
      for(int k = 0; k < 6; ++k) { r.push_back(pr[k]); s.push_back(ps[k]); w.push_back(wt); }
    }
  }
}

long double factorial(int n)
{
  long double f = 1;
  for(int i = 2; i <= n; ++i) f *= i;
  return f;
}

void residuals(const std::vector<Orbit> &orb, const std::vector<long double> &th, int deg,
               std::vector<long double> &res)
{
  std::vector<long double> r, s, w;
  expand(orb, th, r, s, w);
  res.clear();
  for(int i = 0; i <= deg; ++i)
    for(int j = 0; i + j <= deg; ++j) {
      long double sum = 0;
      for(size_t q = 0; q < w.size(); ++q) {
        long double t = w[q];
        for(int k = 0; k < i; ++k) t *= r[q];
        for(int k = 0; k < j; ++k) t *= s[q];
        sum += t;
      }
      res.push_back(sum - factorial(i) * factorial(j) / factorial(i + j + 2));
    }
}

bool refine(const std::vector<Orbit> &orb, std::vector<long double> &th, int deg)
{
  const size_t n = th.size();
  std::vector<long double> r0, r1, r2;
  for(int it = 0; it < 60; ++it) {
    residuals(orb, th, deg, r0);
    const size_t m = r0.size();
    long double nrm = 0;
    for(auto v : r0) nrm = fmaxl(nrm, fabsl(v));
    if(nrm < 1e-19L) return true;
    // Central-difference Jacobian (long double): only the fixed point must be
    // exact, the Jacobian merely steers the iteration.
    std::vector<long double> J(m * n);
    for(size_t k = 0; k < n; ++k) {
      long double h = 1e-9L, keep = th[k];
      th[k] = keep + h; residuals(orb, th, deg, r1);
      th[k] = keep - h; residuals(orb, th, deg, r2);
      th[k] = keep;
      for(size_t i = 0; i < m; ++i) J[i * n + k] = (r1[i] - r2[i]) / (2 * h);
    }
    // Normal equations (J^T J) d = -J^T r, Gaussian elimination with pivoting.
    std::vector<long double> A(n * (n + 1), 0);
    for(size_t a = 0; a < n; ++a) {
      for(size_t b = 0; b < n; ++b) {
        long double t = 0;
        for(size_t i = 0; i < m; ++i) t += J[i * n + a] * J[i * n + b];
        A[a * (n + 1) + b] = t;
      }
      long double t = 0;
      for(size_t i = 0; i < m; ++i) t += J[i * n + a] * r0[i];
      A[a * (n + 1) + n] = -t;
    }
    for(size_t c = 0; c < n; ++c) {
      size_t piv = c;
      for(size_t i = c + 1; i < n; ++i)
        if(fabsl(A[i * (n + 1) + c]) > fabsl(A[piv * (n + 1) + c])) piv = i;
      if(fabsl(A[piv * (n + 1) + c]) < 1e-300L) return false;
      if(piv != c)
        for(size_t k = 0; k <= n; ++k) std::swap(A[c * (n + 1) + k], A[piv * (n + 1) + k]);
      for(size_t i = 0; i < n; ++i) {
        if(i == c) continue;
        long double f = A[i * (n + 1) + c] / A[c * (n + 1) + c];
        for(size_t k = c; k <= n; ++k) A[i * (n + 1) + k] -= f * A[c * (n + 1) + k];
      }
    }
    for(size_t k = 0; k < n; ++k) th[k] += A[k * (n + 1) + n] / A[k * (n + 1) + k];
  }
  residuals(orb, th, deg, r0);
  long double nrm = 0;
  for(auto v : r0) nrm = fmaxl(nrm, fabsl(v));
  return nrm < 1e-17L;
}

}  // namespace

int triangle_rule(int degree, QuadRule &q)
{
  std::vector<Orbit> orb;
  std::vector<long double> th;
  int exactDeg = degree;
  switch(degree) {
    case 1:
      // Centroid rule, exact.
      q.r = {1.0 / 3}; q.s = {1.0 / 3}; q.w = {0.5}; q.degree = 1;
      return FE_OK;
    case 2:
      orb = {{S21, 1}};
      th = {1.0L / 6, 1.0L / 6};
      break;
    case 4:
      orb = {{S21, 1}, {S21, 1}};
      th = {0.0916L, 0.0550L, 0.4459L, 0.1117L};
      break;
    case 5:
      orb = {{CENTROID, 0}, {S21, 1}, {S21, 1}};
      th = {0.1125L, 0.1013L, 0.0630L, 0.4701L, 0.0662L};
      break;
    case 8:
      orb = {{CENTROID, 0}, {S21, 1}, {S21, 1}, {S21, 1}, {S111, 2}};
      th = {0.07216L, 0.17057L, 0.05161L, 0.05055L, 0.01623L, 0.45929L, 0.04755L,
            0.008395L, 0.26311L, 0.013615L};
      break;
    default:
      set_error("triangle quadrature of degree %d is not available (use 1, 2, 4, 5 or 8)", degree);
      return FE_INVALID_ARG;
  }
  if(!refine(orb, th, exactDeg)) {
    set_error("quadrature refinement for degree %d did not converge", degree);
    return FE_ERROR;
  }
  std::vector<long double> r, s, w;
  expand(orb, th, r, s, w);
  q.degree = degree;
  q.r.assign(r.begin(), r.end());
  q.s.assign(s.begin(), s.end());
  q.w.assign(w.begin(), w.end());
  return FE_OK;
}

}  // namespace feng

// ---- tetrahedra ----------------------------------------------------------
//
// Fully symmetric rules in barycentric orbits (l0, l1, l2, l3), with
// (r, s, t) = (l1, l2, l3):
//   C4:        (1/4, 1/4, 1/4, 1/4)
//   S31(a):    three coordinates a, one 1 - 3a          (4 points)
//   S22(a):    two coordinates a, two 1/2 - a           (6 points)
//   S211(a,b): two a, one b, one 1 - 2a - b             (12 points)
// Each rule uses the orbit structure of the reference's rule of the same
// degree; its parameters start from a few-digit approximation and are
// refined by Gauss-Newton on the moment equations
//   sum_q w_q r^i s^j t^k = i! j! k! / (i+j+k+3)!,  i+j+k <= degree,
// in long double.  Points are listed in a fixed order within each orbit
// (the position of the odd coordinate, or of the pairs, in increasing
// order).  The reference tabulates its rules with 13 decimals, so its
// values agree with these to about 1e-13.

namespace feng {

namespace {

enum TetOrbitKind { C4, S31, S22, S211 };

void expand_tet(const std::vector<TetOrbitKind> &orb, const std::vector<long double> &th,
                std::vector<long double> *l, std::vector<long double> &w)
{
  for(int k = 0; k < 4; ++k) l[k].clear();
  w.clear();
  size_t p = 0;
  auto push = [&](long double a0, long double a1, long double a2, long double a3, long double wt) {
    l[0].push_back(a0); l[1].push_back(a1); l[2].push_back(a2); l[3].push_back(a3); w.push_back(wt);
  };
  for(TetOrbitKind o : orb) {
    if(o == C4) {
      push(0.25L, 0.25L, 0.25L, 0.25L, th[p++]);
    } else if(o == S31) {
      const long double a = th[p++], wt = th[p++], b = 1 - 3 * a;
      for(int odd = 0; odd < 4; ++odd) {
        long double v[4] = {a, a, a, a};
        v[odd] = b;
        push(v[0], v[1], v[2], v[3], wt);
      }
    } else if(o == S22) {
      const long double a = th[p++], wt = th[p++], b = 0.5L - a;
      for(int i = 0; i < 4; ++i)
        for(int j = i + 1; j < 4; ++j) {
          long double v[4] = {b, b, b, b};
          v[i] = v[j] = a;
          push(v[0], v[1], v[2], v[3], wt);
        }
    } else {
      const long double a = th[p++], b = th[p++], wt = th[p++], c = 1 - 2 * a - b;
      for(int i = 0; i < 4; ++i)
        for(int j = i + 1; j < 4; ++j) {
          int rest[2], n = 0;
          for(int k = 0; k < 4; ++k)
            if(k != i && k != j) rest[n++] = k;
          for(int s = 0; s < 2; ++s) {
            long double v[4];
            v[i] = v[j] = a;
            v[rest[s]] = b;
            v[rest[1 - s]] = c;
            push(v[0], v[1], v[2], v[3], wt);
          }
        }
    }
  }
}

void tet_residuals(const std::vector<TetOrbitKind> &orb, const std::vector<long double> &th, int deg,
                   std::vector<long double> &res)
{
  std::vector<long double> l[4], w;
  expand_tet(orb, th, l, w);
  res.clear();
  for(int i = 0; i <= deg; ++i)
    for(int j = 0; i + j <= deg; ++j)
      for(int k = 0; i + j + k <= deg; ++k) {
        long double sum = 0;
        for(size_t q = 0; q < w.size(); ++q) {
          long double v = w[q];
          for(int e = 0; e < i; ++e) v *= l[1][q];
          for(int e = 0; e < j; ++e) v *= l[2][q];
          for(int e = 0; e < k; ++e) v *= l[3][q];
          sum += v;
        }
        res.push_back(sum - factorial(i) * factorial(j) * factorial(k) / factorial(i + j + k + 3));
      }
}

// Gauss-Newton on the moment equations (normal equations, central-difference
// Jacobian), as refine() for triangles, over the parameters not listed in
// `fixed` (indices into th held at their given values).
bool refine_tet(const std::vector<TetOrbitKind> &orb, std::vector<long double> &th, int deg,
                const std::vector<size_t> &fixed = {})
{
  std::vector<size_t> freeIdx;
  for(size_t k = 0; k < th.size(); ++k)
    if(std::find(fixed.begin(), fixed.end(), k) == fixed.end()) freeIdx.push_back(k);
  const size_t n = freeIdx.size();
  std::vector<long double> r0, r1, r2;
  for(int it = 0; it < 80; ++it) {
    tet_residuals(orb, th, deg, r0);
    const size_t m = r0.size();
    long double nrm = 0;
    for(auto v : r0) nrm = fmaxl(nrm, fabsl(v));
    if(nrm < 1e-19L) return true;
    std::vector<long double> J(m * n);
    for(size_t k = 0; k < n; ++k) {
      const size_t p = freeIdx[k];
      const long double h = 1e-9L, keep = th[p];
      th[p] = keep + h; tet_residuals(orb, th, deg, r1);
      th[p] = keep - h; tet_residuals(orb, th, deg, r2);
      th[p] = keep;
      for(size_t i = 0; i < m; ++i) J[i * n + k] = (r1[i] - r2[i]) / (2 * h);
    }
    std::vector<long double> A(n * (n + 1), 0);
    for(size_t a = 0; a < n; ++a) {
      for(size_t b = 0; b < n; ++b) {
        long double t = 0;
        for(size_t i = 0; i < m; ++i) t += J[i * n + a] * J[i * n + b];
        A[a * (n + 1) + b] = t;
      }
      long double t = 0;
      for(size_t i = 0; i < m; ++i) t += J[i * n + a] * r0[i];
      A[a * (n + 1) + n] = -t;
    }
    for(size_t c = 0; c < n; ++c) {
      size_t piv = c;
      for(size_t i = c + 1; i < n; ++i)
        if(fabsl(A[i * (n + 1) + c]) > fabsl(A[piv * (n + 1) + c])) piv = i;
      if(fabsl(A[piv * (n + 1) + c]) < 1e-300L) return false;
      if(piv != c)
        for(size_t k = 0; k <= n; ++k) std::swap(A[c * (n + 1) + k], A[piv * (n + 1) + k]);
      for(size_t i = 0; i < n; ++i) {
        if(i == c) continue;
        const long double f = A[i * (n + 1) + c] / A[c * (n + 1) + c];
        for(size_t k = c; k <= n; ++k) A[i * (n + 1) + k] -= f * A[c * (n + 1) + k];
      }
    }
    for(size_t k = 0; k < n; ++k) th[freeIdx[k]] += A[k * (n + 1) + n] / A[k * (n + 1) + k];
  }
  tet_residuals(orb, th, deg, r0);
  long double nrm = 0;
  for(auto v : r0) nrm = fmaxl(nrm, fabsl(v));
  return nrm < 1e-17L;
}

}  // namespace

int tet_rule(int degree, QuadRule &q)
{
  std::vector<TetOrbitKind> orb;
  std::vector<long double> th;  // per orbit: point parameters, then the weight
  std::vector<size_t> fixed;    // parameters at exact positions, not refined
  switch(degree) {
    case 1: orb = {C4}; th = {1.0L / 6}; break;
    case 2: orb = {S31}; th = {0.1382L, 0.04167L}; break;
    case 3: orb = {C4, S31}; th = {-0.1333L, 0.1667L, 0.075L}; break;
    case 4: orb = {C4, S31, S22}; th = {-0.01316L, 0.07143L, 0.007622L, 0.3994L, 0.02489L}; break;
    case 5: orb = {S31, S31, S22}; th = {0.09274L, 0.01225L, 0.3109L, 0.01878L, 0.4545L, 0.007091L}; break;
    case 6:
      orb = {S31, S31, S31, S211};
      th = {0.2146L, 0.006654L, 0.04067L, 0.00168L, 0.3223L, 0.009226L, 0.06366L, 0.2697L, 0.008036L};
      break;
    case 7:
      orb = {S22, C4, S31, S31, S31, S211};
      th = {0.0L, 0.00097L, 0.01826L, 0.07821L, 0.0106L, 0.1218L, -0.06252L, 0.3325L, 0.00489L, 0.1L, 0.2L,
            0.02756L};
      // Degree 7 has a family of solutions with this structure; the
      // reference's member keeps the S22 orbit at (1/2, 1/2, 0, 0) and the
      // S211 orbit at (1/10, 1/10, 1/5, 3/5).
      fixed = {0, 9, 10};
      break;
    case 8:
      orb = {C4, S31, S31, S31, S22, S211, S211};
      th = {-0.0205L, 0.2068L, 0.01425L, 0.0821L, 0.001967L, 0.005782L, 0.00017L, 0.05053L, 0.00458L,
            0.2291L, 0.03564L, 0.005704L, 0.03661L, 0.1905L, 0.002141L};
      break;
    default:
      set_error("tetrahedral quadrature of degree %d is not available (1 to 8)", degree);
      return FE_INVALID_ARG;
  }
  if(!refine_tet(orb, th, degree, fixed)) {
    set_error("tetrahedral quadrature refinement for degree %d did not converge", degree);
    return FE_ERROR;
  }
  std::vector<long double> l[4], w;
  expand_tet(orb, th, l, w);
  q = QuadRule();
  q.degree = degree;
  q.r.assign(l[1].begin(), l[1].end());
  q.s.assign(l[2].begin(), l[2].end());
  q.t.assign(l[3].begin(), l[3].end());
  q.w.assign(w.begin(), w.end());
  return FE_OK;
}

}  // namespace feng
