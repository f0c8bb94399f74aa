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
