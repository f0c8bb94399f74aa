// A feNG driver that solves the Kovasznay problem through the reference's own
// API (mesh reader, spaces, numbering, forms, StationaryIntegrator,
// solveNewtonRaphson) with feLinearSystemCUDA as the linear-system backend.
// Built by tests/test_adapter.py against the reference headers and library
// to show the adapter is a drop-in; running it needs a GPU.
#include <cmath>
#include <cstdio>

#include "feAPI.h"
#include "feLinearSystemCUDA.h"

static double g_re = 40.0;
static double lam() { return g_re / 2. - sqrt(g_re * g_re / 4. + 4. * M_PI * M_PI); }
static void uex(const feFunctionArguments &a, const std::vector<double> &, std::vector<double> &r)
{
  const double e = exp(lam() * a.pos[0]);
  r[0] = 1. - e * cos(2. * M_PI * a.pos[1]);
  r[1] = lam() / (2. * M_PI) * e * sin(2. * M_PI * a.pos[1]);
}
static double pex(const feFunctionArguments &a, const std::vector<double> &)
{
  return 0.5 * (1. - exp(2. * lam() * a.pos[0]));
}

int main(int argc, char **argv)
{
  if(argc < 2) return 2;
  setVerbose(1);
  feMesh2DP1 mesh(argv[1]);
  feVectorFunction fu(uex);
  feFunction fp(pex);
  feConstantFunction mu(1.0 / g_re);
  feSpace *u = nullptr, *uB = nullptr, *p = nullptr, *pP = nullptr;
  feCheck(createFiniteElementSpace(u, &mesh, elementType::VECTOR_LAGRANGE, 2, "U", "Domaine", 8, &fu));
  feCheck(createFiniteElementSpace(uB, &mesh, elementType::VECTOR_LAGRANGE, 2, "U", "Bord", 8, &fu));
  feCheck(createFiniteElementSpace(p, &mesh, elementType::LAGRANGE, 1, "P", "Domaine", 8, &fp));
  feCheck(createFiniteElementSpace(pP, &mesh, elementType::LAGRANGE, 1, "P", "PointPression", 8, &fp));
  std::vector<feSpace *> spaces = {u, uB, p, pP}, essential = {uB, pP};
  feMetaNumber numbering(&mesh, spaces, essential);
  feSolution sol(numbering.getNbDOFs(), spaces, essential);
  feBilinearForm *conv = nullptr, *divU = nullptr, *sigma = nullptr;
  feCheck(createBilinearForm(conv, {u}, new feSysElm_VectorConvectiveAcceleration<2>(&scalarConstant::minusOne)));
  feCheck(createBilinearForm(divU, {p, u}, new feSysElm_MixedDivergence<2>(&scalarConstant::one)));
  feCheck(createBilinearForm(sigma, {u, p}, new feSysElm_DivergenceNewtonianStress<2>(&scalarConstant::one, &mu)));
  std::vector<feBilinearForm *> forms = {conv, divU, sigma};
  std::vector<fe_form_desc> desc = {{FE_FORM_VECTOR_CONVECTIVE_ACCELERATION, -1.0, 0., 0, {0, 0, 0, 0}},
                                    {FE_FORM_MIXED_DIVERGENCE, 1.0, 0., 0, {0, 0, 0, 0}},
                                    {FE_FORM_DIV_NEWTONIAN_STRESS, 1.0, 1.0 / g_re, 0, {0, 0, 0, 0}}};
  feLinearSystem *system = new feLinearSystemCUDA(forms, &numbering, &mesh, desc,
                                                  feLinearSystemCUDA::defaultOptions(8));
  std::vector<feNorm *> norms;
  TimeIntegrator *solver = nullptr;
  feNLSolverOptions NL{1e-10, 1e-12, 1e4, 20, 3, 1e-1};
  feCheck(createTimeIntegrator(solver, timeIntegratorScheme::STATIONARY, NL, system, &sol, &mesh, norms,
                               {nullptr, 1, ""}));
  feCheck(solver->makeSteps(1));
  printf("solved: %d unknowns\n", (int)numbering.getNbUnknowns());
  delete solver;
  delete system;
  for(auto *f : forms) delete f;
  for(auto *s : spaces) delete s;
  return 0;
}
