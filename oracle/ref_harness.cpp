// Test infrastructure only: a driver linked against the reference feNG core
// library (built from its own sources into oracle/_ref/ by oracle/Makefile).
// It produces golden fixtures for the parity tests and validates the CPU
// restatement in oracle/fe_oracle.c.  Nothing in the product links it.
//
// It runs the reference's own mesh reader, FE spaces, DOF numbering,
// coloring, CSR pattern builder (feEZCompressedRowStorage) and element
// kernels (feBilinearForm::computeMatrix/computeResidual).  The backend
// scatter and solve live in the MKL/PETSc classes that cannot be built here
// (no MKL, PETSc, MPI), so feLinearSystemRef below restates the MKL scatter
// (feLinearSystemMklPardiso.cpp:501-749, sorted local indices + linear scan of
// the CSR row) and solves with the vendored Eigen SparseLU.
//
// usage: ref_harness <mesh.msh> <problem> <outdir> [Re] [seed]
//   problem: diffusion | diffusion3d | ns_kovasznay | ns_mms | ns_cavity_bdf2 (then [dt] [steps])
// writes raw little-endian arrays (see write_* calls) and meta.txt.
#include <Eigen/Sparse>
#include <Eigen/SparseLU>
#include <cstdio>
#include <fstream>
#include <random>
#include <string>

#include "feAPI.h"

extern std::vector<double> solAtTimeN;

namespace {

struct CSR : public feEZCompressedRowStorage {
  using feEZCompressedRowStorage::feEZCompressedRowStorage;
  const std::vector<feInt> &ia() const { return ia_Pardiso; }
  const std::vector<feInt> &ja() const { return ja_Pardiso; }
};

class feLinearSystemRef : public feLinearSystem {
 public:
  feInt nInc;
  CSR *crs;
  std::vector<double> values, rhs, du;
  double lastAxb = 0;
  Eigen::SparseMatrix<double> A;
  // Fill-reducing ordering of the direct solve: COLAMD (Eigen's default) or,
  // with FE_HARNESS_ORDERING=amd, minimum degree on A + A^T (much less fill
  // on large 2D meshes).  Both give the solution to rounding.
  Eigen::SparseLU<Eigen::SparseMatrix<double>> lu;
  Eigen::SparseLU<Eigen::SparseMatrix<double>, Eigen::AMDOrdering<int>> luAmd;
  bool useAmd = getenv("FE_HARNESS_ORDERING") && std::string(getenv("FE_HARNESS_ORDERING")) == "amd";
  bool factored = false;

  feLinearSystemRef(std::vector<feBilinearForm *> forms, const feMetaNumber *numbering)
    : feLinearSystem(forms, numbering)
  {
    nInc = numbering->getNbUnknowns();
    crs = new CSR(nInc, _formMatrices, _numMatrixForms, numbering);
    values.assign(crs->ja().size(), 0.);
    rhs.assign(nInc, 0.);
    du.assign(nInc, 0.);
  }
  ~feLinearSystemRef() { delete crs; }
  feInt getSystemSize() const override { return nInc; }
  void getRHSMaxNorm(double *norm) const override
  {
    double m = 0;
    for(double v : rhs) m = std::max(m, std::fabs(v));
    *norm = m;
  }
  void getResidualMaxNorm(double *norm) const override
  {
    double m = 0;
    for(double v : du) m = std::max(m, std::fabs(v));
    *norm = m;
  }
  // As feLinearSystemMklPardiso::setToZero (:967-971): the matrix is kept
  // when the Newton driver reuses the Jacobian.
  void setToZero() override
  {
    if(_recomputeMatrix) setMatrixToZero();
    setResidualToZero();
  }
  void setMatrixToZero() override { std::fill(values.begin(), values.end(), 0.); }
  void setResidualToZero() override { std::fill(rhs.begin(), rhs.end(), 0.); }
  void assemble(const feSolution *sol, const bool onlyTransient) override
  {
    assembleMatrices(sol, onlyTransient);
    assembleResiduals(sol);
  }
  // Scatter restated from feLinearSystemMklPardiso::assembleMatrices.
  void assembleMatrices(const feSolution *sol, const bool onlyTransient) override
  {
    const auto &ia = crs->ia();
    const auto &ja = crs->ja();
    for(int eq = 0; eq < _numMatrixForms; ++eq) {
      feBilinearForm *f = _formMatrices[eq];
      if(onlyTransient && !f->isTransientMatrix()) continue;
      const feCncGeo *cnc = f->getCncGeo();
      for(int c = 0; c < cnc->getNbColor(); ++c) {
        for(int elm : cnc->getListElmPerColor()[c]) {
          f->computeMatrix(sol, elm);
          const double *const *Ae = f->getAe();
          std::vector<feInt> adrI = f->getAdrI(), adrJ = f->getAdrJ(), ni, nj;
          for(size_t i = 0; i < adrI.size(); ++i)
            if(adrI[i] < nInc) ni.push_back(i);
          for(size_t j = 0; j < adrJ.size(); ++j)
            if(adrJ[j] < nInc) nj.push_back(j);
          adrI.erase(std::remove_if(adrI.begin(), adrI.end(), [this](feInt x) { return x >= nInc; }), adrI.end());
          adrJ.erase(std::remove_if(adrJ.begin(), adrJ.end(), [this](feInt x) { return x >= nInc; }), adrJ.end());
          std::vector<feInt> si(adrI.size()), sj(adrJ.size());
          for(size_t i = 0; i < si.size(); ++i) si[i] = i;
          for(size_t j = 0; j < sj.size(); ++j) sj[j] = j;
          std::sort(si.begin(), si.end(), [&](feInt a, feInt b) { return adrI[a] < adrI[b]; });
          std::sort(sj.begin(), sj.end(), [&](feInt a, feInt b) { return adrJ[a] < adrJ[b]; });
          for(size_t i = 0; i < adrI.size(); ++i) {
            const feInt I = adrI[si[i]];
            const feInt beg = ia[I], num = ia[I + 1] - ia[I];
            feInt start = 0;
            for(size_t j = 0; j < adrJ.size(); ++j) {
              for(feInt J = start; J < num; ++J) {
                if(ja[beg + J] == adrJ[sj[j]]) {
                  values[beg + J] += Ae[ni[si[i]]][nj[sj[j]]];
                  start = J;
                  break;
                }
              }
            }
          }
        }
      }
    }
  }
  // Restated from feLinearSystemMklPardiso::assembleResiduals.
  void assembleResiduals(const feSolution *sol) override
  {
    for(int eq = 0; eq < _numResidualForms; ++eq) {
      feBilinearForm *f = _formResiduals[eq];
      const feCncGeo *cnc = f->getCncGeo();
      for(int c = 0; c < cnc->getNbColor(); ++c) {
        for(int elm : cnc->getListElmPerColor()[c]) {
          f->computeResidual(sol, elm);
          const double *Be = f->getBe();
          const std::vector<feInt> &adrI = f->getAdrI();
          for(size_t i = 0; i < adrI.size(); ++i)
            if(adrI[i] < nInc) rhs[adrI[i]] += Be[i];
        }
      }
    }
  }
  void constrainEssentialComponents(const feSolution *) override {}
  void applyPeriodicity() override {}
  void permute() override {}
  bool solve(double *normDx, double *normResidual, double *normAxb, int *nIter) override
  {
    // As feLinearSystemMklPardiso::solve (:893-965): factor only when the
    // matrix was recomputed, otherwise solve with the previous factors.
    const auto &ia = crs->ia();
    const auto &ja = crs->ja();
    if(_recomputeMatrix || !factored) {
      std::vector<Eigen::Triplet<double>> trip;
      trip.reserve(values.size());
      for(feInt r = 0; r < nInc; ++r)
        for(feInt k = ia[r]; k < ia[r + 1]; ++k) trip.emplace_back(r, ja[k], values[k]);
      A = Eigen::SparseMatrix<double>(nInc, nInc);
      A.setFromTriplets(trip.begin(), trip.end());
      A.makeCompressed();
      if(useAmd) {
        luAmd.compute(A);
        if(luAmd.info() != Eigen::Success) return false;
      } else {
        lu.compute(A);
        if(lu.info() != Eigen::Success) return false;
      }
      factored = true;
    }
    Eigen::Map<Eigen::VectorXd> b(rhs.data(), nInc);
    Eigen::VectorXd x = useAmd ? Eigen::VectorXd(luAmd.solve(b)) : Eigen::VectorXd(lu.solve(b));
    for(feInt i = 0; i < nInc; ++i) du[i] = x[i];
    double mdu = 0, mr = 0, axb = 0;
    Eigen::VectorXd res = A * x - b;
    for(feInt i = 0; i < nInc; ++i) {
      mdu = std::max(mdu, std::fabs(du[i]));
      mr = std::max(mr, std::fabs(rhs[i]));
      axb = std::max(axb, std::fabs(res[i]));
    }
    *normDx = mdu; *normResidual = mr; *normAxb = axb; *nIter = 0;
    lastAxb = axb;
    return true;
  }
  void correctSolution(feSolution *sol, const bool correctDot) override
  {
    std::vector<double> &s = correctDot ? sol->getSolutionDot() : sol->getSolution();
    for(feInt i = 0; i < nInc; ++i) s[i] += du[i];
  }
  void assignResidualToDCResidual(feSolutionContainer *c) override
  {
    for(feInt i = 0; i < nInc; ++i) c->_fResidual[0][i] = rhs[i];
  }
  void applyCorrectionToResidual(double coeff, std::vector<double> &d) override
  {
    for(feInt i = 0; i < nInc; ++i) rhs[i] += coeff * d[i];
  }
  void viewMatrix() const override {}
  void viewRHS() const override {}
  void viewResidual() const override {}
  void writeMatrix(const std::string, const double) override {}
  void writeRHS(const std::string, const double) override {}
  void writeResidual(const std::string, const double) override {}
};

template <typename T>
void write_raw(const std::string &path, const std::vector<T> &v)
{
  std::ofstream f(path, std::ios::binary);
  f.write(reinterpret_cast<const char *>(v.data()), v.size() * sizeof(T));
}

double g_re = 40.0;
double g_dt = 0.01;
int g_steps = 6;

// Lid-driven cavity: u = (1, 0) on the lid y = 1, zero elsewhere.
void cavity_lid(const feFunctionArguments &a, const std::vector<double> &, std::vector<double> &r)
{
  r[0] = std::fabs(a.pos[1] - 1.0) <= 1e-12 ? 1.0 : 0.0;
  r[1] = 0.0;
}

double sinsin(const feFunctionArguments &a, const std::vector<double> &)
{
  return sin(M_PI * a.pos[0]) * sin(M_PI * a.pos[1]);
}
double sinsin_src(const feFunctionArguments &a, const std::vector<double> &)
{
  return -2. * M_PI * M_PI * sin(M_PI * a.pos[0]) * sin(M_PI * a.pos[1]);
}
double sinsinsin(const feFunctionArguments &a, const std::vector<double> &)
{
  return sin(M_PI * a.pos[0]) * sin(M_PI * a.pos[1]) * sin(M_PI * a.pos[2]);
}
double sinsinsin_src(const feFunctionArguments &a, const std::vector<double> &)
{
  return -3. * M_PI * M_PI * sin(M_PI * a.pos[0]) * sin(M_PI * a.pos[1]) * sin(M_PI * a.pos[2]);
}
double kov_lambda() { return g_re / 2. - sqrt(g_re * g_re / 4. + 4. * M_PI * M_PI); }
void kov_u(const feFunctionArguments &a, const std::vector<double> &, std::vector<double> &r)
{
  const double l = kov_lambda(), e = exp(l * a.pos[0]);
  r[0] = 1. - e * cos(2. * M_PI * a.pos[1]);
  r[1] = l / (2. * M_PI) * e * sin(2. * M_PI * a.pos[1]);
}
double kov_p(const feFunctionArguments &a, const std::vector<double> &)
{
  return 0.5 * (1. - exp(2. * kov_lambda() * a.pos[0]));
}
void mms_u(const feFunctionArguments &a, const std::vector<double> &, std::vector<double> &r)
{
  const double x = a.pos[0], y = a.pos[1];
  r[0] = pow(x, 4) * pow(y, 4);
  r[1] = -4. / 5. * pow(x, 3) * pow(y, 5);
}
double mms_p(const feFunctionArguments &a, const std::vector<double> &)
{
  const double x = a.pos[0], y = a.pos[1];
  return x * x * y * y;
}
void mms_src(const feFunctionArguments &a, const std::vector<double> &, std::vector<double> &res)
{
  // Same manufactured source as tests/withLinearSolver/navier_stokes.cpp:33-51.
  const double x = a.pos[0], y = a.pos[1];
  const double mdpdx[2] = {-2. * x * y * y, -2. * x * x * y};
  const double lap[2] = {12. * (x * x * y * y * y * y + x * x * x * x * y * y),
                         -4. / 5. * (6. * x * y * y * y * y * y + 20. * x * x * x * y * y * y)};
  const double u[2] = {x * x * x * x * y * y * y * y, (-4. / 5. * x * x * x * y * y * y * y * y)};
  const double g[2][2] = {{4. * x * x * x * y * y * y * y, -12. * x * x * y * y * y * y * y / 5.},
                          {4. * x * x * x * x * y * y * y, -4. * x * x * x * y * y * y * y}};
  const double c[2] = {u[0] * g[0][0] + u[1] * g[1][0], u[0] * g[0][1] + u[1] * g[1][1]};
  res[0] = -(-c[0] + mdpdx[0] + lap[0]);
  res[1] = -(-c[1] + mdpdx[1] + lap[1]);
}

}  // namespace

// The solution as the reference's legacy VTK exporter writes it
// (feExporterVTK::writeStep, src/feExporter.cpp:854-990).
// With a pressure field, also the pressure alone (requiredFields {"P"}):
// a P1 field only, so 3-node triangles without mid-edge nodes.
feStatus write_vtk(const std::string &dir, feMetaNumber &numbering, feSolution &sol, feMesh2DP1 &mesh,
                   const std::vector<feSpace *> &spaces)
{
  feExporter *exporter = nullptr;
  feCheck(createVisualizationExporter(exporter, VTK, &numbering, &sol, &mesh, spaces));
  feCheck(exporter->writeStep(dir + "/solution.vtk"));
  delete exporter;
  bool hasP = false;
  for(feSpace *s : spaces) hasP |= s->getFieldID() == "P";
  if(hasP) {
    feCheck(createVisualizationExporter(exporter, VTK, &numbering, &sol, &mesh, spaces));
    feCheck(exporter->writeStep(dir + "/solution_p.vtk", {"P"}));
    delete exporter;
  }
  return FE_STATUS_OK;
}

int main(int argc, char **argv)
{
  if(argc < 4) {
    fprintf(stderr, "usage: %s mesh.msh diffusion|diffusion3d|ns_kovasznay|ns_mms|ns_cavity_bdf2 outdir [Re] [seed] [dt] [steps]\n", argv[0]);
    return 2;
  }
  const std::string meshFile = argv[1], problem = argv[2], out = argv[3];
  if(argc > 4) g_re = atof(argv[4]);
  const unsigned long seed = argc > 5 ? strtoul(argv[5], nullptr, 10) : 1;
  if(argc > 6) g_dt = atof(argv[6]);
  if(argc > 7) g_steps = atoi(argv[7]);
  setVerbose(getenv("FE_HARNESS_VERBOSE") ? atoi(getenv("FE_HARNESS_VERBOSE")) : 0);

  feMesh2DP1 mesh(meshFile);
  feFunction fSinSin(sinsin), fSrc(sinsin_src), fKovP(kov_p), fMmsP(mms_p);
  feFunction fSin3(sinsinsin), fSrc3(sinsinsin_src);
  const bool dim3 = problem == "diffusion3d";
  feVectorFunction fKovU(kov_u), fMmsU(mms_u), fMmsSrc(mms_src);
  feConstantFunction fMu(1.0 / g_re);
  feVectorFunction fLid(cavity_lid);
  const bool cavity = problem == "ns_cavity_bdf2";

  std::vector<feSpace *> spaces, essential, domainSpaces;
  std::vector<feBilinearForm *> forms;
  int degQ = 4;
  // Tetrahedral runs may ask for another rule (its values are written out).
  if(dim3 && getenv("FE_HARNESS_QDEG")) degQ = atoi(getenv("FE_HARNESS_QDEG"));
  if(problem == "diffusion" || dim3) {
    feSpace *u = nullptr, *uB = nullptr;
    feCheck(createFiniteElementSpace(uB, &mesh, elementType::LAGRANGE, 2, "U", "Bord", degQ, dim3 ? &fSin3 : &fSinSin));
    feCheck(createFiniteElementSpace(u, &mesh, elementType::LAGRANGE, 2, "U", "Domaine", degQ, &scalarConstant::zero));
    spaces = {uB, u};
    essential = {uB};
    domainSpaces = {u};
  } else {
    degQ = 8;
    const bool kov = problem == "ns_kovasznay";
    feSpace *u = nullptr, *uB = nullptr, *p = nullptr, *pP = nullptr;
    const feVectorFunction *uex = cavity ? &fLid : kov ? &fKovU : &fMmsU;
    const feFunction *pex = cavity ? &scalarConstant::zero : kov ? &fKovP : &fMmsP;
    feCheck(createFiniteElementSpace(u, &mesh, elementType::VECTOR_LAGRANGE, 2, "U", "Domaine", degQ, uex));
    feCheck(createFiniteElementSpace(uB, &mesh, elementType::VECTOR_LAGRANGE, 2, "U", "Bord", degQ, uex));
    feCheck(createFiniteElementSpace(p, &mesh, elementType::LAGRANGE, 1, "P", "Domaine", degQ, pex));
    feCheck(createFiniteElementSpace(pP, &mesh, elementType::LAGRANGE, 1, "P", "PointPression", degQ, pex));
    spaces = {u, uB, p, pP};
    essential = {uB, pP};
    domainSpaces = {u, p};
  }
  feMetaNumber numbering(&mesh, spaces, essential);
  feSolution sol(numbering.getNbDOFs(), spaces, essential);

  if(problem == "diffusion" || dim3) {
    feBilinearForm *diff = nullptr, *src = nullptr;
    if(dim3)
      feCheck(createBilinearForm(diff, {domainSpaces[0]}, new feSysElm_Diffusion<3>(&scalarConstant::one)));
    else
      feCheck(createBilinearForm(diff, {domainSpaces[0]}, new feSysElm_Diffusion<2>(&scalarConstant::one)));
    feCheck(createBilinearForm(src, {domainSpaces[0]}, new feSysElm_Source(dim3 ? &fSrc3 : &fSrc)));
    forms = {diff, src};
  } else {
    feSpace *u = domainSpaces[0], *p = domainSpaces[1];
    const bool kov = problem == "ns_kovasznay";
    feBilinearForm *conv = nullptr, *divU = nullptr, *sigma = nullptr, *src = nullptr;
    // Sign convention of the steady tests (navier_stokes.cpp:83-90), or of
    // the unsteady ones (vectorFEunsteady.cpp:562-584) for the cavity.
    const feConstantFunction *cConv = cavity ? &scalarConstant::one : &scalarConstant::minusOne;
    const feConstantFunction *cSigma = cavity ? &scalarConstant::minusOne : &scalarConstant::one;
    feCheck(createBilinearForm(conv, {u}, new feSysElm_VectorConvectiveAcceleration<2>(cConv)));
    feCheck(createBilinearForm(divU, {p, u}, new feSysElm_MixedDivergence<2>(&scalarConstant::one)));
    feCheck(createBilinearForm(sigma, {u, p}, new feSysElm_DivergenceNewtonianStress<2>(cSigma, (kov || cavity) ? &fMu : &scalarConstant::one)));
    forms = {conv, divU, sigma};
    if(cavity) {
      feBilinearForm *mass = nullptr;
      feCheck(createBilinearForm(mass, {u}, new feSysElm_TransientVectorMass<2>(&scalarConstant::one)));
      forms.insert(forms.begin(), mass);
    } else if(!kov) {
      feCheck(createBilinearForm(src, {u}, new feSysElm_VectorSource<2>(&fMmsSrc)));
      forms.push_back(src);
    }
  }

  feLinearSystemRef *sys = new feLinearSystemRef(forms, &numbering);
  const feInt nInc = numbering.getNbUnknowns(), nDofs = numbering.getNbDOFs();

  // Element tables of the domain spaces (fused layout: first space then second).
  const int nElm = mesh.getNumElements("Domaine");
  std::vector<int64_t> adr;
  for(int e = 0; e < nElm; ++e)
    for(feSpace *s : domainSpaces) {
      std::vector<feInt> a(s->getNumFunctions());
      s->initializeAddressingVector(e, a);
      for(feInt v : a) adr.push_back(v);
    }
  const feCncGeo *cnc = forms[0]->getCncGeo();
  std::vector<int64_t> colOff = {0};
  std::vector<int32_t> colEl;
  for(int c = 0; c < cnc->getNbColor(); ++c) {
    for(int e : cnc->getListElmPerColor()[c]) colEl.push_back(e);
    colOff.push_back((int64_t)colEl.size());
  }
  std::vector<int64_t> ia(sys->crs->ia().begin(), sys->crs->ia().end());
  std::vector<int64_t> ja(sys->crs->ja().begin(), sys->crs->ja().end());

  // Quadrature rule of the domain space.
  std::vector<double> quad;
  {
    feSpace *s = domainSpaces[0];
    const auto &w = s->getQuadratureWeights();
    const auto &r = s->getRQuadraturePoints();
    const auto &q = s->getSQuadraturePoints();
    const auto &z = s->getTQuadraturePoints();
    for(size_t k = 0; k < w.size(); ++k) {
      quad.push_back(r[k]);
      quad.push_back(q[k]);
      if(dim3) quad.push_back(z[k]);  // 3D rules: r, s, t, w
      quad.push_back(w[k]);
    }
  }
  write_raw(out + "/quad.f64", quad);  // also when a later step fails

  if(cavity) {
    // BDF2 from rest (BDF1 starter of 0.1 dt, the reference's default) with
    // tight absolute Newton tolerances; writes the solution after every step.
    const int nSteps = g_steps;
    TimeIntegrator *ti = nullptr;
    std::vector<feNorm *> norms;
    feNLSolverOptions NL{1e-11, 1e-13, 1e12, 30, 3, 1e-1};
    feCheck(createTimeIntegrator(ti, timeIntegratorScheme::BDF2, NL, sys, &sol, &mesh, norms, {nullptr, 1, ""},
                                 0.0, nSteps * g_dt, nSteps));
    feCheck(ti->makeSteps(nSteps));
    std::vector<double> traj = sol.getSolution();
    {
      // Transient assembly state: the last step's BDF coefficient c0 and
      // time derivative, unknowns replaced by U(-1,1) (std::mt19937_64 with
      // the seed): the residual and the Jacobian, TransientVectorMass
      // included, at that state.
      std::vector<double> ut = traj;
      std::mt19937_64 rng(seed);
      std::uniform_real_distribution<double> U(-1.0, 1.0);
      for(feInt i = 0; i < nInc; ++i) ut[i] = U(rng);
      sol.getSolution() = ut;
      solAtTimeN = ut;
      const std::vector<double> udt = sol.getSolutionDot();
      sys->setMatrixToZero();
      sys->setResidualToZero();
      sys->assembleResiduals(&sol);
      sys->assembleMatrices(&sol, false);
      write_raw(out + "/u0.f64", ut);
      write_raw(out + "/udot0.f64", udt);
      write_raw(out + "/values0.f64", sys->values);
      write_raw(out + "/rhs0.f64", sys->rhs);
      std::vector<double> c0t = {sol.getC0(), sol.getCurrentTime()};
      write_raw(out + "/c0t.f64", c0t);
      sol.getSolution() = traj;
    }
    feCheck(write_vtk(out, numbering, sol, mesh, spaces));
    write_raw(out + "/ia.i64", ia);
    write_raw(out + "/ja.i64", ja);
    write_raw(out + "/adr.i64", adr);
    write_raw(out + "/color_offsets.i64", colOff);
    write_raw(out + "/color_elements.i32", colEl);
    write_raw(out + "/traj.f64", traj);
    write_raw(out + "/quad.f64", quad);
    FILE *f = fopen((out + "/meta.txt").c_str(), "w");
    fprintf(f, "problem %s\nnInc %ld\nnDofs %ld\nnnz %zu\nnElm %d\nnColors %d\nnloc %zu\nquad_degree %d\nre %.17g\nseed %lu\ndt %.17g\nsteps %d\n",
            problem.c_str(), (long)nInc, (long)nDofs, ja.size(), nElm, cnc->getNbColor(),
            adr.size() / nElm, degQ, g_re, seed, g_dt, nSteps);
    fclose(f);
    delete ti;
    delete sys;
    for(auto *fm : forms) delete fm;
    for(auto *s : spaces) delete s;
    return 0;
  }

  // Assembly state: essential values from the exact solution, unknowns
  // uniform in [-1,1] (std::mt19937_64 with the given seed).
  TimeIntegrator *ti = nullptr;
  std::vector<feNorm *> norms;
  feNLSolverOptions NL{1e-10, 1e-12, 1e4, 30, 3, 1e-1};
  feCheck(createTimeIntegrator(ti, timeIntegratorScheme::STATIONARY, NL, sys, &sol, &mesh, norms, {nullptr, 1, ""}));
  std::vector<double> u0 = sol.getSolution();  // essential DOFs initialised by the integrator
  if(getenv("FE_HARNESS_U0")) {
    // Unknowns of the assembly state from a raw file of nInc doubles (large
    // cases: the fixture script draws them from a seed the tests can redraw).
    FILE *fu = fopen(getenv("FE_HARNESS_U0"), "rb");
    if(!fu || fread(u0.data(), sizeof(double), nInc, fu) != (size_t)nInc) {
      fprintf(stderr, "cannot read %ld doubles from %s\n", (long)nInc, getenv("FE_HARNESS_U0"));
      return 1;
    }
    fclose(fu);
  } else {
    std::mt19937_64 rng(seed);
    std::uniform_real_distribution<double> U(-1.0, 1.0);
    for(feInt i = 0; i < nInc; ++i) u0[i] = U(rng);
  }
  std::vector<double> ubc = sol.getSolution();
  sol.getSolution() = u0;
  solAtTimeN = sol.getSolution();
  sys->setToZero();
  sys->assembleResiduals(&sol);
  sys->assembleMatrices(&sol, false);
  std::vector<double> values0 = sys->values, rhs0 = sys->rhs;

  if(getenv("FE_HARNESS_NOSOLVE")) {
    // Assembly state only (large meshes whose direct solve takes long).
    write_raw(out + "/ia.i64", ia);
    write_raw(out + "/ja.i64", ja);
    write_raw(out + "/adr.i64", adr);
    write_raw(out + "/color_offsets.i64", colOff);
    write_raw(out + "/color_elements.i32", colEl);
    write_raw(out + "/u0.f64", u0);
    write_raw(out + "/values0.f64", values0);
    write_raw(out + "/rhs0.f64", rhs0);
    FILE *f = fopen((out + "/meta.txt").c_str(), "w");
    fprintf(f, "problem %s\nnInc %ld\nnDofs %ld\nnnz %zu\nnElm %d\nnColors %d\nnloc %zu\nquad_degree %d\nre %.17g\nseed %lu\n",
            problem.c_str(), (long)nInc, (long)nDofs, ja.size(), nElm, cnc->getNbColor(),
            adr.size() / nElm, degQ, g_re, seed);
    fclose(f);
    return 0;
  }
  // Converged solution from the BC-initialised zero state.
  for(feInt i = 0; i < nInc; ++i) ubc[i] = 0.;
  sol.getSolution() = ubc;
  feCheck(ti->makeSteps(1));
  std::vector<double> usol = sol.getSolution();
  sys->setToZero();
  solAtTimeN = usol;
  sys->assembleResiduals(&sol);
  double rfinal = 0;
  sys->getRHSMaxNorm(&rfinal);
  if(!dim3) feCheck(write_vtk(out, numbering, sol, mesh, spaces));

  write_raw(out + "/ia.i64", ia);
  write_raw(out + "/ja.i64", ja);
  write_raw(out + "/adr.i64", adr);
  write_raw(out + "/color_offsets.i64", colOff);
  write_raw(out + "/color_elements.i32", colEl);
  write_raw(out + "/u0.f64", u0);
  write_raw(out + "/values0.f64", values0);
  write_raw(out + "/rhs0.f64", rhs0);
  write_raw(out + "/usol.f64", usol);
  write_raw(out + "/quad.f64", quad);
  FILE *f = fopen((out + "/meta.txt").c_str(), "w");
  fprintf(f, "problem %s\nnInc %ld\nnDofs %ld\nnnz %zu\nnElm %d\nnColors %d\nnloc %zu\nquad_degree %d\nre %.17g\nseed %lu\nfinal_residual %.17g\n",
          problem.c_str(), (long)nInc, (long)nDofs, ja.size(), nElm, cnc->getNbColor(),
          adr.size() / nElm, degQ, g_re, seed, rfinal);
  fclose(f);
  delete ti;
  delete sys;
  for(auto *fm : forms) delete fm;
  for(auto *s : spaces) delete s;
  return 0;
}
