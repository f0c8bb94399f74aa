// feLinearSystemCUDA: the drop-in feLinearSystem backend of feNG
// (src/feLinearSystem.h:43-169) that runs element assembly, the colored
// scatter and the Krylov solve on the GPU through the C ABI of
// include/feng_cuda.h.  It is meant to be compiled inside feNG (it includes
// feNG's headers) next to feLinearSystemMklPardiso / feLinearSystemPETSc;
// it is not part of the CUDA library itself.
//
// Usage, in place of createLinearSystem(system, MKLPARDISO, forms, &numbering):
//
//   std::vector<fe_form_desc> desc = {
//     {FE_FORM_VECTOR_CONVECTIVE_ACCELERATION, -1.0},
//     {FE_FORM_MIXED_DIVERGENCE, 1.0},
//     {FE_FORM_DIV_NEWTONIAN_STRESS, 1.0, 1.0 / Re}};   // one entry per form, same order
//   fe_cuda_options opt = feLinearSystemCUDA::defaultOptions(8);
//   feLinearSystem *system = new feLinearSystemCUDA(forms, &numbering, &mesh, desc, opt);
//
// The coefficients are passed explicitly because feSysElm keeps its
// feFunction pointers private; constant coefficients (feConstantFunction)
// and the closed FE_SRC_* source registry are what the device evaluates.
#ifndef FELINEARSYSTEMCUDA_H
#define FELINEARSYSTEMCUDA_H

#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>

#include "feLinearSystem.h"
#include "feng_cuda.h"

class feLinearSystemCUDA : public feLinearSystem
{
  // Reads the reference's own pattern (protected members of the CSR builder).
  struct Pattern : public feEZCompressedRowStorage {
    using feEZCompressedRowStorage::feEZCompressedRowStorage;
    const std::vector<feInt> &ia() const { return ia_Pardiso; }
    const std::vector<feInt> &ja() const { return ja_Pardiso; }
  };

  fe_cuda_system *_sys = nullptr;
  feInt _nInc = 0, _nDofs = 0, _nnz = 0;
  bool _constrainInit = false, _periodicInit = false;
  int _nIterLast = 0;

  static void check(int status, const char *what)
  {
    if(status != FE_CUDA_OK)
      throw std::runtime_error(std::string(what) + ": " + fe_cuda_last_error());
  }

  void upload(const feSolution *sol)
  {
    check(fe_cuda_set_solution(_sys, sol->getSolution().data(), sol->getSolutionDot().data()),
          "fe_cuda_set_solution");
    check(fe_cuda_set_time(_sys, sol->getCurrentTime(), sol->getC0()), "fe_cuda_set_time");
  }

public:
  static fe_cuda_options defaultOptions(int quadratureDegree)
  {
    fe_cuda_options o{};
    o.krylov = 1;            // FGMRES
    o.restart = 50;
    o.max_iter = 10000;
    o.rel_tol = 1e-8;        // feLinearSystem::_rel_tol
    o.abs_tol = 1e-14;
    o.div_tol = 1e6;
    o.precond = 3;           // multigrid saddle-point / scalar preconditioner
    o.pc_block_rows = 256;
    o.precision = 0;
    o.quad_degree = quadratureDegree;
    o.mg_inner = 0;
    o.mg_smooth = 1;
    o.gs_passes = 1;
    return o;
  }

  feLinearSystemCUDA(std::vector<feBilinearForm *> bilinearForms, const feMetaNumber *numbering,
                     feMesh *mesh, const std::vector<fe_form_desc> &desc, const fe_cuda_options &opt)
    : feLinearSystem(bilinearForms, numbering)
  {
    if(desc.size() != bilinearForms.size())
      throw std::runtime_error("one fe_form_desc per bilinear form");
    _nInc = numbering->getNbUnknowns();
    _nDofs = numbering->getNbDOFs();
    // The fused element layout is the column layout of the widest form
    // (U then P for Taylor-Hood, U for a scalar field).
    feBilinearForm *widest = bilinearForms[0];
    for(feBilinearForm *f : bilinearForms)
      if(f->getLocalMatrixN() > widest->getLocalMatrixN()) widest = f;
    const int nloc = (int)widest->getLocalMatrixN();
    const int elemType = nloc == 15 ? FE_ELEM_TAYLOR_HOOD : nloc == 6 ? FE_ELEM_P2 : 0;
    if(!elemType) throw std::runtime_error("unsupported element layout");
    const feCncGeo *cnc = widest->getCncGeo();
    const int nElm = cnc->getNumElements();
    std::vector<int64_t> adr((size_t)nElm * nloc);
    std::vector<double> xy((size_t)nElm * 6), coord(3 * cnc->getNumVerticesPerElem());
    for(int e = 0; e < nElm; ++e) {
      widest->initializeAddressingVectors(e);
      const std::vector<feInt> &a = widest->getAdrJ();
      for(int i = 0; i < nloc; ++i) adr[(size_t)e * nloc + i] = a[i];
      mesh->getCoord(widest->getCncGeoTag(), e, coord);
      for(int k = 0; k < 3; ++k) {
        xy[6 * e + 2 * k] = coord[3 * k];
        xy[6 * e + 2 * k + 1] = coord[3 * k + 1];
      }
    }
    std::vector<int64_t> colorOffsets(1, 0);
    std::vector<int32_t> colorElements;
    for(int c = 0; c < cnc->getNbColor(); ++c) {
      for(int e : cnc->getListElmPerColor()[c]) colorElements.push_back(e);
      colorOffsets.push_back((int64_t)colorElements.size());
    }
    Pattern pat(_nInc, _formMatrices, _numMatrixForms, numbering);
    std::vector<int64_t> ia(pat.ia().begin(), pat.ia().end());
    std::vector<int32_t> ja(pat.ja().begin(), pat.ja().end());
    _nnz = (feInt)ja.size();
    check(fe_cuda_system_create_from_tables(elemType, nElm, adr.data(), xy.data(), _nInc, _nDofs,
                                            cnc->getNbColor(), colorOffsets.data(), colorElements.data(),
                                            ia.data(), ja.data(), nullptr, desc.data(), (int)desc.size(),
                                            &opt, &_sys),
          "fe_cuda_system_create_from_tables");
  }

  ~feLinearSystemCUDA() { fe_cuda_system_destroy(_sys); }

  feInt getSystemSize() const override { return _nInc; }

  void getRHSMaxNorm(double *norm) const override
  {
    check(fe_cuda_get_rhs_max_norm(_sys, norm), "fe_cuda_get_rhs_max_norm");
  }
  void getResidualMaxNorm(double *norm) const override
  {
    // reduced on the device: du stays there
    check(fe_cuda_get_du_max_norm(_sys, norm), "fe_cuda_get_du_max_norm");
  }

  void setToZero() override { check(fe_cuda_set_to_zero(_sys), "fe_cuda_set_to_zero"); }
  void setMatrixToZero() override { check(fe_cuda_set_matrix_to_zero(_sys), "fe_cuda_set_matrix_to_zero"); }
  void setResidualToZero() override { check(fe_cuda_set_residual_to_zero(_sys), "fe_cuda_set_residual_to_zero"); }

  void assemble(const feSolution *sol, const bool onlyTransient) override
  {
    assembleMatrices(sol, onlyTransient);
    assembleResiduals(sol);
  }
  void assembleMatrices(const feSolution *sol, const bool onlyTransient) override
  {
    // The reference's backends then assemble only the forms with
    // isTransientMatrix() (solves for the time derivative); the fused device
    // kernels assemble every form together, so that mode is refused rather
    // than silently solved with the full Jacobian.
    if(onlyTransient)
      throw std::runtime_error("feLinearSystemCUDA: transient-only matrix assembly is not offloaded");
    upload(sol);
    check(fe_cuda_assemble_matrices(_sys), "fe_cuda_assemble_matrices");
  }
  void assembleResiduals(const feSolution *sol) override
  {
    upload(sol);
    check(fe_cuda_assemble_residuals(_sys), "fe_cuda_assemble_residuals");
  }

  // Partially essential vector spaces and periodicity are not offloaded.
  // Rows of the essential components of vector spaces, gathered once as
  // feLinearSystemMklPardiso::constrainEssentialComponents does
  // (src/feLinearSystemMklPardiso.cpp:994-1050), then constrained on the device.
  void constrainEssentialComponents(const feSolution *sol) override
  {
    if(!_constrainInit) {
      _constrainInit = true;
      std::vector<int64_t> rows;
      std::vector<feInt> adr;
      for(const auto &space : sol->_spaces) {
        const int nc = space->getNumComponents(), nf = space->getNumFunctions(), ne = space->getNumElements();
        if(nc <= 1) continue;
        adr.resize(nf);
        for(int i = 0; i < nc; ++i) {
          if(!space->isEssentialComponent(i)) continue;
          for(int e = 0; e < ne; ++e) {
            space->initializeAddressingVector(e, adr);
            for(int j = 0; j < nf; ++j)
              if(j % nc == i && adr[j] < _nInc) rows.push_back((int64_t)adr[j]);
          }
        }
      }
      check(fe_cuda_set_constrained_rows(_sys, rows.data(), (int64_t)rows.size()), "fe_cuda_set_constrained_rows");
    }
    check(fe_cuda_constrain_essential_components(_sys), "fe_cuda_constrain_essential_components");
  }
  // Periodic slave rows (feLinearSystemMklPardiso::applyPeriodicity, :1119-1149).
  void applyPeriodicity() override
  {
    if(!_periodicInit) {
      _periodicInit = true;
      std::vector<int64_t> m, sl;
      for(const auto &pr : _numbering->PeriodicDOF()) {
        m.push_back(pr.first);
        sl.push_back(pr.second);
      }
      check(fe_cuda_set_periodic_pairs(_sys, m.data(), sl.data(), (int64_t)m.size()), "fe_cuda_set_periodic_pairs");
    }
    check(fe_cuda_apply_periodicity(_sys), "fe_cuda_apply_periodicity");
  }
  void permute() override {}

  bool solve(double *normDx, double *normResidual, double *normAxb, int *nIter) override
  {
    check(fe_cuda_set_tolerances(_sys, _rel_tol, _abs_tol, _max_iter), "fe_cuda_set_tolerances");
    const int s = fe_cuda_solve(_sys, normDx, normResidual, normAxb, nIter);
    _nIterLast = *nIter;
    return s == FE_CUDA_OK;
  }

  void correctSolution(feSolution *sol, const bool correctSolutionDot) override
  {
    std::vector<double> du(_nInc);
    check(fe_cuda_get_du(_sys, du.data()), "fe_cuda_get_du");
    std::vector<double> &s = correctSolutionDot ? sol->getSolutionDot() : sol->getSolution();
    for(feInt i = 0; i < _nInc; ++i) s[i] += du[i];
  }

  void assignResidualToDCResidual(feSolutionContainer *c) override
  {
    std::vector<double> rhs(_nInc);
    check(fe_cuda_get_rhs(_sys, rhs.data()), "fe_cuda_get_rhs");
    for(feInt i = 0; i < _nInc; ++i) c->_fResidual[0][i] = rhs[i];
  }
  void applyCorrectionToResidual(double, std::vector<double> &) override
  {
    throw std::runtime_error("deferred-correction residual updates are not offloaded");
  }

  void viewMatrix() const override {}
  void viewRHS() const override {}
  void viewResidual() const override {}
  void writeMatrix(const std::string fileName, const double) override
  {
    std::vector<double> v(_nnz);
    check(fe_cuda_get_matrix(_sys, v.data()), "fe_cuda_get_matrix");
    FILE *f = fopen(fileName.c_str(), "w");
    if(!f) return;
    for(double x : v) fprintf(f, "%+-1.16e\n", x);
    fclose(f);
  }
  void writeRHS(const std::string fileName, const double) override
  {
    std::vector<double> v(_nInc);
    check(fe_cuda_get_rhs(_sys, v.data()), "fe_cuda_get_rhs");
    FILE *f = fopen(fileName.c_str(), "w");
    if(!f) return;
    for(double x : v) fprintf(f, "%+-1.16e\n", x);
    fclose(f);
  }
  void writeResidual(const std::string fileName, const double) override
  {
    std::vector<double> v(_nInc);
    check(fe_cuda_get_du(_sys, v.data()), "fe_cuda_get_du");
    FILE *f = fopen(fileName.c_str(), "w");
    if(!f) return;
    for(double x : v) fprintf(f, "%+-1.16e\n", x);
    fclose(f);
  }
};

#endif
