// Device-resident BDF2 time integration with a choice of Newton initial
// guess, restating BDF2Integrator::makeSteps (src/feTimeIntegration.cpp:449-547)
// with its BDF1 starter (startWithBDF1, :383-435), the variable-step BDF2
// coefficients (feSolutionContainer::computeBDFCoefficients,
// src/feSolutionContainer.cpp:82-101) and the history rotation (rotate, :291-304).
//
// Initial guess of each step's Newton solve:
//   previous      u^n (what the reference does: the solution container's
//                 current solution carries over);
//   extrapolate   u^n + (dt_n / dt_{n-1}) (u^n - u^{n-1});
//   learned       the extrapolation plus a per-node correction predicted by
//                 an MLP (fe_mlp.h) from the last three solutions and the
//                 local geometry, trained online on the corrections that the
//                 converged steps reveal.  The correction is tried at full,
//                 half and quarter length; those candidates and the plain
//                 extrapolation are evaluated with the full FP64 residual and
//                 the smallest start is used, so the extrapolation is the
//                 fallback and the converged answer does not depend on the
//                 network.
// The Newton stop is relative to the residual of u^n at the new time level
// (fixed before any guess is formed), so a better guess can only save work.
#pragma once

#include <cstdint>

#include "fe_common.h"
#include "fe_mlp.h"
#include "fe_system.h"

namespace feng {

enum GuessKind { GUESS_PREVIOUS = 0, GUESS_EXTRAPOLATE = 1, GUESS_LEARNED = 2 };

struct TransientOptions {
  double dt = 0.005;
  double t0 = 0.0;
  int guess = GUESS_EXTRAPOLATE;
  int trainFrom = 20;      // first step whose (features, correction) pair trains the network
  int useFrom = 25;        // first step that may use the learned guess
  int trainIters = 8;      // Adam steps per time step
  int64_t batch = 16384;   // nodes per Adam step
  double lr = 1e-3;
  uint64_t seed = 1;
};

struct StepStats {
  int step = 0;
  double t = 0;
  int newtonIterations = 0, krylovIterations = 0, status = 0;
  int guessUsed = 0;            // GuessKind actually used
  double residualRef = 0;       // ||R(u^n)||inf at the new time level
  double residualGuess = 0;     // ||R||inf at the guess used
  double residualExtrap = 0;    // ||R||inf at the extrapolation (when evaluated, else 0)
  double residual = 0;          // final ||R||inf
  double stepMs = 0, guessMs = 0, trainMs = 0;
  double trainLoss = -1;        // loss of the last Adam step of this time step (-1: none)
  double guessScale = 0;        // step length alpha of the learned correction (0: none formed)
};

class Transient {
 public:
  ~Transient();
  int init(SystemCUDA *sys, const TransientOptions &o, const NewtonOptions &n);
  int step(StepStats &st);
  int64_t nodes() const { return nNodes_; }
  int stepsDone() const { return steps_; }
  // The learned guess's network parameters (MLPDims::P floats, host): a
  // network saved from an earlier run warm-starts this one (it counts as
  // trained, so it may be used from use_from on).
  int getNetwork(float *params) const
  {
    if(o_.guess != GUESS_LEARNED) { set_error("the integrator has no network (guess is not learned)"); return FE_INVALID_ARG; }
    return mlp_.getParams(params);
  }
  int setNetwork(const float *params)
  {
    if(o_.guess != GUESS_LEARNED) { set_error("the integrator has no network (guess is not learned)"); return FE_INVALID_ARG; }
    const int s = mlp_.setParams(params);
    if(s == 0 && trained_ == 0) trained_ = 1;
    return s;
  }

 private:
  SystemCUDA *sys_ = nullptr;
  TransientOptions o_;
  NewtonOptions no_;
  int64_t nNodes_ = 0;
  int32_t *nodeDof_ = nullptr;  // [nNodes x 4]: u, v, p0, p1 (p0 == p1 at vertices)
  float *geo_ = nullptr;        // [nNodes x 6] geometry features
  double *h3_ = nullptr;        // u^{n-2}
  double *ue_ = nullptr, *um_ = nullptr;  // extrapolated and learned guesses
  double *dv_ = nullptr, *jd_ = nullptr;  // learned correction d (unknowns) and J d
  float *X_ = nullptr, *Y_ = nullptr, *T_ = nullptr, *M_ = nullptr;
  float *sig_ = nullptr;        // [2] scales of the last solution differences (velocity, pressure)
  float *loss_ = nullptr;       // [1] last Adam loss
  int32_t *idx_ = nullptr;      // minibatch rows
  MLPDevice mlp_;
  double tHist_[3] = {0, 0, 0};  // times of u^n, u^{n-1}, u^{n-2}
  int nHist_ = 0;               // valid history levels
  int steps_ = 0;
  int trained_ = 0;             // time steps that trained the network
  int lostStreak_ = 0;          // consecutive steps the learned candidate lost
  int skipUntil_ = 0;           // back-off: no network evaluation or training before this step
  // step start, end of the guess, start and end of training
  cudaEvent_t e0_ = nullptr, e1_ = nullptr, e2_ = nullptr, e3_ = nullptr;
  int residualNorm(double *norm);
  int newton(double scale, NewtonStats &ns, bool residualReady = false);
  int bdf1Start(StepStats &st);
};

}  // namespace feng
