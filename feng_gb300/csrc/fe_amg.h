// Smoothed-aggregation algebraic multigrid (Vanek, Mandel, Brezina, "Algebraic
// multigrid by smoothed aggregation for second and fourth order elliptic
// problems", Computing 56, 1996) for scalar SPD operators: host set-up once
// per mesh, V-cycles with Chebyshev smoothing on the device.
//
// Used as the velocity-block solve of the block-triangular saddle-point
// preconditioner and as the preconditioner of scalar diffusion.  The
// reference has no counterpart (its solves are PETSc/MKL library calls); it
// is the device replacement that makes the Krylov solve converge in a
// mesh-independent number of iterations.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

namespace feng {

struct HostCSR {
  int64_t n = 0, m = 0;  // rows, columns
  std::vector<int64_t> ia;
  std::vector<int32_t> ja;
  std::vector<double> a;
  int64_t nnz() const { return ia.empty() ? 0 : ia.back(); }
};

struct AMGLevel {
  HostCSR A, P, R;
  std::vector<double> dinv;
  double lmax = 0;  // spectral radius estimate of D^-1 A
};

struct AMGHierarchy {
  std::vector<AMGLevel> levels;  // last level: only A (coarsest)
  std::vector<double> coarseInv; // dense inverse of the coarsest A, row-major
};

struct AMGParams {
  double theta = 0.08;     // strength of connection
  int maxLevels = 12;
  int64_t coarseSize = 1200;
  int chebyDegree = 2;
  // smoothing interval [low, high] * lmax; degree 1 is damped Jacobi with
  // weight 1 / theta, theta = (low + high) / 2 * lmax = 0.7 lmax: measured on
  // the 256 x 256 Kovasznay system (FGMRES iterations per solve for theta /
  // lmax = 0.525 / 0.6 / 0.675 / 0.7 / 0.775: diverged / 574 / 553 / 555 /
  // 555), the flat side of the optimum, away from the divergence
  double chebyLow = 0.35;
  double chebyHigh = 1.05;
  // levels whose operator averages more entries per row take the tentative
  // prolongator unsmoothed (smoothing it multiplies the stencil of the next
  // Galerkin operator: 189 -> 2,427 entries per row on the 32^3 cube's
  // shifted velocity operator; two-dimensional P2 hierarchies stay below 48)
  double smoothMaxRow = 64.0;
  // smooth the prolongator with the filtered operator (weak couplings lumped
  // onto the diagonal): the transient velocity hierarchies (K + (c0/mu) M),
  // whose mass couplings are weak; measured: cavity 32.9 -> 30.3 ms per step,
  // 64^3 cube 250 -> 234 ms, at the same iteration counts, while the steady
  // Kovasznay operator needs 674 instead of 555 iterations with it
  bool filterSmoothing = false;
};

int amg_build(const HostCSR &A, const AMGParams &p, AMGHierarchy &H);

template <typename V>
struct DevLevelT;

// Device hierarchy and V-cycle, in FP64 or FP32.
class AMGDevice {
 public:
  ~AMGDevice();
  int upload(const AMGHierarchy &H, const AMGParams &p, int fp32, cudaStream_t s);
  // x = V-cycle(b) for the finest operator (x overwritten).
  void vcycle64(const double *b, double *x);
  void vcycle32(const float *b, float *x);
  // The same V-cycle on two right-hand sides stored interleaved
  // (b[2 i + c], component c of row i): one pass over each operator.
  // The caller's vector for the result of a paired V-cycle: component c of
  // finest row i goes, times *scale, to z[dofX[i]] (c = 0) or z[dofY[i]].
  struct OutMap {
    const int32_t *dofX = nullptr, *dofY = nullptr;
    const double *scale = nullptr;
    void *z = nullptr;
    // Optional pressure fold of the steady saddle-point preconditioner
    // (bgu set): the velocity result is (x - c bgu) * scale, c = *cr and
    // bgu interleaved like x, and extra blocks of the same launch write the
    // nP pressure rows z[pRows[k]] = sc_k (r_i - c m_k / cMc) + c / cSc,
    // i = pRows[k], sc = pScale (the vector type), m = pMass,
    // cSc = consts[1], cMc = consts[2].
    const double *cr = nullptr;
    const void *bgu = nullptr;
    int64_t nP = 0;
    const int32_t *pRows = nullptr;
    const void *pScale = nullptr;
    const double *pMass = nullptr, *consts = nullptr;
    const void *r = nullptr;
  };
  // Whether the finest level runs on its sliced-ELL copy (then a paired
  // V-cycle with an OutMap always writes through it).
  bool fineSell() const { return !lv_.empty() && lv_[0].sellPtr != nullptr; }
  // Both components at once (x, b interleaved).  With om, the finest
  // post-smoothing pass writes the result through om when it can (then
  // returns true; x does not hold the result), otherwise x holds it.
  bool vcycle2_64(const double *b, double *x, const OutMap *om = nullptr);
  bool vcycle2_32(const float *b, float *x, const OutMap *om = nullptr);
  // Three interleaved components (b[3 i + c]): the velocity of tetrahedral
  // Taylor-Hood systems, one pass over each level operator; x holds the result.
  void vcycle3_64(const double *b, double *x);
  void vcycle3_32(const float *b, float *x);
  // y = A x with the finest operator.
  void spmv64(const double *x, double *y);
  void spmv32(const float *x, float *y);
  // The finest-level pre-smoothing pass (zero start + first Chebyshev step
  // in one kernel) on two interleaved components, on the level's own work
  // vectors: one of the two finest-level kernels of every V-cycle.
  void fineStep2();
  // Algorithmic bytes of fineStep2: the level operator once (values,
  // columns, row pointers) and every vector entry it reads or writes once.
  int64_t fineStep2Bytes() const;
  int64_t n() const { return n0_; }
  int levels() const { return (int)lv_.size(); }
  double finestDiagSum() const { return diagSum_; }

 private:
  struct Lev {
    int64_t n = 0, nc = 0;
    int32_t *Aia = nullptr, *Aja = nullptr, *Pia = nullptr, *Pja = nullptr, *Ria = nullptr, *Rja = nullptr;
    void *Aa = nullptr, *Pa = nullptr, *Ra = nullptr, *dinv = nullptr, *diag = nullptr;
    void *x = nullptr, *b = nullptr, *r = nullptr, *d0 = nullptr, *d1 = nullptr;
    double lmax = 0;
    int lanesA = 4, lanesP = 4, lanesR = 4;
    // Sliced-ELL copy of A (slices of 32 rows, each padded to its longest
    // row with a valid column and value 0, entries column-major in the
    // slice): one thread per row, every load a full line.  Built for the
    // finest level only, for A and for the prolongation P.
    int32_t *sellPtr = nullptr;  // [nSlices + 1] first entry of each slice
    int32_t *sellCol = nullptr;
    void *sellVal = nullptr;
    int32_t *sellPPtr = nullptr, *sellPCol = nullptr;  // the same for P
    void *sellPVal = nullptr;
  };
  template <typename V, int NV> void vcycle_t(int l, const V *b, V *x);
  OutMap out_;
  bool outWritten_ = false;
  std::vector<Lev> lv_;
  void *coarseInv_ = nullptr;
  int64_t nCoarse_ = 0, n0_ = 0, nnz0_ = 0;
  int fp32_ = 0;
  AMGParams p_;
  double diagSum_ = 0;
  cudaStream_t s_ = 0;
  const int *skip_ = nullptr;

 public:
  // Device flag: when set (nonzero) every kernel of the V-cycle returns at
  // once (a converged Krylov cycle replayed from a CUDA graph).
  void setSkip(const int *skip) { skip_ = skip; }
};

}  // namespace feng
