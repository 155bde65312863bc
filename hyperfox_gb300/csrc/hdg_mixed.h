// Mixed-precision HDG solve (internal): FP64 matrix-free residual of the full
// HDG system, FP32 element condensation / trace solve / recovery as the
// correction, iterative refinement until the FP64 residual is small.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

#include "hfx_device.h"
#include "krylov.h"

namespace hfx {

struct ResidualParams {
  int nCells;
  const double* coords;
  const int* cells;
  const int* cell2face;
  const uint8_t* perm;
  const int* face2cell;
  const double* tau;
  int tauVals;
  const double* kappa;
  int kc, kappaLayout;
  int srcMode;
  const double* src;
  double srcParam;
  double dt;
  const double* uOld;
  const double* tab;
  const int* itab;
  // state (u, q, lambda) in FP64
  const double* sol;    // [nCells][N]
  const double* flux;   // [nCells][N*D]
  const double* trace;  // [nFaces][NF]
  // outputs
  double* ru;  // [nCells][N]
  double* rq;  // [nCells][N*D]
  double* rl;  // [nCells][LL] element part of the face rows
};

struct FaceResidualParams {
  int nFaces, NF, F, LL;
  const int* face2cell;
  const int* cell2face;
  const uint8_t* perm;
  const uint8_t* isBnd;
  const double* rl;
  const double* dirichlet;
  const double* trace;
  double* rtrace;  // [nFaces][NF]
};

cudaError_t launch_residual(int dim, int order, const ResidualParams& p, const FaceResidualParams& fp,
                            cudaStream_t s);

// FP32 scatter of element S (and of S0 + the FP64 face residual into the FP32 rhs).
struct Scatter32Params {
  int nFaces, NF, LL, F;
  int64_t nBlocks;
  const int64_t* browptr;
  const int* brow;
  const int *src0, *src1;
  const uint8_t *loc0, *loc1;
  const uint8_t* perm;
  const int* cell2face;
  const int* face2cell;
  const float* S;    // [nCells][LL*LL]
  const float* S0;   // [nCells][LL]
  const double* rtrace;  // FP64 face residual added to the gathered S0
  float* val;        // scalar-CSR order
  float* rhs;        // [nFaces*NF]
};
cudaError_t launch_scatter32(const Scatter32Params& p, bool values, cudaStream_t s);

// sol += U dl + U0, flux += Q dl + Q0, trace += dl (FP32 corrections, FP64 state)
struct Correct32Params {
  int nCells, F, NF, LU, LQ, LL;
  int64_t nTrace;
  const int* cell2face;
  const uint8_t* perm;
  const float *U, *Q, *U0, *Q0;
  const float* dl;
  double* sol;
  double* flux;
  double* trace;
};
cudaError_t launch_correct32(const Correct32Params& p, cudaStream_t s);

// sum of squares of up to three FP64 vectors (deterministic partials, host sums)
cudaError_t launch_sumsq(const double* a, int64_t na, const double* b, int64_t nb, const double* c, int64_t nc,
                         double* partials, int grid, cudaStream_t s);

// FP32 solve of A' d = rhs on the raw FP32 trace values (Dirichlet elimination
// and sign flip applied on the fly): CG when symmetric, else GMRES. Returns an
// HFX status; iterations added to *its.
struct F32SolveArgs {
  int dim;
  TraceView A;
  const float* val;
  const float* rhs;
  float* x;
  int precond;
  int gmres;
  int restart;
  double rtol;
  int maxits;
  TraceWorkspace ws;
  cudaStream_t stream;
  KernelTimer* timer;
  bool rebuildPrecond;
};
int trace_solve_f32(const F32SolveArgs& a, int* its);
int trace_gmres_f32(const F32SolveArgs& a, int* its);

}  // namespace hfx
