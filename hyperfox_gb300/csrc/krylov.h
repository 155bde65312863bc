// Trace-system Krylov solver (internal interface).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

#include "coarse.h"
#include "timer.h"

namespace hfx {

// Face-block view of the trace system: rows = faces, block columns = sorted
// neighbour faces, values in scalar-CSR order (see hdg_trace.cu).
struct TraceView {
  int64_t nFaces;
  int NF;
  const int64_t* browptr;
  const int* bcol;
  const uint8_t* isBnd;  // Dirichlet (boundary) faces
  // Symmetric half storage of the FP32 operator (optional): for block k of row
  // f, hidx[k] >= 0 is the stored block (f, g >= f), column-major; hidx[k] < 0
  // means block (g, f) stored at -hidx[k]-1, read transposed.
  const int* hidx = nullptr;
  int64_t nHalf = 0;
  // the same rows as a fixed-width table (ELL): slot k of face f holds (bcol, hidx)
  // at ell[f * ellWidth + k], unused slots (0, INT_MIN); nullptr when not built
  const int2* ell = nullptr;
  int ellWidth = 0;
};

// Device-resident solver scalars. Reductions finish in the last block, which
// writes here; "done" makes every later kernel of the solve return at entry.
struct CgState {
  double rz, rr, bb, alpha, beta;
  double res_rr, res_bb;
  int iters, maxits, done, status;
  unsigned ticket;
  int pad;
};

struct TraceWorkspace {
  double *bS, *r, *z, *p0, *p1, *q, *pc64;
  float *val32, *pc32, *r32, *z32, *p032, *p132, *q32, *d32, *rhs32, *bS32;
  float* val32h;  // symmetric half storage of A' (FP32), nHalf blocks
  double* partials;
  CgState* state;
  // GMRES: Krylov bases (restart+1 vectors) and the small device vector of coefficients
  double* V64;
  float* V32;
  double* hdev;
};

struct TraceSolveArgs {
  int dim;
  TraceView A;
  const double* val;  // reference values (scalar-CSR order)
  const double* rhs;  // reference right-hand side
  double* x;          // solution (in: initial guess if use_initial_guess)
  int precond;        // 0 none, 1 Jacobi, 2 block Jacobi, 3 two-level (block Jacobi + vertex coarse space)
  int mixed;          // FP32 inner CG inside FP64 refinement
  double rtol, inner_rtol;
  int maxits, max_refinements, check_every, use_initial_guess;
  int restart;        // GMRES restart length
  TraceWorkspace ws;
  cudaStream_t stream;
  KernelTimer* timer;
  const CoarseSolver* coarse;  // set up for precond 3
  int coarse_guess;            // start from the prolongated coarse solution of b'
  // training samples of the learned coarse polynomial (FP64 two-level CG only):
  // every sampleStride-th coarse solve copies its restricted residual P^T r
  float* sampleBuf;            // [sampleCap][nV]
  int sampleCap, sampleStride;
  int* sampleCount;            // host counter
  int prepared;                // GMRES: b' and the preconditioner are already in ws (trace_prepare ran)
  // launch tuner of the FP32 half-storage operator (mixed CG): -1 not tuned yet, then the
  // kernel chosen (0 row per lane, 1 blocks staged by bulk copies, 2 row per lane with paired
  // loads of transposed blocks, 3 the same with float4 reads of the gathered x) and their
  // times (ms, four)
  int* spmvChoice;
  float* spmvTimes;
  // mixed CG: iterations of the first stretch of the last solve on this context (host; 0
  // unknown), used to size the first batch of queued iterations
  int* stretchHint;
};

struct TraceSolveResult {
  int iterations = 0, refinements = 0;
  double rel_residual = 0.0, bb = 0.0;
  cudaError_t cudaErr = cudaSuccess;
};

// Returns an HFX status code (0 = converged).
int trace_solve(const TraceSolveArgs& a, TraceSolveResult* out);   // CG (symmetric systems)
int trace_gmres(const TraceSolveArgs& a, TraceSolveResult* out);   // GMRES (any system)
// Least-squares initial guess for the eliminated system A' x = b' from K <= 8 earlier
// solutions X[i] (projection onto previous solutions for a sequence of systems): writes
// x0 = sum_i c_i X[i] into a.x with c minimising ||b' - A' sum_i c_i X[i]||_2; Y is
// K * n scratch. Needs trace_prepare(a) (b' in a.ws.bS). Returns the number of vectors
// kept (nearly dependent ones are dropped), 0 leaving a.x as it was.
int trace_projection_guess(const TraceSolveArgs& a, const double* const* X, int K, double* Y);
size_t trace_partials_needed();
// Shared pieces: b', the FP32 copy of A' (mixed) and the preconditioner; the
// reference-system residual into out->rel_residual.
void trace_prepare(const TraceSolveArgs& a);
// FP32 right-hand side b' of the eliminated system and (optionally) the FP32
// preconditioner, from raw FP32 trace values (mixed-precision corrections).
void trace_prepare_f32(int dim, const TraceView& A, const float* val, const float* rhs, float* bS, int pcType,
                       float* pc, cudaStream_t s);
void trace_ref_residual(const TraceSolveArgs& a, TraceSolveResult* out);

}  // namespace hfx
