// Two-level preconditioner for the condensed trace system: a coarse space of
// one degree of freedom per mesh vertex, prolongated to the trace nodes of the
// faces through per-node weights (by default the node's barycentric coordinates
// on its face, i.e. continuous piecewise-linear interpolation), with the
// Galerkin coarse operator A_c = P^T A' P assembled element by element from the
// condensed element matrices S_e, and a fixed-degree Chebyshev iteration on A_c
// as the coarse solve. The preconditioner applied in CG is
//     M^{-1} r = B^{-1} r + P q(A_c) P^T r
// with B the face-block Jacobi matrix and q(A_c) the Chebyshev polynomial
// approximation of A_c^{-1}; both terms are symmetric positive (semi)definite,
// so M^{-1} is a fixed SPD operator and plain PCG applies.
//
// The reference solves the trace system with PETSc GMRES + point Jacobi
// (src/resolution/PetscInterface.cpp:222-247, src/resolution/PetscOpts.h:12-28);
// the coarse space has no counterpart there.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <string>
#include <vector>

#include "hfx_host.h"

namespace hfx {

// Host-built structure (depends on the mesh only).
struct CoarseHost {
  int nV = 0;                     // coarse DOFs = distinct cell vertices
  int dim = 0, NF = 0, F = 0, LL = 0, NV1 = 0;
  std::vector<int> vertexNode;    // [nV] mesh node id of each coarse DOF
  std::vector<int> cellV;         // [nCells][NV1] coarse id of the cell's vertices
  std::vector<int> faceV;         // [nFaces][dim] coarse id of the face's vertices (face order)
  std::vector<int> rowptr, col;   // coarse CSR pattern (vertices sharing a cell)
  std::vector<int> cptr, cidx;    // per coarse non-zero: element contributions (cell*NV1^2 + m*NV1 + m2)
  std::vector<int> rptr, ridx;    // per vertex: incident (face*dim + k)
  int ellW = 0;
  std::vector<int> ellCol, ellSrc; // [ellW][nV]
  std::vector<float> Wf;          // [NF][dim] default face weights (barycentric)
  std::vector<float> Wc;          // [F*NF][NV1] cell-local weights (barycentric, element face-node order)
};
// cellVerts: [nCells][dim+1] mesh node ids of the cell vertices (nodes 0..dim).
bool build_coarse_host(const RefEl& re, int nCells, const int* cellVerts, const Topology& t, CoarseHost* out,
                       std::string* err);

// Reference-face barycentric table [NF][dim] and the cell-local table
// [F*NF][dim+1], both from the reference nodes (vertices are nodes 0..dim).
bool coarse_weight_tables(const RefEl& re, std::vector<double>* Wf, std::vector<double>* Wc, std::string* err);

// Device view.
struct CoarseDev {
  int nV, dim, NF, F, LL, NV1;
  int64_t nFaces, nCells, nnz;
  const int *rowptr, *col, *cptr, *cidx, *rptr, *ridx, *faceV, *cell2face;
  const uint8_t* isBnd;
  float *Wf, *Wc;       // [NF*dim], [LL*NV1] (device, current weights)
  float* Ce;            // [nCells][NV1*NV1]
  float *val, *dinv;    // coarse operator values, inverse diagonal (0 for inactive)
  int ellW;             // ELL copy of the coarse operator for the Chebyshev steps:
  const int* ellCol;    // [ellW][nV] column (padding: the row itself)
  float* ellVal;        // [ellW][nV] value (padding: 0)
  const int* ellSrc;    // [ellW][nV] position in the CSR values (-1: padding)
  float *rc, *yc, *cr, *cd0, *cd1, *lz;  // work vectors [nV]
  double* partials;     // reductions for the eigenvalue estimate
  float theta;          // Chebyshev centre (start: d0 = D^{-1} r / theta)
  unsigned* barrier;    // [2] grid barrier of the one-launch coarse solve: count, generation
  int* error;           // set when a grid barrier wait ran out (the solve is then invalid)
  int* testHold;        // test hook, one shot: block 0 withholds its first barrier arrival
  double* lanczosOut;   // [2*30+3] alpha, beta, step count, start norm and row-sum bound of the one-launch Lanczos
};

// Coarse solver state: device view plus the polynomial schedule. Both coarse
// solves run y = sum_k d_k with r_{k+1} = r_k - A_c d_k and
// d_{k+1} = c1[k] d_k + c2[k] D^{-1} r_{k+1}, d_0 = d0scale D^{-1} r_0:
//  - Chebyshev on [lmin, lmax] of D^{-1} A_c (the default), or
//  - the learned polynomial: Richardson steps with trained weights theta_k
//    (c1 = 0, c2[k] = theta_{k+1}, d0scale = theta_0), i.e. the residual
//    polynomial prod_k (1 - theta_k lambda) fitted to the coarse residuals the
//    solver itself produces (coarse_train).
struct CoarseSolver {
  CoarseDev dev{};
  bool ready = false;   // operator and schedule match the assembled system
  int coopGrid = 0;     // >0: blocks of the cooperative one-launch coarse solve
  int clusterGrid = 0;  // >0: CTAs of the one-cluster coarse solve (small coarse spaces)
  bool forceCoop = false;  // test hook: the cooperative solve even where one cluster would do
  int degree = 0;
  double lmin = 0.0, lmax = 0.0;
  // of D^{-1/2} A_c D^{-1/2}: extreme Ritz values of the Lanczos steps (inside the spectrum)
  // and the infinity norm (above the spectral radius)
  double ritzMin = 0.0, ritzMax = 0.0, rowBound = 0.0;
  std::vector<float> c1, c2;  // Chebyshev schedule
  // learned polynomial: weights scaled by lmax (theta_k = thetaHat_k / lmax), so
  // that a trained schedule carries over to a re-assembled operator
  std::vector<double> thetaHat;
  bool useLearned = false;    // apply the learned schedule (set per solve)
};

// Result of training the learned coarse polynomial.
struct CoarseTrainResult {
  int degree = 0, samples = 0, steps = 0, accepted = 0;
  double lossStart = 0.0, lossChebyshev = 0.0, lossLearned = 0.0, maxGain = 0.0, ms = 0.0;
  int lowerSteps = 0, rejectedSteps = 0;  // steps that lowered the loss / were refused by the polynomial check
  double lossFirstStep = 0.0;
};

// Fit theta (K weights) to the coarse residual samples [S][nV] (column-major:
// sample s contiguous) by Adam on log(theta * lmax), with the project's forward
// and backward kernels. Accepted only if prod_k (1 - theta_k lambda) <= 1 on
// [0, lmax] (the coarse solve then stays symmetric positive semidefinite)
// and the loss beats Chebyshev of the same degree. feasible: every step is shortened
// (halved, at most twelve times) until the residual polynomial stays <= 1, so the
// optimiser moves only through polynomials that could be accepted.
cudaError_t coarse_train(CoarseSolver* c, const float* samples, int S, int K, int steps, double lr, cudaStream_t s,
                         CoarseTrainResult* out, bool feasible = false);
// Loss and gradient of the learned polynomial for given theta (unscaled) on
// samples [S][nV]: the GPU kernels coarse_train uses (for gradient checks).
cudaError_t coarse_loss_grad(const CoarseSolver& c, const float* samples, int S, int K, const double* theta,
                             double* loss, double* grad, cudaStream_t s);

// Coarse operator from the condensed element matrices (T = double or float),
// its eigenvalue bounds and the Chebyshev schedule. Returns a CUDA error.
template <typename T>
cudaError_t coarse_setup(CoarseSolver* c, const T* S, int maxDegree, double target, cudaStream_t s);
// yc = q(A_c) P^T r, r on trace DOFs (interior rows only). Every kernel
// returns at entry when *skip != 0 (the Krylov solve has converged).
template <typename T>
cudaError_t coarse_apply(const CoarseSolver& c, const T* r, const int* skip, cudaStream_t s);
// x += P yc on interior trace rows (initial guess from the coarse solve).
template <typename T>
cudaError_t coarse_prolong_add(const CoarseSolver& c, T* x, cudaStream_t s);

}  // namespace hfx
