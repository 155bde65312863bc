// Device-side parameter blocks and launcher declarations (internal).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

namespace hfx {

// Compile-time sizes of a simplex HDG element of dimension D and order P.
__host__ __device__ constexpr int simplex_nodes(int D, int P) {
  return D == 1 ? P + 1 : (D == 2 ? (P + 1) * (P + 2) / 2 : (P + 1) * (P + 2) * (P + 3) / 6);
}
// Number of points of the order-2P rule HyperFox uses (TestCubature.cpp:41-44).
__host__ __device__ constexpr int cubature_points(int D, int P) {
  return D == 1 ? P + 1
                : (D == 2 ? (P == 1 ? 3 : P == 2 ? 6 : P == 3 ? 12 : P == 4 ? 16 : 25)
                          : (P == 1 ? 4 : P == 2 ? 14 : P == 3 ? 24 : P == 4 ? 46 : 81));
}

template <int D, int P>
struct Dims {
  static constexpr int N = simplex_nodes(D, P);
  static constexpr int NF = simplex_nodes(D - 1, P);
  static constexpr int F = D + 1;
  static constexpr int NI = cubature_points(D, P);
  static constexpr int NIF = cubature_points(D - 1, P);
  static constexpr int LU = N;
  static constexpr int LQ = D * N;
  static constexpr int LL = F * NF;
};

// Everything the element kernel reads and writes (device pointers).
struct LocalParams {
  int nCells;
  const double* coords;        // [nNodes][D]
  const int* cells;            // [nCells][N]
  const int* cell2face;        // [nCells][F]
  const uint8_t* perm;         // [nCells][F][NF]
  const int* face2cell;        // [nFaces][2]
  const uint8_t* isBoundary;   // [nFaces]
  const double* tau;           // [nFaces][NF][tauVals]
  int tauVals;
  const double* kappa;         // layout 0: [nNodes][kc], 1: [nCells][N][kc]
  int kc, kappaLayout;
  int srcMode;
  const double* src;           // [nCells][NI]
  double srcParam;
  const double* dirichlet;     // [nFaces][NF]
  double dt;
  const double* uOld;          // [nCells][N]
  const double* tab;           // phi, dphi, w, fphi, fdphi, fw (padded to whole 16-byte units)
  const float* tab32;          // the same table in FP32 (the FP32 element kernel's bulk copy)
  const int* itab;             // faceNodes[F*NF], faceOpposite[F]
  void *S, *S0, *U, *Q, *U0, *Q0;  // double (fp32 == 0) or float (fp32 == 1)
  int* status;                 // first error: 1 = singular block
  int fp32;                    // element arithmetic in FP32 (mixed-precision path)
  // Residual mode (mixed-precision corrections): when rhsU is set, the element
  // right-hand side is (rhsU, rhsQ) = the FP64 residual rows instead of the
  // source, S0 gets no Dirichlet values, and U0/Q0 are the corrections' local parts.
  const double* rhsU;          // [nCells][N]
  const double* rhsQ;          // [nCells][N*D]
  int writeOps;                // write S, U, Q (else only S0, U0, Q0)
  // HDGSolverType (HDGSolverOpts.h:6-10) 1 WEXPLICIT / 2 SEXPLICIT: S = Sll and
  // S0 = -Slu sol - Slq flux from the current state (HDGSolver.cpp:349-354)
  int explicitMode;
  const double* solState;      // [nCells][N]
  const double* fluxState;     // [nCells][N*D] node-major
  // RungeKutta stage (RungeKutta.cpp:90-129) on the U rows of the local system:
  // K' = cStiff K + [M 0 0], f' = dt f + M uOld - K w with the stage vector
  // w = (dt - cStiff) ut + dt^2 sum_{i<s} a_si k_i, cStiff = dt a_ss; w given as its
  // cell parts and its face part (trace numbering). rkWu == nullptr: no stage.
  double cStiff;
  const double* rkWu;          // [nCells][N]
  const double* rkWq;          // [nCells][N*D] node-major
  const double* rkWl;          // [nFaces][NF]
  // FP32 path only: the element blocks (C_d, K_d, M, T, E_d, H_d, f_u) from the tensor-core
  // contraction kernel (tc_assembly.cu), [nCells][tcStride]; when set, the element kernel
  // loads them instead of integrating over the element (no Runge-Kutta stage, no explicit mode)
  const float* tcBlocks;
  int64_t tcStride;
};

cudaError_t launch_local_condense(int dim, int order, const LocalParams& p, cudaStream_t s);

// Vector Burgers element kernel (hdg_burgers.cu): nd = dim unknowns per node.
struct BurgersParams {
  int nCells;
  const double* coords;        // [nNodes][D]
  const int* cells;            // [nCells][N]
  const int* cell2face;        // [nCells][F]
  const uint8_t* perm;         // [nCells][F][NF] face2CellMap (node level)
  const int* face2cell;        // [nFaces][2]
  const uint8_t* isBoundary;   // [nFaces]
  const double* tau;           // [nFaces][NF][tauSides][ND*ND], ND x ND column-major
  int tauSides;                // 1 or 2 (double valued)
  const double* nu;            // diffusion tensor: layout 0 [nNodes][kc], 1 [nCells][N][kc]
  int kc, nuLayout;            // kc 0 = no diffusion operator, 1 scalar, D*D tensor
  const double* src;           // [nCells][NI][ND] source at the IPs, or nullptr
  const double* dirichlet;     // [nFaces][NF*ND] face order
  double dt;                   // > 0: implicit Euler about uOld
  const double* uOld;          // [nCells][N*ND]
  const double* buf;           // BufferSolution [nCells][N*ND] (linearisation point)
  const double* trace;         // Trace [nFaces][NF*ND]
  const double* tab;           // phi, dphi, w, fphi, fdphi, fw
  const int* itab;             // faceNodes[F*NF], faceOpposite[F]
  double *S, *S0, *U, *U0;     // Q, Q0 are not stored: launch_burgers_q forms them on demand
  int* status;                 // 1 = singular Schur block
  // per-element cache of the state-independent blocks ([nCells][burgers_cache_doubles]):
  // cacheMode 0 compute only, 1 compute and store, 2 load (geometry, tau, diffusion unchanged)
  double* cache;
  int cacheMode;
};
bool burgers_supported(int dim, int order);
size_t burgers_cache_doubles(int dim, int order);
size_t burgers_smem_bytes(int dim, int order);
cudaError_t launch_burgers_local(int dim, int order, const BurgersParams& p, cudaStream_t s);
// Solution = U lambda + U0 and Flux from the cache (M^-1 C, M^-1 E) of the last assembly
struct BurgersRecoverParams {
  int64_t nCells;
  const int* cell2face;        // [nCells][F]
  const uint8_t* permx;        // [nCells][F][NF*ND]
  const double *U, *U0;        // element blocks of the last assembly
  const double* cache;         // [nCells][burgers_cache_doubles]
  const double* trace;         // [nFaces][NF*ND]
  double* sol;                 // [nCells][N*ND]
  double* flux;                // [nCells][D*N*ND]
};
cudaError_t launch_burgers_recover(int dim, int order, const BurgersRecoverParams& p, cudaStream_t s);
// Q [nCells][NQ*NL] and Q0 [nCells][NQ] (column-major) from U, U0 and the cache
cudaError_t launch_burgers_q(int dim, int order, int64_t nCells, const double* U, const double* U0,
                             const double* cache, double* Q, double* Q0, cudaStream_t s);
// NonLinearWrapper pieces: out[0] = sum (sol - buf)^2, out[1] = sum buf^2 (deterministic
// block order); then both fields <- (1 - damp) sol + damp buf
size_t newton_partials_needed();
cudaError_t launch_newton_residual(int64_t n, const double* sol, const double* buf, double* partials,
                                   unsigned* ticket, double* out, cudaStream_t s);
cudaError_t launch_newton_update(int64_t n, double damp, double* sol, double* buf, cudaStream_t s);

// out[i] = alpha a[i] + sum_j coef[j] ptr[j][i] (rk.cu), element by element (out may alias an input)
struct RkTerms {
  static constexpr int MAX = 8;
  int n;
  double coef[MAX];
  const double* ptr[MAX];
};
cudaError_t launch_rk_lincomb(int64_t n, double* out, double alpha, const double* a, const RkTerms& terms,
                              cudaStream_t s);
bool local_condense_supported(int dim, int order);

// Affine elements with a symmetric, cell-constant diffusion tensor (hdg_affine.cu):
// S, S0, U, U0 from reference operators; geo[nCells][D*D + F*D] holds the
// factors the recovery (and the Q export) needs. atab from affine_tables().
cudaError_t launch_local_affine(int dim, int order, const LocalParams& p, const double* atab, double* geo,
                                double* prep, cudaStream_t s);
// doubles per element of the affine per-element record (geometry, coefficients, source)
int64_t affine_prep_doubles(int dim, int order);

// Trace-system scatter (face-block rows, values in scalar-CSR order).
struct ScatterParams {
  int nFaces, NF, LL;
  const int64_t* browptr;  // [nFaces+1]
  const int* brow;         // [nBlocks] row face of every block
  int64_t nBlocks;
  const int* src0;         // [nBlocks]
  const int* src1;
  const uint8_t* loc0;
  const uint8_t* loc1;
  const uint8_t* perm;     // [nCells][F][NF]
  const double* S;         // [nCells][LL*LL] column-major
  const double* S0;        // [nCells][LL]
  const int* cell2face;
  const int* face2cell;
  int F;
  double* val;             // scalar-CSR ordered values
  double* rhs;             // [nFaces*NF]
};
cudaError_t launch_scatter(const ScatterParams& p, cudaStream_t s);
cudaError_t launch_block_rows(const int64_t* browptr, int nFaces, int* brow, cudaStream_t s);
// trace_f = S_f^{-1} S0_f with S_f the diagonal face block (SEXPLICIT); status 1: singular block
cudaError_t launch_face_block_solve(int nFaces, int NF, const int64_t* browptr, const int* bcol, const double* val,
                                   const double* rhs, double* x, int* status, cudaStream_t s);

struct RecoverParams {
  int nCells, F, NF, LU, LQ, LL;
  const int* cell2face;
  const uint8_t* perm;
  const double *U, *Q, *U0, *Q0;
  const double* trace;
  double* sol;
  double* flux;
};
cudaError_t launch_recover(const RecoverParams& p, cudaStream_t s);
cudaError_t launch_recover_affine(int dim, int order, const RecoverParams& p, const double* atab, const double* geo,
                                  cudaStream_t s);
cudaError_t launch_q_from_u(int dim, int order, int nCells, const double* U, const double* U0, const double* atab,
                            const double* geo, double* Q, double* Q0, cudaStream_t s);

struct IpCoordParams {
  int nCells, N, NI, D;
  const double* coords;
  const int* cells;
  const double* phi;  // [NI][N]
  double* out;        // [nCells][NI][D]
};
cudaError_t launch_ip_coords(const IpCoordParams& p, cudaStream_t s);

}  // namespace hfx
