// CG element operators (Mass, Diffusion, Convection), internal interface.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <vector>

namespace hfx {

struct CgOpParams {
  int64_t nCells;
  const double* coords;   // [nNodes][D]
  const int* cells;       // [nCells][N]
  const double* kappa;    // diffusion field: layout 0 [nNodes][kc], 1 [nCells][N][kc]; kc 0 = identity
  int kc, kappaLayout;
  const double* vel;      // velocity: layout 0 [nNodes][D], 1 [nCells][N][D]; may be null
  int velLayout;
  const double* tab;      // phi, dphi, w (the element kernels' packed FP64 table)
  const float* tctab;     // tc_cg_table() image (tensor-core path)
  int which;              // bit 0 mass, 1 diffusion, 2 convection
  double* out;            // [nCells][3][N*N], op(i, j) at j N + i
  int* status;            // 2 = a tensor-core wait ran out
};

cudaError_t launch_cg_operators_f64(int dim, int order, const CgOpParams& p, cudaStream_t s);
// the same operators contracted on the tensor cores (tc_assembly.cu)
std::vector<float> tc_cg_table(int dim, int order, const double* tab64);
cudaError_t launch_cg_operators_tc(int dim, int order, const CgOpParams& p, cudaStream_t s);

}  // namespace hfx
