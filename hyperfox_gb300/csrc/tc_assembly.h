// Tensor-core element contractions (tc_assembly.cu), internal interface.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <vector>

namespace hfx {

struct TcBlockParams {
  int64_t nCells;
  const double* coords;       // [nNodes][D]
  const int* cells;           // [nCells][N]
  const int* cell2face;       // [nCells][F]
  const uint8_t* perm;        // [nCells][F][NF]
  const int* face2cell;       // [nFaces][2]
  const double* tau;          // [nFaces][NF][tauVals]
  int tauVals;
  const double* kappa;        // layout 0: [nNodes][kc], 1: [nCells][N][kc]; kc 0 = identity
  int kc, kappaLayout;
  int srcMode;                // 0 none, 1 values at the IPs, 2 srcParam * prod sin(pi x)
  const double* src;          // [nCells][NI]
  double srcParam;
  const int* itab;            // faceNodes[F*NF], faceOpposite[F]
  const float* tctab;         // tc_table() image (16-byte aligned)
  float* out;                 // [nCells][tc_blocks_stride]
  int* status;                // 2 = a tensor-core wait ran out
};

bool tc_blocks_supported(int dim, int order);
// floats per element of the output: volume rows (C_d, K_d, M) x N, face rows (T, E_d, H_d) x NF, f_u
int64_t tc_blocks_stride(int dim, int order);
// the packed FP32 table (TF32 hi/lo B images + basis tables) from the FP64 reference tables
// (phi, dphi, w, fphi, fdphi, fw as the element kernels take them)
std::vector<float> tc_table(int dim, int order, const double* tab64);
cudaError_t launch_tc_blocks(int dim, int order, const TcBlockParams& p, cudaStream_t s);

}  // namespace hfx
