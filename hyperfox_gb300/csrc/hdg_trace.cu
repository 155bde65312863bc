// Trace-system scatter, local recovery and integration-point coordinates.
//
// Trace values are stored per face-block row (rows = faces, blocks = the
// sorted neighbour faces), block by block in CSR order, each Nf x Nf block
// column-major: entry (row node a, column node b) of block k at
// k*Nf*Nf + b*Nf + a. The scalar pattern is PETSc's AIJ pattern of the
// reference system (sorted columns, explicit zeros kept); the scalar column
// array is implied by the block columns and never stored, and hfx_get_csr
// reorders the values row-major for export.
#include "hfx_device.h"

namespace hfx {
namespace {

// One thread per stored value: sum of the (one or two) element contributions,
// first the lower cell then the upper one (the order HyperFox adds them in,
// HDGSolver.cpp:605-625). With at most two addends the sum is exact-order
// independent.
__global__ void scatter_values(ScatterParams p, const int* brow, int64_t nBlocks) {
  const int NF = p.NF, LL = p.LL, F = p.F;
  const int64_t total = nBlocks * NF * NF;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    int64_t k = idx / (NF * NF);
    int ab = (int)(idx % (NF * NF));
    int a = ab / NF, b = ab % NF;
    double v = 0.0;
    for (int s = 0; s < 2; ++s) {
      int c = s == 0 ? p.src0[k] : p.src1[k];
      if (c < 0) continue;
      int loc = s == 0 ? p.loc0[k] : p.loc1[k];
      int li = loc >> 4, lj = loc & 15;
      // local node positions whose face-order positions are a (row) and b (col)
      const uint8_t* pi = p.perm + ((int64_t)c * F + li) * NF;
      const uint8_t* pj = p.perm + ((int64_t)c * F + lj) * NF;
      int ja = 0, jb = 0;
      for (int q = 0; q < NF; ++q) {
        if (pi[q] == a) ja = q;
        if (pj[q] == b) jb = q;
      }
      v += p.S[(int64_t)c * LL * LL + (li * NF + ja) + (int64_t)(lj * NF + jb) * LL];
    }
    p.val[k * NF * NF + (int64_t)b * NF + a] = v;  // block k column-major
  }
}

// Same values, one warp per block: the warp inverts the (at most two) face
// permutations once into shared memory, then writes the block's NF*NF values
// with consecutive lanes on consecutive (column-major) positions.
constexpr int kScatterWarps = 8;
__global__ void __launch_bounds__(32 * kScatterWarps) scatter_values_w(ScatterParams p) {
  const int NF = p.NF, LL = p.LL, F = p.F;
  __shared__ uint8_t inv[kScatterWarps][2][2][16];  // [warp][contribution][row, col][face position]
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t nW = (int64_t)gridDim.x * kScatterWarps;
  for (int64_t k = (int64_t)blockIdx.x * kScatterWarps + warp; k < p.nBlocks; k += nW) {
    const int c0 = p.src0[k], c1 = p.src1[k];
    const int l0 = p.loc0[k], l1 = p.loc1[k];
    {
      const int sIdx = lane >> 4, q = lane & 15;
      const int c = sIdx == 0 ? c0 : c1;
      const int loc = sIdx == 0 ? l0 : l1;
      if (q < NF && c >= 0) {
        const int li = loc >> 4, lj = loc & 15;
        inv[warp][sIdx][0][p.perm[((int64_t)c * F + li) * NF + q]] = (uint8_t)q;
        inv[warp][sIdx][1][p.perm[((int64_t)c * F + lj) * NF + q]] = (uint8_t)q;
      }
    }
    __syncwarp();
    for (int idx = lane; idx < NF * NF; idx += 32) {
      const int a = idx % NF, b = idx / NF;
      double v = 0.0;
      if (c0 >= 0) {
        const int li = l0 >> 4, lj = l0 & 15;
        v += p.S[(int64_t)c0 * LL * LL + (li * NF + inv[warp][0][0][a]) + (int64_t)(lj * NF + inv[warp][0][1][b]) * LL];
      }
      if (c1 >= 0) {
        const int li = l1 >> 4, lj = l1 & 15;
        v += p.S[(int64_t)c1 * LL * LL + (li * NF + inv[warp][1][0][a]) + (int64_t)(lj * NF + inv[warp][1][1][b]) * LL];
      }
      p.val[k * NF * NF + idx] = v;  // block k column-major: (a, b) at b*NF + a
    }
    __syncwarp();
  }
}

__global__ void scatter_rhs(ScatterParams p) {
  const int NF = p.NF, LL = p.LL, F = p.F;
  const int64_t total = (int64_t)p.nFaces * NF;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    int f = (int)(idx / NF), a = (int)(idx % NF);
    double v = 0.0;
    for (int s = 0; s < 2; ++s) {
      int c = p.face2cell[2 * (int64_t)f + s];
      if (c < 0) continue;
      int li = 0;
      for (int i = 0; i < F; ++i)
        if (p.cell2face[(int64_t)c * F + i] == f) li = i;
      const uint8_t* pi = p.perm + ((int64_t)c * F + li) * NF;
      int ja = 0;
      for (int q = 0; q < NF; ++q)
        if (pi[q] == a) ja = q;
      v += p.S0[(int64_t)c * LL + li * NF + ja];
    }
    p.rhs[idx] = v;
  }
}

// SEXPLICIT trace (HDGSolver.cpp:709-729): every face solves its own block,
// trace_f = S_f^{-1} S0_f, S_f being the diagonal block of the assembled system
// (the explicit modes' system has no other block). One thread per face,
// Gauss-Jordan with partial pivoting; a zero pivot sets *status.
__global__ void face_block_solve(int nFaces, int NF, const int64_t* __restrict__ browptr, const int* __restrict__ bcol,
                                 const double* __restrict__ val, const double* __restrict__ rhs, double* __restrict__ x,
                                 int* status) {
  for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < nFaces; f += gridDim.x * blockDim.x) {
    int64_t kd = -1;
    for (int64_t k = browptr[f]; k < browptr[f + 1]; ++k)
      if (bcol[k] == f) kd = k;
    if (kd < 0) {
      atomicCAS(status, 0, 2);
      continue;
    }
    double B[10][11];
    for (int a = 0; a < NF; ++a) {
      for (int b = 0; b < NF; ++b) B[a][b] = val[kd * NF * NF + (int64_t)b * NF + a];
      B[a][NF] = rhs[(int64_t)f * NF + a];
    }
    bool ok = true;
    for (int k = 0; k < NF; ++k) {
      int pr = k;
      for (int i = k + 1; i < NF; ++i)
        if (fabs(B[i][k]) > fabs(B[pr][k])) pr = i;
      if (B[pr][k] == 0.0) {
        ok = false;
        break;
      }
      if (pr != k)
        for (int j = 0; j <= NF; ++j) {
          double t = B[k][j];
          B[k][j] = B[pr][j];
          B[pr][j] = t;
        }
      const double inv = 1.0 / B[k][k];
      for (int j = k; j <= NF; ++j) B[k][j] *= inv;
      for (int i = 0; i < NF; ++i) {
        if (i == k) continue;
        const double l = B[i][k];
        for (int j = k; j <= NF; ++j) B[i][j] -= l * B[k][j];
      }
    }
    if (!ok) {
      atomicCAS(status, 0, 1);
      continue;
    }
    for (int a = 0; a < NF; ++a) x[(int64_t)f * NF + a] = B[a][NF];
  }
}

__global__ void block_rows(const int64_t* browptr, int nFaces, int* brow) {
  for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < nFaces; f += gridDim.x * blockDim.x)
    for (int64_t k = browptr[f]; k < browptr[f + 1]; ++k) brow[k] = f;
}

// One CTA per element: thread r computes row r of [U; Q] * lambda + [U0; Q0]
// (HDGSolver.cpp:741-775). Columns of U and Q are contiguous per element, so
// consecutive threads read consecutive addresses.
__global__ void recover_kernel(RecoverParams p) {
  extern __shared__ double lam[];
  const int F = p.F, NF = p.NF, LU = p.LU, LQ = p.LQ, LL = p.LL;
  for (int64_t e = blockIdx.x; e < p.nCells; e += gridDim.x) {
    for (int j = threadIdx.x; j < LL; j += blockDim.x) {
      int i = j / NF;
      int f = p.cell2face[e * F + i];
      lam[j] = p.trace[(int64_t)f * NF + p.perm[(e * F + i) * NF + (j % NF)]];
    }
    __syncthreads();
    for (int r = threadIdx.x; r < LU + LQ; r += blockDim.x) {
      double acc;
      if (r < LU) {
        const double* U = p.U + e * LU * LL;
        acc = p.U0[e * LU + r];
        for (int c = 0; c < LL; ++c) acc += U[r + (int64_t)c * LU] * lam[c];
        p.sol[e * LU + r] = acc;
      } else {
        int rq = r - LU;
        const double* Q = p.Q + e * LQ * LL;
        acc = p.Q0[e * LQ + rq];
        for (int c = 0; c < LL; ++c) acc += Q[rq + (int64_t)c * LQ] * lam[c];
        p.flux[e * LQ + rq] = acc;
      }
    }
    __syncthreads();
  }
}

__global__ void ip_coords_kernel(IpCoordParams p) {
  const int64_t total = (int64_t)p.nCells * p.NI * p.D;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    int64_t c = idx / (p.NI * p.D);
    int q = (int)((idx / p.D) % p.NI), d = (int)(idx % p.D);
    double acc = 0.0;
    for (int i = 0; i < p.N; ++i) acc += p.phi[q * p.N + i] * p.coords[(int64_t)p.cells[c * p.N + i] * p.D + d];
    p.out[idx] = acc;
  }
}

unsigned grid_for(int64_t n, int threads) {
  int64_t g = (n + threads - 1) / threads;
  if (g > 152 * 64) g = 152 * 64;
  return (unsigned)(g < 1 ? 1 : g);
}

}  // namespace

cudaError_t launch_block_rows(const int64_t* browptr, int nFaces, int* brow, cudaStream_t s) {
  block_rows<<<grid_for(nFaces, 256), 256, 0, s>>>(browptr, nFaces, brow);
  return cudaGetLastError();
}

cudaError_t launch_face_block_solve(int nFaces, int NF, const int64_t* browptr, const int* bcol, const double* val,
                                   const double* rhs, double* x, int* status, cudaStream_t s) {
  if (NF > 10) return cudaErrorInvalidValue;
  face_block_solve<<<grid_for(nFaces, 128), 128, 0, s>>>(nFaces, NF, browptr, bcol, val, rhs, x, status);
  return cudaGetLastError();
}

cudaError_t launch_scatter(const ScatterParams& p, cudaStream_t s) {
  if (p.NF <= 16) {
    int64_t g = (p.nBlocks + kScatterWarps - 1) / kScatterWarps;
    if (g > 152 * 64) g = 152 * 64;
    scatter_values_w<<<(unsigned)(g < 1 ? 1 : g), 32 * kScatterWarps, 0, s>>>(p);
  } else {
    scatter_values<<<grid_for(p.nBlocks * p.NF * p.NF, 256), 256, 0, s>>>(p, p.brow, p.nBlocks);
  }
  scatter_rhs<<<grid_for((int64_t)p.nFaces * p.NF, 256), 256, 0, s>>>(p);
  return cudaGetLastError();
}

cudaError_t launch_recover(const RecoverParams& p, cudaStream_t s) {
  int threads = ((p.LU + p.LQ + 31) / 32) * 32;
  if (threads > 256) threads = 256;
  int64_t grid = p.nCells < 152 * 256 ? p.nCells : 152 * 256;
  recover_kernel<<<(unsigned)(grid < 1 ? 1 : grid), threads, p.LL * sizeof(double), s>>>(p);
  return cudaGetLastError();
}

cudaError_t launch_ip_coords(const IpCoordParams& p, cudaStream_t s) {
  ip_coords_kernel<<<grid_for((int64_t)p.nCells * p.NI * p.D, 256), 256, 0, s>>>(p);
  return cudaGetLastError();
}

}  // namespace hfx
