// FP32 scatter, FP32 corrections into the FP64 state, and norms, for the
// mixed-precision solve (see hdg_mixed.h).
#include "hdg_mixed.h"

namespace hfx {
namespace {

unsigned grid_for(int64_t n, int threads) {
  int64_t g = (n + threads - 1) / threads;
  if (g > 152 * 64) g = 152 * 64;
  return (unsigned)(g < 1 ? 1 : g);
}

// FP32 copy of the trace-system scatter (same order as hdg_trace.cu)
__global__ void scatter32_values(Scatter32Params p) {
  const int NF = p.NF, LL = p.LL, F = p.F;
  const int64_t total = p.nBlocks * NF * NF;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    int64_t k = idx / (NF * NF);
    int ab = (int)(idx % (NF * NF));
    int a = ab / NF, b = ab % NF;
    float v = 0.f;
    for (int s = 0; s < 2; ++s) {
      int c = s == 0 ? p.src0[k] : p.src1[k];
      if (c < 0) continue;
      int loc = s == 0 ? p.loc0[k] : p.loc1[k];
      int li = loc >> 4, lj = loc & 15;
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

// rhs = gathered element S0 (correction part) + FP64 face residual
__global__ void scatter32_rhs(Scatter32Params p) {
  const int NF = p.NF, LL = p.LL, F = p.F;
  const int64_t total = (int64_t)p.nFaces * NF;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    int f = (int)(idx / NF), a = (int)(idx % NF);
    double v = p.rtrace[idx];
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
      v += (double)p.S0[(int64_t)c * LL + li * NF + ja];
    }
    p.rhs[idx] = (float)v;
  }
}

// one CTA per element: rows of [U; Q] * dl + [U0; Q0], added to the FP64 state
__global__ void correct32_kernel(Correct32Params p) {
  extern __shared__ float lam[];
  const int F = p.F, NF = p.NF, LU = p.LU, LQ = p.LQ, LL = p.LL;
  for (int64_t e = blockIdx.x; e < p.nCells; e += gridDim.x) {
    for (int j = threadIdx.x; j < LL; j += blockDim.x) {
      int i = j / NF;
      int f = p.cell2face[e * F + i];
      lam[j] = p.dl[(int64_t)f * NF + p.perm[(e * F + i) * NF + (j % NF)]];
    }
    __syncthreads();
    for (int r = threadIdx.x; r < LU + LQ; r += blockDim.x) {
      float acc;
      if (r < LU) {
        const float* U = p.U + e * LU * LL;
        acc = p.U0[e * LU + r];
        for (int c = 0; c < LL; ++c) acc = fmaf(U[r + (int64_t)c * LU], lam[c], acc);
        p.sol[e * LU + r] += (double)acc;
      } else {
        int rq = r - LU;
        const float* Q = p.Q + e * LQ * LL;
        acc = p.Q0[e * LQ + rq];
        for (int c = 0; c < LL; ++c) acc = fmaf(Q[rq + (int64_t)c * LQ], lam[c], acc);
        p.flux[e * LQ + rq] += (double)acc;
      }
    }
    __syncthreads();
  }
}

__global__ void trace_add(int64_t n, const float* __restrict__ d, double* __restrict__ x) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    x[i] += (double)d[i];
}

__global__ void sumsq_kernel(const double* a, int64_t na, const double* b, int64_t nb, const double* c, int64_t nc,
                             double* partials) {
  __shared__ double red[32];
  double acc = 0.0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < na; i += stride) acc += a[i] * a[i];
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nb; i += stride) acc += b[i] * b[i];
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nc; i += stride) acc += c[i] * c[i];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
    partials[blockIdx.x] = s;
  }
}

}  // namespace

cudaError_t launch_scatter32(const Scatter32Params& p, bool values, cudaStream_t s) {
  if (values) scatter32_values<<<grid_for(p.nBlocks * p.NF * p.NF, 256), 256, 0, s>>>(p);
  scatter32_rhs<<<grid_for((int64_t)p.nFaces * p.NF, 256), 256, 0, s>>>(p);
  return cudaGetLastError();
}

cudaError_t launch_correct32(const Correct32Params& p, cudaStream_t s) {
  int threads = ((p.LU + p.LQ + 31) / 32) * 32;
  if (threads > 256) threads = 256;
  int64_t grid = p.nCells < 152 * 256 ? p.nCells : 152 * 256;
  correct32_kernel<<<(unsigned)(grid < 1 ? 1 : grid), threads, p.LL * sizeof(float), s>>>(p);
  trace_add<<<grid_for(p.nTrace, 256), 256, 0, s>>>(p.nTrace, p.dl, p.trace);
  return cudaGetLastError();
}

cudaError_t launch_sumsq(const double* a, int64_t na, const double* b, int64_t nb, const double* c, int64_t nc,
                         double* partials, int grid, cudaStream_t s) {
  sumsq_kernel<<<grid, 256, 0, s>>>(a, na, b, nb, c, nc, partials);
  return cudaGetLastError();
}

}  // namespace hfx
