// Runge-Kutta field updates (RungeKutta.cpp:90-213) as one device kernel:
// out = alpha a + sum_j coef_j k_j over a field's values, for the stage vector
// of apply() (w = (dt - c) ut + dt^2 sum_{i<s} a_si k_i), the stage derivative
// and update of computeStage() and the final combination of computeSolution().
// Bandwidth-bound and tiny next to the assembly: grid-stride, coalesced.
#include <cuda_runtime.h>

#include "hfx_device.h"

namespace hfx {
namespace {

__global__ void rk_lincomb(int64_t n, double* out, double alpha, const double* a, RkTerms terms) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double v = alpha * a[i];
    for (int j = 0; j < terms.n; ++j) v += terms.coef[j] * terms.ptr[j][i];
    out[i] = v;
  }
}

}  // namespace

cudaError_t launch_rk_lincomb(int64_t n, double* out, double alpha, const double* a, const RkTerms& terms,
                              cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  if (terms.n < 0 || terms.n > RkTerms::MAX) return cudaErrorInvalidValue;
  int64_t grid = (n + 255) / 256;
  if (grid > 152 * 16) grid = 152 * 16;
  rk_lincomb<<<(unsigned)grid, 256, 0, s>>>(n, out, alpha, a, terms);
  return cudaGetLastError();
}

}  // namespace hfx
