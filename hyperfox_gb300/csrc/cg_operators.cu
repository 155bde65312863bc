// CG element operators in FP64 on the CUDA cores, element by element.
//
// Restates HyperFox's continuous-Galerkin operators with one DOF per node:
//   Mass       M(i,j) = sum_q dV phi_i phi_j                          Mass.cpp:5-38
//   Diffusion  D(i,j) = sum_q dV (K grad phi_i)^T grad phi_j          Diffusion.cpp:5-43
//              K the nodal diffusion field at the IP (setDiffTensor, Diffusion.cpp:59-69:
//              scalar times the identity, or a d x d tensor; none: identity)
//   Convection C(k,l) = sum_q dV phi_k (v . grad phi_l)               Convection.cpp:21-46
//              v the nodal velocity at the IP (setVelocity, Convection.cpp:5-19)
// with grad phi = J^{-1} grad_ref phi and dV = w |J| (Operator.cpp:14-84).
//
// One CTA per element (grid-stride): the threads evaluate the geometry per IP and
// the physical gradients into shared memory, then one thread per (i, j) entry
// sums over the IPs and writes the three operators column-major (coalesced).
#include "cg_operators.h"
#include "hfx_device.h"

namespace hfx {
namespace {

template <int D, int P>
struct CgDims {
  using K = Dims<D, P>;
  static constexpr int N = K::N, NI = K::NI;
  static constexpr int THREADS = N * N <= 128 ? 128 : 256;
};

template <int D, int P>
__global__ void __launch_bounds__(CgDims<D, P>::THREADS) cg_operators_f64(CgOpParams p) {
  using C = CgDims<D, P>;
  constexpr int N = C::N, NI = C::NI, NT = C::THREADS;
  __shared__ double phi[NI * N], dphi[NI * N * D], w[NI];
  __shared__ double X[N * D], dV[NI], Kq[NI * D * D], vq[NI * D];
  __shared__ double G[NI * N * D];  // physical gradients [q][i][a]
  __shared__ double iJ[NI * D * D];
  for (int i = threadIdx.x; i < NI * N; i += NT) phi[i] = p.tab[i];
  for (int i = threadIdx.x; i < NI * N * D; i += NT) dphi[i] = p.tab[NI * N + i];
  for (int i = threadIdx.x; i < NI; i += NT) w[i] = p.tab[NI * N + NI * N * D + i];
  __syncthreads();
  for (int64_t e = blockIdx.x; e < p.nCells; e += gridDim.x) {
    const int* cell = p.cells + e * N;
    for (int i = threadIdx.x; i < N * D; i += NT) X[i] = p.coords[(int64_t)cell[i / D] * D + (i % D)];
    __syncthreads();
    for (int q = threadIdx.x; q < NI; q += NT) {
      double J[D][D];
      for (int r = 0; r < D; ++r)
        for (int s = 0; s < D; ++s) {
          double acc = 0.0;
          for (int i = 0; i < N; ++i) acc += dphi[(q * N + i) * D + r] * X[i * D + s];
          J[r][s] = acc;
        }
      double det, iv[D][D];
      if (D == 2) {
        det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
        const double id = 1.0 / det;
        iv[0][0] = J[1][1] * id;
        iv[0][1] = -J[0][1] * id;
        iv[1][0] = -J[1][0] * id;
        iv[1][1] = J[0][0] * id;
      } else {
        const double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
        const double c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
        const double c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
        det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
        const double id = 1.0 / det;
        iv[0][0] = c00 * id;
        iv[1][0] = c01 * id;
        iv[2][0] = c02 * id;
        iv[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * id;
        iv[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * id;
        iv[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * id;
        iv[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * id;
        iv[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * id;
        iv[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * id;
      }
      dV[q] = w[q] * det;
      for (int a = 0; a < D; ++a)
        for (int b = 0; b < D; ++b) iJ[(q * D + a) * D + b] = iv[a][b];
      // diffusion field at the IP (column-major d x d), identity when none is set
      for (int a = 0; a < D; ++a)
        for (int b = 0; b < D; ++b) {
          double acc = (p.kc == 0 && a == b) ? 1.0 : 0.0;
          if (p.kc > 0)
            for (int j = 0; j < N; ++j) {
              const int64_t bk = p.kappaLayout == 0 ? (int64_t)cell[j] * p.kc : (e * N + j) * p.kc;
              const double kv = p.kc == 1 ? (a == b ? p.kappa[bk] : 0.0) : p.kappa[bk + a + b * D];
              acc += phi[q * N + j] * kv;
            }
          Kq[(q * D + a) * D + b] = acc;
        }
      for (int a = 0; a < D; ++a) {
        double acc = 0.0;
        if (p.vel)
          for (int j = 0; j < N; ++j) {
            const int64_t bv = p.velLayout == 0 ? (int64_t)cell[j] * D : (e * N + j) * D;
            acc += phi[q * N + j] * p.vel[bv + a];
          }
        vq[q * D + a] = acc;
      }
    }
    __syncthreads();
    for (int qi = threadIdx.x; qi < NI * N; qi += NT) {
      const int q = qi / N, i = qi % N;
      for (int a = 0; a < D; ++a) {
        double acc = 0.0;
        for (int r = 0; r < D; ++r) acc += iJ[(q * D + a) * D + r] * dphi[(q * N + i) * D + r];
        G[qi * D + a] = acc;
      }
    }
    __syncthreads();
    double* out = p.out + e * 3 * N * N;
    for (int ji = threadIdx.x; ji < N * N; ji += NT) {
      const int j = ji / N, i = ji % N;  // column-major: entry (i, j) at j N + i
      double m = 0.0, dd = 0.0, cc = 0.0;
      for (int q = 0; q < NI; ++q) {
        const double* gi = G + (q * N + i) * D;
        const double* gj = G + (q * N + j) * D;
        m += phi[q * N + i] * phi[q * N + j] * dV[q];
        double v = 0.0;
        for (int a = 0; a < D; ++a) {
          double kg = 0.0;
          for (int b = 0; b < D; ++b) kg += Kq[(q * D + a) * D + b] * gi[b];
          v += kg * gj[a];
        }
        dd += v * dV[q];
        double vg = 0.0;
        for (int a = 0; a < D; ++a) vg += vq[q * D + a] * gj[a];
        cc += dV[q] * phi[q * N + i] * vg;
      }
      if (p.which & 1) out[ji] = m;
      if (p.which & 2) out[N * N + ji] = dd;
      if (p.which & 4) out[2 * N * N + ji] = cc;
    }
    __syncthreads();
  }
}

template <int D, int P>
cudaError_t launch_t(const CgOpParams& p, cudaStream_t s) {
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  int64_t grid = (int64_t)nsm * 8;
  if (grid > p.nCells) grid = p.nCells;
  if (grid < 1) grid = 1;
  cg_operators_f64<D, P><<<(unsigned)grid, CgDims<D, P>::THREADS, 0, s>>>(p);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_cg_operators_f64(int dim, int order, const CgOpParams& p, cudaStream_t s) {
  if (dim == 2) {
    switch (order) {
      case 1: return launch_t<2, 1>(p, s);
      case 2: return launch_t<2, 2>(p, s);
      case 3: return launch_t<2, 3>(p, s);
      case 4: return launch_t<2, 4>(p, s);
      case 5: return launch_t<2, 5>(p, s);
    }
  } else if (dim == 3) {
    switch (order) {
      case 1: return launch_t<3, 1>(p, s);
      case 2: return launch_t<3, 2>(p, s);
      case 3: return launch_t<3, 3>(p, s);
    }
  }
  return cudaErrorInvalidValue;
}

}  // namespace hfx
