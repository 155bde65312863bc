// Restarted GMRES on the trace system (PETSc's KSPGMRES default,
// PetscOpts.h:12), for trace systems that are not symmetric: HyperFox weights
// only the Suq/Slq blocks by the diffusion tensor, so a tensor that varies
// inside a cell makes the condensed system non-symmetric.
//
// Right preconditioning by the per-face block Jacobi inverse keeps the tested
// residual the true ||b' - A' x||, which equals the reference system's
// ||b - A x|| (see krylov.cu). Classical Gram-Schmidt applied twice; the
// partial dot products are per-block sums added on the host in block order
// (deterministic). Mixed precision: FP32 GMRES on the FP32 copy of A' inside
// FP64 iterative refinement.
#include <algorithm>
#include <cmath>
#include <vector>

#include "hdg_mixed.h"
#include "krylov.h"

namespace hfx {
namespace {

constexpr int kT = 256;

template <int NF, int NBMAX>
struct Cfg {
  static constexpr int FPW = 32 / NF;
  static constexpr int NPOS = NBMAX * NF;
};

// out = A' in ; MASKED applies the reference values with the Dirichlet
// elimination and the sign flip on the fly, else val holds A'. Thread per row,
// blocks column-major (same layout and mapping as the CG kernel).
template <typename T, int NF, int NBMAX, bool MASKED>
__global__ void __launch_bounds__(kT) op_apply(TraceView A, const T* __restrict__ val, const T* __restrict__ in,
                                               T* __restrict__ out) {
  constexpr int FPW = Cfg<NF, NBMAX>::FPW;
  __shared__ T xsh[kT / 32][FPW][Cfg<NF, NBMAX>::NPOS];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int slot = lane / NF, a = lane % NF;
  const bool laneUsed = slot < FPW;
  const int64_t stride = (int64_t)gridDim.x * (kT / 32) * FPW;
  for (int64_t fb = ((int64_t)blockIdx.x * (kT / 32) + warp) * FPW; fb < A.nFaces; fb += stride) {
    const int64_t f = fb + slot;
    const bool act = laneUsed && f < A.nFaces;
    const int64_t b0 = act ? A.browptr[f] : 0;
    const int nb = act ? (int)(A.browptr[f + 1] - b0) : 0;
    const bool rowBnd = MASKED && act && A.isBnd[f];
    T* xs = laneUsed ? xsh[warp][slot] : nullptr;
    if (act)
      for (int k = 0; k < nb; ++k) {
        int g = A.bcol[b0 + k];
        T v = in[(int64_t)g * NF + a];
        if (MASKED && (rowBnd || A.isBnd[g])) v = T(0);
        xs[k * NF + a] = v;
      }
    __syncwarp();
    if (act) {
      const T* base = val + b0 * NF * NF + a;
      T acc = T(0);
      for (int k = 0; k < nb; ++k) {
        const T* blk = base + (int64_t)k * NF * NF;
#pragma unroll
        for (int b = 0; b < NF; ++b) acc += __ldg(blk + b * NF) * xs[k * NF + b];
      }
      int64_t i = f * NF + a;
      out[i] = MASKED ? (rowBnd ? in[i] : -acc) : acc;
    }
    __syncwarp();
  }
}

// out = M^{-1} in, per face (PC: 0 none, 1 Jacobi, 2 block Jacobi)
// out = M^{-1} in, one thread per trace value (face f, row a): consecutive threads read
// consecutive entries of the column-major face blocks, the row's sum runs over b in order.
template <typename T, int NF, int PC>
__global__ void pc_apply(int64_t nFaces, const T* __restrict__ pc, const T* __restrict__ in, T* __restrict__ out) {
  const int64_t n = nFaces * NF;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t f = i / NF;
    const int a = (int)(i % NF);
    T z;
    if (PC == 0) z = in[i];
    else if (PC == 1) z = pc[i] * in[i];
    else {
      z = 0;
      const T* blk = pc + f * NF * NF + a;
      const T* v = in + f * NF;
      for (int b = 0; b < NF; ++b) z += blk[b * NF] * v[b];  // column-major
    }
    out[i] = z;
  }
}

// partial[j*grid + block] = sum_i V[j][i] w[i], j < m
template <typename T>
__global__ void __launch_bounds__(kT) multi_dot(int64_t n, int m, const T* __restrict__ V,
                                                const T* __restrict__ w, double* __restrict__ partial) {
  __shared__ double red[kT / 32];
  for (int j = 0; j < m; ++j) {
    double acc = 0.0;
    const T* v = V + (int64_t)j * n;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
      acc += (double)v[i] * (double)w[i];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
      double s = 0.0;
      for (int k = 0; k < kT / 32; ++k) s += red[k];
      partial[(int64_t)j * gridDim.x + blockIdx.x] = s;
    }
    __syncthreads();
  }
}

// w -= sum_j V[j] h[j]
// All m dot products <V_j, w> in one launch: block (x, j) sums a grid-stride chunk of
// V_j . w, so the m products stream at once at full occupancy (w is re-read from L2);
// per-block sums go to partial[j * gridDim.x + x], added on the host in block order.
template <typename T>
__global__ void __launch_bounds__(kT) multi_dot_cols(int64_t n, const T* __restrict__ V, const T* __restrict__ w,
                                                     double* __restrict__ partial) {
  __shared__ double red[kT / 32];
  const int j = blockIdx.y;
  const T* v = V + (int64_t)j * n;
  double acc = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    acc += (double)v[i] * (double)w[i];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double sum = 0.0;
    for (int k = 0; k < kT / 32; ++k) sum += red[k];
    partial[(int64_t)j * gridDim.x + blockIdx.x] = sum;
  }
}

template <typename T>
__global__ void multi_axpy(int64_t n, int m, const T* __restrict__ V, const double* __restrict__ h, T* __restrict__ w) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double acc = (double)w[i];
    for (int j = 0; j < m; ++j) acc -= (double)V[(int64_t)j * n + i] * h[j];
    w[i] = (T)acc;
  }
}

// out = sum_j V[j] y[j]
template <typename T>
__global__ void combine(int64_t n, int m, const T* __restrict__ V, const double* __restrict__ y, T* __restrict__ out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double acc = 0.0;
    for (int j = 0; j < m; ++j) acc += (double)V[(int64_t)j * n + i] * y[j];
    out[i] = (T)acc;
  }
}

template <typename T>
__global__ void scale_into(int64_t n, double a, const T* __restrict__ in, T* __restrict__ out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (T)(a * (double)in[i]);
}

// r = b - r (r holds A x on entry)
template <typename T>
__global__ void rsub(int64_t n, const T* __restrict__ b, T* __restrict__ r) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    r[i] = b[i] - r[i];
}

template <typename T>
__global__ void axpy1(int64_t n, const T* __restrict__ d, T* __restrict__ x) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    x[i] += d[i];
}

template <typename T>
__global__ void add_into(int64_t n, double a, const T* __restrict__ d, double* __restrict__ x) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    x[i] += a * (double)d[i];
}

__global__ void to_f32(int64_t n, const double* __restrict__ src, double scale, float* __restrict__ dst) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = (float)(src[i] * scale);
}

template <int NF>
__global__ void copy_bnd(TraceView A, const double* __restrict__ bS, double* __restrict__ x) {
  for (int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; f < A.nFaces; f += (int64_t)gridDim.x * blockDim.x)
    if (A.isBnd[f])
      for (int a = 0; a < NF; ++a) x[f * NF + a] = bS[f * NF + a];
}

template <typename K>
int grid_for(K k, int threads) {
  int dev = 0, nsm = 0, perSM = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, k, threads, 0);
  return nsm * (perSM < 1 ? 1 : perSM);
}

// One restarted GMRES cycle sequence in precision T on A' (values val, masked
// on the fly when MASKED), solving A' x = b from x = 0. Returns status; adds
// the iterations to *its.
template <typename T, int NF, int NBMAX, bool MASKED>
int gmres_run(const TraceView& A, const T* val, int pcT, const T* pc, const T* b, T* x, T* V, T* w, T* t,
              double* partials, double* hdev, int m, double rtol, int maxits, int* its, double* relres,
              cudaStream_t s, KernelTimer* tm, int kid) {
  const int64_t n = A.nFaces * NF;
  const int gOp = grid_for(op_apply<T, NF, NBMAX, MASKED>, kT);
  const int gVec = grid_for(multi_dot<T>, kT);
  const int gPc = (int)std::min<int64_t>((A.nFaces * NF + 127) / 128, 152 * 64);
  std::vector<double> hp((size_t)(m + 1) * gVec), H((size_t)(m + 1) * m), cs(m), sn(m), g(m + 1);
  auto apply_pc = [&](const T* in, T* out) {
    switch (pcT) {
      case 0: pc_apply<T, NF, 0><<<gPc, 128, 0, s>>>(A.nFaces, pc, in, out); break;
      case 1: pc_apply<T, NF, 1><<<gPc, 128, 0, s>>>(A.nFaces, pc, in, out); break;
      default: pc_apply<T, NF, 2><<<gPc, 128, 0, s>>>(A.nFaces, pc, in, out); break;
    }
  };
  auto op = [&](const T* in, T* out) {
    tm->begin(kid, s);
    op_apply<T, NF, NBMAX, MASKED><<<gOp, kT, 0, s>>>(A, val, in, out);
    tm->end(kid, s);
  };
  auto dots = [&](const T* W, int cnt, const T* Vb, std::vector<double>& out) {
    // Gram-Schmidt: the cnt products side by side, about gVec blocks in all
    const int gd = cnt > 1 ? std::max(8, gVec / cnt) : gVec;
    if (cnt > 1) multi_dot_cols<T><<<dim3(gd, cnt), kT, 0, s>>>(n, Vb, W, partials);
    else multi_dot<T><<<gd, kT, 0, s>>>(n, cnt, Vb, W, partials);
    cudaMemcpyAsync(hp.data(), partials, sizeof(double) * cnt * gd, cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    out.assign(cnt, 0.0);
    for (int j = 0; j < cnt; ++j)
      for (int k = 0; k < gd; ++k) out[j] += hp[(size_t)j * gd + k];
  };
  auto norm = [&](const T* W) {
    std::vector<double> o;
    dots(W, 1, W, o);
    return std::sqrt(o[0]);
  };
  cudaMemsetAsync(x, 0, sizeof(T) * n, s);
  double bnorm = norm(b);
  if (bnorm == 0.0) {
    *relres = 0.0;
    return 0;
  }
  int it = 0;
  double rnorm = bnorm;
  // r = b (x = 0)
  scale_into<T><<<gVec, kT, 0, s>>>(n, 1.0, b, w);
  while (true) {
    if (it > 0) {  // true residual at a restart: r = b - A' x
      op(x, w);
      rsub<T><<<gVec, kT, 0, s>>>(n, b, w);
    }
    rnorm = norm(w);
    if (!std::isfinite(rnorm)) return 7;
    if (rnorm <= rtol * bnorm) break;
    if (it >= maxits) {
      *its += it;
      *relres = rnorm / bnorm;
      return 5;
    }
    scale_into<T><<<gVec, kT, 0, s>>>(n, 1.0 / rnorm, w, V);
    std::fill(g.begin(), g.end(), 0.0);
    g[0] = rnorm;
    int j = 0;
    bool breakdown = false;
    for (; j < m && it < maxits; ++j, ++it) {
      T* vj1 = V + (size_t)(j + 1) * n;
      apply_pc(V + (size_t)j * n, t);
      op(t, vj1);
      std::vector<double> h1, h2;
      for (int pass = 0; pass < 2; ++pass) {
        std::vector<double>& hh = pass == 0 ? h1 : h2;
        dots(vj1, j + 1, V, hh);
        cudaMemcpyAsync(hdev, hh.data(), sizeof(double) * (j + 1), cudaMemcpyHostToDevice, s);
        multi_axpy<T><<<gVec, kT, 0, s>>>(n, j + 1, V, hdev, vj1);
      }
      for (int i = 0; i <= j; ++i) H[i + (size_t)j * (m + 1)] = h1[i] + h2[i];
      double hn = norm(vj1);
      H[j + 1 + (size_t)j * (m + 1)] = hn;
      if (hn > 0.0) scale_into<T><<<gVec, kT, 0, s>>>(n, 1.0 / hn, vj1, vj1);
      for (int i = 0; i < j; ++i) {
        double a0 = H[i + (size_t)j * (m + 1)], b0 = H[i + 1 + (size_t)j * (m + 1)];
        H[i + (size_t)j * (m + 1)] = cs[i] * a0 + sn[i] * b0;
        H[i + 1 + (size_t)j * (m + 1)] = -sn[i] * a0 + cs[i] * b0;
      }
      double a0 = H[j + (size_t)j * (m + 1)], b0 = H[j + 1 + (size_t)j * (m + 1)];
      double den = std::sqrt(a0 * a0 + b0 * b0);
      if (den == 0.0 || !std::isfinite(den)) {
        breakdown = true;
        break;
      }
      cs[j] = a0 / den;
      sn[j] = b0 / den;
      H[j + (size_t)j * (m + 1)] = den;
      H[j + 1 + (size_t)j * (m + 1)] = 0.0;
      g[j + 1] = -sn[j] * g[j];
      g[j] = cs[j] * g[j];
      if (std::fabs(g[j + 1]) <= rtol * bnorm || hn == 0.0) {
        ++j;
        ++it;
        break;
      }
    }
    if (j > 0) {
      std::vector<double> y(j);
      for (int i = j - 1; i >= 0; --i) {
        double acc = g[i];
        for (int k = i + 1; k < j; ++k) acc -= H[i + (size_t)k * (m + 1)] * y[k];
        y[i] = acc / H[i + (size_t)i * (m + 1)];
      }
      cudaMemcpyAsync(hdev, y.data(), sizeof(double) * j, cudaMemcpyHostToDevice, s);
      combine<T><<<gVec, kT, 0, s>>>(n, j, V, hdev, w);
      apply_pc(w, t);
      axpy1<T><<<gVec, kT, 0, s>>>(n, t, x);  // x += M^{-1} V y
    }
    if (breakdown) {
      *its += it;
      return 6;
    }
    if (it == 0) break;
  }
  *its += it;
  *relres = rnorm / bnorm;
  return 0;
}

template <int NF, int NBMAX>
int drive(const TraceSolveArgs& a, TraceSolveResult* out) {
  cudaStream_t s = a.stream;
  const TraceView& A = a.A;
  const int64_t n = A.nFaces * NF;
  const int m = a.restart;
  KernelTimer* tm = a.timer;
  if (!a.prepared) trace_prepare(a);
  const int gVec = grid_for(multi_dot<double>, kT);
  double* x = a.x;
  int its = 0, status = 0, refinements = 0;
  double relres = 0.0;
  if (!a.mixed) {
    // FP64 GMRES on A' for the correction d of x0 = [0, g]: A' d = b' - A' x0
    copy_bnd<NF><<<(unsigned)((A.nFaces + 255) / 256), 256, 0, s>>>(A, a.ws.bS, x);
    if (!a.use_initial_guess) {
      cudaMemsetAsync(x, 0, sizeof(double) * n, s);
      copy_bnd<NF><<<(unsigned)((A.nFaces + 255) / 256), 256, 0, s>>>(A, a.ws.bS, x);
    }
    double* r = a.ws.r;
    op_apply<double, NF, NBMAX, true><<<grid_for(op_apply<double, NF, NBMAX, true>, kT), kT, 0, s>>>(A, a.val, x, r);
    rsub<double><<<gVec, kT, 0, s>>>(n, a.ws.bS, r);
    // tolerance relative to the reference ||b||
    std::vector<double> hp(gVec);
    multi_dot<double><<<gVec, kT, 0, s>>>(n, 1, a.rhs, a.rhs, a.ws.partials);
    cudaMemcpyAsync(hp.data(), a.ws.partials, sizeof(double) * gVec, cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    double bb = 0.0;
    for (double v : hp) bb += v;
    multi_dot<double><<<gVec, kT, 0, s>>>(n, 1, r, r, a.ws.partials);
    cudaMemcpyAsync(hp.data(), a.ws.partials, sizeof(double) * gVec, cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    double rr = 0.0;
    for (double v : hp) rr += v;
    double rtol_rel = rr > 0 ? a.rtol * std::sqrt(bb) / std::sqrt(rr) : 1.0;
    if (rr > 0 && rtol_rel < 1.0) {
      double* d = a.ws.z;
      status = gmres_run<double, NF, NBMAX, true>(A, a.val, a.precond, a.ws.pc64, r, d, a.ws.V64, a.ws.q, a.ws.p0,
                                                   a.ws.partials, a.ws.hdev, m, rtol_rel, a.maxits, &its, &relres, s,
                                                   tm, K_SPMV64);
      add_into<double><<<gVec, kT, 0, s>>>(n, 1.0, d, x);
    }
  } else {
    // FP64 refinement around FP32 GMRES on the FP32 copy of A'
    if (!a.use_initial_guess) {
      cudaMemsetAsync(x, 0, sizeof(double) * n, s);
      copy_bnd<NF><<<(unsigned)((A.nFaces + 255) / 256), 256, 0, s>>>(A, a.ws.bS, x);
    }
    std::vector<double> hp(gVec);
    auto dot64 = [&](const double* u, const double* v) {
      multi_dot<double><<<gVec, kT, 0, s>>>(n, 1, u, v, a.ws.partials);
      cudaMemcpyAsync(hp.data(), a.ws.partials, sizeof(double) * gVec, cudaMemcpyDeviceToHost, s);
      cudaStreamSynchronize(s);
      double acc = 0.0;
      for (double v2 : hp) acc += v2;
      return acc;
    };
    double bb = dot64(a.rhs, a.rhs);
    int left = a.maxits;
    while (true) {
      double* r = a.ws.r;
      op_apply<double, NF, NBMAX, true><<<grid_for(op_apply<double, NF, NBMAX, true>, kT), kT, 0, s>>>(A, a.val, x, r);
      rsub<double><<<gVec, kT, 0, s>>>(n, a.ws.bS, r);
      double rr = dot64(r, r);
      if (!std::isfinite(rr)) {
        status = 7;
        break;
      }
      if (rr <= a.rtol * a.rtol * bb) break;
      if (left <= 0 || refinements >= a.max_refinements) {
        status = 5;
        break;
      }
      double rn = std::sqrt(rr);
      // FP32 right-hand side r / ||r||
      to_f32<<<gVec, kT, 0, s>>>(n, r, 1.0 / rn, a.ws.rhs32);
      double want = a.rtol * std::sqrt(bb) / rn;
      double inner = a.inner_rtol > want ? a.inner_rtol : want;
      int it = 0;
      double rres = 0.0;
      int st = gmres_run<float, NF, NBMAX, false>(A, a.ws.val32, a.precond, a.ws.pc32, a.ws.rhs32, a.ws.d32,
                                                   a.ws.V32, a.ws.q32, a.ws.p032, a.ws.partials, a.ws.hdev, m, inner,
                                                   left, &it, &rres, s, tm, K_SPMV32);
      its += it;
      left -= it;
      refinements += 1;
      if (st != 0 && st != 5) {
        status = st;
        break;
      }
      add_into<float><<<gVec, kT, 0, s>>>(n, rn, a.ws.d32, x);
    }
  }
  out->iterations = its;
  out->refinements = refinements;
  trace_ref_residual(a, out);
  cudaError_t e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    out->cudaErr = e;
    return 3;
  }
  return status;
}

}  // namespace

template <int NF, int NBMAX>
int projection_t(const TraceSolveArgs& a, const double* const* X, int K, double* Y) {
  cudaStream_t s = a.stream;
  const TraceView& A = a.A;
  const int64_t n = A.nFaces * NF;
  const int gOp = grid_for(op_apply<double, NF, NBMAX, true>, kT);
  const int gVec = grid_for(multi_dot<double>, kT);
  for (int i = 0; i < K; ++i) op_apply<double, NF, NBMAX, true><<<gOp, kT, 0, s>>>(A, a.val, X[i], Y + (size_t)i * n);
  // Gram matrix G_ij = <Y_i, Y_j> and g_i = <Y_i, b'>: one batched dot launch per column
  std::vector<double> G((size_t)K * K), g(K), hp((size_t)(K + 1) * gVec);
  auto dots = [&](const double* w, int cnt, std::vector<double>& out) {
    const int gd = cnt > 1 ? std::max(8, gVec / cnt) : gVec;
    if (cnt > 1) multi_dot_cols<double><<<dim3(gd, cnt), kT, 0, s>>>(n, Y, w, a.ws.partials);
    else multi_dot<double><<<gd, kT, 0, s>>>(n, 1, Y, w, a.ws.partials);
    cudaMemcpyAsync(hp.data(), a.ws.partials, sizeof(double) * cnt * gd, cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    out.assign(cnt, 0.0);
    for (int j = 0; j < cnt; ++j)
      for (int k = 0; k < gd; ++k) out[j] += hp[(size_t)j * gd + k];
  };
  std::vector<double> col;
  for (int j = 0; j < K; ++j) {
    dots(Y + (size_t)j * n, K, col);
    for (int i = 0; i < K; ++i) G[i + (size_t)j * K] = col[i];
  }
  dots(a.ws.bS, K, col);
  g = col;
  // Cholesky of G with the nearly dependent directions dropped (successive solutions are
  // close to parallel): a pivot below 1e-12 of the largest diagonal removes that vector
  double dmax = 0.0;
  for (int i = 0; i < K; ++i) dmax = std::max(dmax, G[i + (size_t)i * K]);
  if (!(dmax > 0.0) || !std::isfinite(dmax)) return 0;
  std::vector<double> Lc((size_t)K * K, 0.0), c(K, 0.0), z(K, 0.0);
  std::vector<int> keep;
  for (int i = 0; i < K; ++i) {
    double d = G[i + (size_t)i * K];
    for (size_t a2 = 0; a2 < keep.size(); ++a2) d -= Lc[i + (size_t)keep[a2] * K] * Lc[i + (size_t)keep[a2] * K];
    if (!(d > 1e-12 * dmax)) continue;
    const double ld = std::sqrt(d);
    Lc[i + (size_t)i * K] = ld;
    for (int r = i + 1; r < K; ++r) {
      double v = G[r + (size_t)i * K];
      for (int kk : keep) v -= Lc[r + (size_t)kk * K] * Lc[i + (size_t)kk * K];
      Lc[r + (size_t)i * K] = v / ld;
    }
    keep.push_back(i);
  }
  if (keep.empty()) return 0;
  for (size_t a2 = 0; a2 < keep.size(); ++a2) {  // L z = g on the kept indices
    const int i = keep[a2];
    double v = g[i];
    for (size_t b2 = 0; b2 < a2; ++b2) v -= Lc[i + (size_t)keep[b2] * K] * z[keep[b2]];
    z[i] = v / Lc[i + (size_t)i * K];
  }
  for (int a2 = (int)keep.size() - 1; a2 >= 0; --a2) {  // L^T c = z
    const int i = keep[a2];
    double v = z[i];
    for (size_t b2 = a2 + 1; b2 < keep.size(); ++b2) v -= Lc[keep[b2] + (size_t)i * K] * c[keep[b2]];
    c[i] = v / Lc[i + (size_t)i * K];
  }
  for (double v : c)
    if (!std::isfinite(v)) return 0;
  // x0 = sum_i c_i X_i: the X_i are separate buffers, so add them one by one
  scale_into<double><<<gVec, kT, 0, s>>>(n, c[0], X[0], a.x);
  for (int i = 1; i < K; ++i) add_into<double><<<gVec, kT, 0, s>>>(n, c[i], X[i], a.x);
  return (int)keep.size();
}

int trace_projection_guess(const TraceSolveArgs& a, const double* const* X, int K, double* Y) {
  if (K < 1 || K > 8) return 0;
  const int NF = a.A.NF;
  if (a.dim == 2) {
    switch (NF) {
      case 2: return projection_t<2, 5>(a, X, K, Y);
      case 3: return projection_t<3, 5>(a, X, K, Y);
      case 4: return projection_t<4, 5>(a, X, K, Y);
      case 5: return projection_t<5, 5>(a, X, K, Y);
      case 6: return projection_t<6, 5>(a, X, K, Y);
      case 8: return projection_t<8, 5>(a, X, K, Y);
      case 10: return projection_t<10, 5>(a, X, K, Y);
      case 12: return projection_t<12, 5>(a, X, K, Y);
    }
  } else if (a.dim == 3) {
    switch (NF) {
      case 3: return projection_t<3, 7>(a, X, K, Y);
      case 6: return projection_t<6, 7>(a, X, K, Y);
      case 10: return projection_t<10, 7>(a, X, K, Y);
    }
  }
  return 0;
}

template <int NF, int NBMAX>
int gmres_f32_t(const F32SolveArgs& a, int* its) {
  trace_prepare_f32(a.dim, a.A, a.val, a.rhs, a.ws.bS32, a.rebuildPrecond ? a.precond : 0, a.ws.pc32, a.stream);
  double relres = 0.0;
  return gmres_run<float, NF, NBMAX, true>(a.A, a.val, a.precond, a.ws.pc32, a.ws.bS32, a.x, a.ws.V32, a.ws.q32,
                                          a.ws.p032, a.ws.partials, a.ws.hdev, a.restart, a.rtol, a.maxits, its,
                                          &relres, a.stream, a.timer, K_SPMV32);
}

int trace_gmres_f32(const F32SolveArgs& a, int* its) {
  const int NF = a.A.NF;
  if (a.dim == 2) {
    switch (NF) {
      case 2: return gmres_f32_t<2, 5>(a, its);
      case 3: return gmres_f32_t<3, 5>(a, its);
      case 4: return gmres_f32_t<4, 5>(a, its);
      case 5: return gmres_f32_t<5, 5>(a, its);
      case 6: return gmres_f32_t<6, 5>(a, its);
    }
  } else if (a.dim == 3) {
    switch (NF) {
      case 3: return gmres_f32_t<3, 7>(a, its);
      case 6: return gmres_f32_t<6, 7>(a, its);
      case 10: return gmres_f32_t<10, 7>(a, its);
    }
  }
  return 9;
}

int trace_gmres(const TraceSolveArgs& a, TraceSolveResult* out) {
  const int NF = a.A.NF;
  if (a.dim == 2) {
    switch (NF) {
      case 2: return drive<2, 5>(a, out);
      case 3: return drive<3, 5>(a, out);
      case 4: return drive<4, 5>(a, out);
      case 5: return drive<5, 5>(a, out);
      case 6: return drive<6, 5>(a, out);
      // vector (Burgers) trace blocks, Nf * dim values per face
      case 8: return drive<8, 5>(a, out);
      case 10: return drive<10, 5>(a, out);
      case 12: return drive<12, 5>(a, out);
    }
  } else if (a.dim == 3) {
    switch (NF) {
      case 3: return drive<3, 7>(a, out);
      case 6: return drive<6, 7>(a, out);
      case 10: return drive<10, 7>(a, out);
    }
  }
  return 9;
}

}  // namespace hfx
