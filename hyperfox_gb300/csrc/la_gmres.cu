// Generic sparse system (LinAlgebraInterface drop-in) and its device GMRES.
//
// Replaces PetscInterface (PetscInterface.cpp:48-265) for any nonsingular
// system: KSPGMRES with restart (PETSc default 30) and a Jacobi
// preconditioner (PetscOpts.h:12-16). Right preconditioning keeps the tested
// residual the true ||b - A x|| (PetscOpts::rtol semantics), with classical
// Gram-Schmidt applied twice for orthogonality.
#include <algorithm>
#include <cmath>

#include "la_gmres.h"

namespace hfx {
namespace {

__global__ void csr_spmv_jac(int n, const int64_t* __restrict__ rp, const int* __restrict__ col,
                             const double* __restrict__ val, const double* __restrict__ dinv,
                             const double* __restrict__ v, double* __restrict__ y) {
  // y = A (D^{-1} v), one warp per row
  int lane = threadIdx.x & 31;
  for (int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; row < n;
       row += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    double acc = 0.0;
    for (int64_t k = rp[row] + lane; k < rp[row + 1]; k += 32) {
      int j = col[k];
      acc += val[k] * (dinv ? dinv[j] * v[j] : v[j]);
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (lane == 0) y[row] = acc;
  }
}

// partial dots of w against V[0..m) (column-major n x m), per block
__global__ void multi_dot(int n, int m, const double* __restrict__ V, const double* __restrict__ w,
                          double* __restrict__ partial) {
  __shared__ double red[32][8];
  for (int j = 0; j < m; ++j) {
    double acc = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
      acc += V[(int64_t)j * n + i] * w[i];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) red[0][threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
      double s = 0.0;
      for (int k = 0; k < (int)(blockDim.x >> 5); ++k) s += red[0][k];
      partial[(int64_t)j * gridDim.x + blockIdx.x] = s;
    }
    __syncthreads();
  }
}

// w -= V h (h on the device, m entries)
__global__ void multi_axpy(int n, int m, const double* __restrict__ V, const double* __restrict__ h,
                           double* __restrict__ w) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double acc = w[i];
    for (int j = 0; j < m; ++j) acc -= V[(int64_t)j * n + i] * h[j];
    w[i] = acc;
  }
}

__global__ void scale_copy(int n, double a, const double* __restrict__ src, double* __restrict__ dst) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = a * src[i];
}

__global__ void sub_from(int n, const double* __restrict__ b, double* __restrict__ y) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = b[i] - y[i];
}

// x += D^{-1} (V y)
__global__ void update_x(int n, int m, const double* __restrict__ V, const double* __restrict__ y,
                         const double* __restrict__ dinv, double* __restrict__ x) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double acc = 0.0;
    for (int j = 0; j < m; ++j) acc += V[(int64_t)j * n + i] * y[j];
    x[i] += dinv ? dinv[i] * acc : acc;
  }
}

struct Buf {
  void* p = nullptr;
  ~Buf() {
    if (p) cudaFree(p);
  }
};

}  // namespace

void LaSystem::allocate(int n) {
  n_ = n;
  assembled_ = false;
  rows_.assign(n, {});
  rhs_.assign(n, 0.0);
  rowptr_.clear();
  col_.clear();
  val_.clear();
}

bool LaSystem::add_block(int nr, const int* rows, int nc, const int* cols, const double* vals, bool insert,
                         std::string* err) {
  for (int i = 0; i < nr; ++i)
    for (int j = 0; j < nc; ++j) {
      int r = rows[i], c = cols[j];
      if (r < 0 || r >= n_ || c < 0 || c >= n_) {
        *err = "la: index out of range";
        return false;
      }
      double v = vals[(int64_t)i * nc + j];  // row-major is.size() x js.size() (HDGSolver.cpp:558)
      if (insert) rows_[r][c] = v;
      else rows_[r][c] += v;
    }
  return true;
}

bool LaSystem::add_rhs(int n, const int* idx, const double* vals, bool insert, std::string* err) {
  for (int i = 0; i < n; ++i) {
    if (idx[i] < 0 || idx[i] >= n_) {
      *err = "la: index out of range";
      return false;
    }
    if (insert) rhs_[idx[i]] = vals[i];
    else rhs_[idx[i]] += vals[i];
  }
  return true;
}

bool LaSystem::zero_rows(int n, const int* rows, std::string* err) {
  // MatZeroRows(M, n, rows, 0.0, 0, 0): entries zeroed, pattern kept
  for (int i = 0; i < n; ++i) {
    if (rows[i] < 0 || rows[i] >= n_) {
      *err = "la: index out of range";
      return false;
    }
    for (auto& kv : rows_[rows[i]]) kv.second = 0.0;
  }
  return true;
}

void LaSystem::assemble() {
  rowptr_.assign(n_ + 1, 0);
  col_.clear();
  val_.clear();
  std::vector<std::pair<int, double>> tmp;
  for (int r = 0; r < n_; ++r) {
    tmp.assign(rows_[r].begin(), rows_[r].end());
    std::sort(tmp.begin(), tmp.end());
    for (auto& kv : tmp) {
      col_.push_back(kv.first);
      val_.push_back(kv.second);
    }
    rowptr_[r + 1] = (int64_t)col_.size();
  }
  assembled_ = true;
}

void LaSystem::clear() {
  // MatZeroEntries + VecSet(b, 0) + assemble (PetscInterface.cpp:249-259)
  for (auto& row : rows_)
    for (auto& kv : row) kv.second = 0.0;
  std::fill(rhs_.begin(), rhs_.end(), 0.0);
  assemble();
}

int LaSystem::solve(double rtol, int maxits, int restart, int jacobi, cudaStream_t s, double* xh, LaSolveResult* res,
                    std::string* err) {
  const int n = n_;
  const int m = std::max(1, std::min(restart, n));
  const int threads = 256;
  const int grid = (int)std::min<int64_t>(1024, (n + threads - 1) / threads);
  const int gridRows = (int)std::min<int64_t>(4096, ((int64_t)n * 32 + threads - 1) / threads);
  std::vector<double> dinv(n, 1.0);
  if (jacobi)
    for (int r = 0; r < n; ++r)
      for (int64_t k = rowptr_[r]; k < rowptr_[r + 1]; ++k)
        if (col_[k] == r && val_[k] != 0.0) dinv[r] = 1.0 / val_[k];
  Buf bRp, bCol, bVal, bDinv, bB, bX, bW, bV, bH, bPart;
  auto alloc = [&](Buf& b, size_t bytes) { return cudaMalloc(&b.p, bytes > 0 ? bytes : 8); };
  if (alloc(bRp, sizeof(int64_t) * (n + 1)) || alloc(bCol, sizeof(int) * col_.size()) ||
      alloc(bVal, sizeof(double) * val_.size()) || alloc(bDinv, sizeof(double) * n) || alloc(bB, sizeof(double) * n) ||
      alloc(bX, sizeof(double) * n) || alloc(bW, sizeof(double) * n) ||
      alloc(bV, sizeof(double) * (size_t)n * (m + 1)) || alloc(bH, sizeof(double) * (m + 1)) ||
      alloc(bPart, sizeof(double) * (size_t)(m + 1) * grid)) {
    *err = "la_solve: device allocation failed";
    return 4;
  }
  int64_t* rp = (int64_t*)bRp.p;
  int* col = (int*)bCol.p;
  double *val = (double*)bVal.p, *dv = (double*)bDinv.p, *b = (double*)bB.p, *x = (double*)bX.p, *w = (double*)bW.p;
  double *V = (double*)bV.p, *h = (double*)bH.p, *part = (double*)bPart.p;
  const double* dinvp = jacobi ? dv : nullptr;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, s);
  cudaMemcpyAsync(rp, rowptr_.data(), sizeof(int64_t) * (n + 1), cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(col, col_.data(), sizeof(int) * col_.size(), cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(val, val_.data(), sizeof(double) * val_.size(), cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(dv, dinv.data(), sizeof(double) * n, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(b, rhs_.data(), sizeof(double) * n, cudaMemcpyHostToDevice, s);
  cudaMemsetAsync(x, 0, sizeof(double) * n, s);
  std::vector<double> hp((size_t)(m + 1) * grid), H((size_t)(m + 1) * m), cs(m), sn(m), g(m + 1), hv(m + 1);
  auto dots = [&](const double* W, int cnt, std::vector<double>& out) {
    multi_dot<<<grid, threads, 0, s>>>(n, cnt, V, W, part);
    cudaMemcpyAsync(hp.data(), part, sizeof(double) * cnt * grid, cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    out.assign(cnt, 0.0);
    for (int j = 0; j < cnt; ++j)
      for (int k = 0; k < grid; ++k) out[j] += hp[(size_t)j * grid + k];
  };
  auto norm2 = [&](const double* W) {
    // ||W||: place W as column 0 of a temporary V view
    multi_dot<<<grid, threads, 0, s>>>(n, 1, W, W, part);
    cudaMemcpyAsync(hp.data(), part, sizeof(double) * grid, cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    double a = 0.0;
    for (int k = 0; k < grid; ++k) a += hp[k];
    return std::sqrt(a);
  };
  double bnorm = norm2(b);
  int it = 0, status = 0;
  double rnorm = 0.0;
  if (bnorm == 0.0) {
    cudaMemcpy(xh, x, sizeof(double) * n, cudaMemcpyDeviceToHost);
    res->iterations = 0;
    res->rel_residual = 0.0;
    return 0;
  }
  while (true) {
    // r = b - A x  (x is the unpreconditioned iterate, so apply A directly)
    csr_spmv_jac<<<gridRows, threads, 0, s>>>(n, rp, col, val, nullptr, x, w);
    sub_from<<<grid, threads, 0, s>>>(n, b, w);
    rnorm = norm2(w);
    if (!std::isfinite(rnorm)) {
      status = 7;
      break;
    }
    if (rnorm <= rtol * bnorm) break;
    if (it >= maxits) {
      status = 5;
      break;
    }
    scale_copy<<<grid, threads, 0, s>>>(n, 1.0 / rnorm, w, V);
    std::fill(g.begin(), g.end(), 0.0);
    g[0] = rnorm;
    int j = 0;
    bool stop = false;
    for (; j < m && it < maxits; ++j, ++it) {
      double* vj1 = V + (size_t)(j + 1) * n;
      csr_spmv_jac<<<gridRows, threads, 0, s>>>(n, rp, col, val, dinvp, V + (size_t)j * n, vj1);
      std::vector<double> h1, h2;
      for (int pass = 0; pass < 2; ++pass) {
        dots(vj1, j + 1, pass == 0 ? h1 : h2);
        std::vector<double>& hh = pass == 0 ? h1 : h2;
        cudaMemcpyAsync(h, hh.data(), sizeof(double) * (j + 1), cudaMemcpyHostToDevice, s);
        multi_axpy<<<grid, threads, 0, s>>>(n, j + 1, V, h, vj1);
      }
      for (int i = 0; i <= j; ++i) H[i + (size_t)j * (m + 1)] = h1[i] + h2[i];
      double hn = norm2(vj1);
      H[j + 1 + (size_t)j * (m + 1)] = hn;
      if (hn > 0.0) scale_copy<<<grid, threads, 0, s>>>(n, 1.0 / hn, vj1, vj1);
      for (int i = 0; i < j; ++i) {
        double a = H[i + (size_t)j * (m + 1)], bb = H[i + 1 + (size_t)j * (m + 1)];
        H[i + (size_t)j * (m + 1)] = cs[i] * a + sn[i] * bb;
        H[i + 1 + (size_t)j * (m + 1)] = -sn[i] * a + cs[i] * bb;
      }
      double a = H[j + (size_t)j * (m + 1)], bb = H[j + 1 + (size_t)j * (m + 1)];
      double den = std::sqrt(a * a + bb * bb);
      if (den == 0.0) {
        stop = true;
        break;
      }
      cs[j] = a / den;
      sn[j] = bb / den;
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
        double sacc = g[i];
        for (int k = i + 1; k < j; ++k) sacc -= H[i + (size_t)k * (m + 1)] * y[k];
        y[i] = sacc / H[i + (size_t)i * (m + 1)];
      }
      cudaMemcpyAsync(h, y.data(), sizeof(double) * j, cudaMemcpyHostToDevice, s);
      update_x<<<grid, threads, 0, s>>>(n, j, V, h, dinvp, x);
    }
    if (stop) {
      status = 6;
      break;
    }
  }
  cudaEventRecord(e1, s);
  cudaMemcpyAsync(xh, x, sizeof(double) * n, cudaMemcpyDeviceToHost, s);
  cudaError_t ce = cudaStreamSynchronize(s);
  cudaEventElapsedTime(&res->ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  res->iterations = it;
  res->rel_residual = rnorm / bnorm;
  if (ce != cudaSuccess) {
    *err = std::string("la_solve: ") + cudaGetErrorString(ce);
    return 3;
  }
  if (status == 5) *err = "la_solve: not converged within maxits";
  else if (status == 6) *err = "la_solve: GMRES breakdown";
  else if (status == 7) *err = "la_solve: NaN or Inf";
  return status;
}

}  // namespace hfx
