// CG solve of a small trace system that allocates no device memory.
//
// Some callers cannot call cudaMalloc: code that runs while a CUDA stream is
// being captured into a graph (an allocation there breaks or invalidates the
// capture), code inside a framework whose caching allocator owns all device
// memory (a raw cudaMalloc would fragment its pool or exceed its budget), and
// real-time loops that forbid allocation latency. They own their device
// buffers, hand this entry point the system and the solution buffer, and the
// solver's own working memory (the CG vectors, the block-Jacobi inverses, the
// reduction partials and the solver state) lives in one file-scope
// __device__ array of fixed size, resident on every GPU that loads the
// library until the process exits.
//
// The computation is the FP64 CG + per-face block-Jacobi solve of hfx_solve
// (HFX_KSP_CG, HFX_PC_BLOCK_JACOBI): the Dirichlet rows are eliminated
// symmetrically and the interior block negated, and the result is the
// solution of the stored system. Limits: at most HFX_NOALLOC_MAX_DOFS trace
// DOFs and HFX_NOALLOC_MAX_NF nodes per face.
//
// Every call shares the scratch array and leaves the last call's contents in
// it; the entry point clears what must start at zero itself. Calls that
// overlap on the GPU (two streams, two host threads) race on the scratch and
// must be serialised by the caller.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <mutex>

#include <cuda_runtime.h>

#include "../../include/hfx_gb300.h"
#include "krylov.h"

namespace hfx {
namespace {

constexpr int64_t kMaxDofs = HFX_NOALLOC_MAX_DOFS;
constexpr int kMaxNF = HFX_NOALLOC_MAX_NF;
constexpr int kThreads = 256;
constexpr int kMaxBlocks = 1024;  // reduction partials per value
constexpr int kStateDoubles = (int)((sizeof(CgState) + sizeof(double) - 1) / sizeof(double));
// scratch layout (doubles): bS, r, z, p, q | inverse face blocks | partials | state
constexpr int64_t kOffPc = 5 * kMaxDofs;
constexpr int64_t kOffPart = kOffPc + kMaxDofs * kMaxNF;
constexpr int64_t kOffState = kOffPart + 3 * kMaxBlocks;
constexpr int64_t kScratchDoubles = kOffState + kStateDoubles + 8;

__device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

struct NoallocSys {
  int64_t nFaces;
  int NF, nbmax;
  const int64_t* browptr;
  const int* bcol;
  const unsigned char* isBnd;
  const double* val;
  const double* rhs;
};

// last-block-done reduction of NV sums into tot (fixed order), no spin-waits
template <int NV>
__device__ bool reduce_last(double (&v)[NV], double* partials, unsigned* ticket, double (&tot)[NV]) {
  __shared__ double red[NV][kThreads / 32];
  __shared__ bool amLast;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int k = 0; k < NV; ++k) {
    double x = v[k];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) red[k][wid] = x;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 0; k < NV; ++k) {
      double s = 0.0;
      for (int w = 0; w < kThreads / 32; ++w) s += red[k][w];
      partials[(size_t)k * gridDim.x + blockIdx.x] = s;
    }
    __threadfence();
    amLast = atomicAdd(ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!amLast) return false;
  __threadfence();
  if (threadIdx.x == 0) {
    for (int k = 0; k < NV; ++k) {
      double s = 0.0;
      for (unsigned b = 0; b < gridDim.x; ++b) s += ((volatile double*)partials)[(size_t)k * gridDim.x + b];
      tot[k] = s;
    }
    *ticket = 0u;
  }
  return true;
}

// b' (Dirichlet lift, sign flip), inverse diagonal face blocks, x0 = [0, g],
// r0 = b' - A' x0, z0 = M^{-1} r0, p0 = z0; sums r.z, r.r, ||b||^2.
__global__ void __launch_bounds__(kThreads) nk_start(NoallocSys A, double* scr, double* x) {
  const int NF = A.NF;
  const int64_t n = A.nFaces * NF;
  double *bS = scr, *r = scr + kMaxDofs, *z = scr + 2 * kMaxDofs, *p = scr + 3 * kMaxDofs;
  double* pc = scr + kOffPc;
  CgState* st = (CgState*)(scr + kOffState);
  double rz = 0.0, rr = 0.0, bb = 0.0;
  for (int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; f < A.nFaces; f += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b0 = A.browptr[f];
    const int nb = (int)(A.browptr[f + 1] - b0), npos = nb * NF;
    const bool rb = A.isBnd[f];
    double B[kMaxNF][kMaxNF], Bi[kMaxNF][kMaxNF];
    int kd = 0;
    for (int k = 0; k < nb; ++k)
      if (A.bcol[b0 + k] == (int)f) kd = k;
    for (int a = 0; a < NF; ++a) {
      const double* row = A.val + b0 * NF * NF + (int64_t)a * npos;
      double lift = 0.0;
      for (int m = 0; m < npos; ++m) {
        int g = A.bcol[b0 + m / NF];
        if (!rb && A.isBnd[g]) lift += row[m] * A.rhs[(int64_t)g * NF + m % NF];
      }
      int64_t i = f * NF + a;
      bS[i] = rb ? A.rhs[i] : -(A.rhs[i] - lift);
      bb += A.rhs[i] * A.rhs[i];
      for (int b = 0; b < NF; ++b) {
        B[a][b] = rb ? (a == b ? 1.0 : 0.0) : -row[kd * NF + b];
        Bi[a][b] = (a == b) ? 1.0 : 0.0;
      }
    }
    for (int k = 0; k < NF; ++k) {  // Gauss-Jordan, SPD block
      double inv = 1.0 / B[k][k];
      for (int j = 0; j < NF; ++j) {
        B[k][j] *= inv;
        Bi[k][j] *= inv;
      }
      for (int i2 = 0; i2 < NF; ++i2) {
        if (i2 == k) continue;
        double l = B[i2][k];
        for (int j = 0; j < NF; ++j) {
          B[i2][j] -= l * B[k][j];
          Bi[i2][j] -= l * Bi[k][j];
        }
      }
    }
    double rl[kMaxNF];
    for (int a = 0; a < NF; ++a) {
      int64_t i = f * NF + a;
      x[i] = rb ? bS[i] : 0.0;
      rl[a] = rb ? 0.0 : bS[i];
      r[i] = rl[a];
      rr += rl[a] * rl[a];
      for (int b = 0; b < NF; ++b) pc[(f * NF + a) * NF + b] = Bi[a][b];
    }
    for (int a = 0; a < NF; ++a) {
      double zi = 0.0;
      for (int b = 0; b < NF; ++b) zi += Bi[a][b] * rl[b];
      z[f * NF + a] = zi;
      p[f * NF + a] = zi;
      rz += rl[a] * zi;
    }
  }
  (void)n;
  double v[3] = {rz, rr, bb}, tot[3];
  if (reduce_last<3>(v, scr + kOffPart, &st->ticket, tot) && threadIdx.x == 0) {
    st->rz = tot[0];
    st->rr = tot[1];
    st->bb = tot[2];
  }
}

// q = A' p (warp per face), p.q, alpha in the last block
__global__ void __launch_bounds__(kThreads) nk_spmv(NoallocSys A, double* scr) {
  CgState* st = (CgState*)(scr + kOffState);
  if (st->done) return;
  const int NF = A.NF;
  const double* p = scr + 3 * kMaxDofs;
  double* q = scr + 4 * kMaxDofs;
  const int lane = threadIdx.x & 31;
  double pq = 0.0;
  for (int64_t f = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; f < A.nFaces;
       f += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    const int64_t b0 = A.browptr[f];
    const int nb = (int)(A.browptr[f + 1] - b0), npos = nb * NF;
    const bool rb = A.isBnd[f];
    for (int a = 0; a < NF; ++a) {
      const double* row = A.val + b0 * NF * NF + (int64_t)a * npos;
      double acc = 0.0;
      for (int m = lane; m < npos; m += 32) {
        int g = A.bcol[b0 + m / NF];
        if (!rb && !A.isBnd[g]) acc += row[m] * p[(int64_t)g * NF + m % NF];
      }
      for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
      if (lane == 0) {
        int64_t i = f * NF + a;
        double qi = rb ? p[i] : -acc;
        q[i] = qi;
        pq += p[i] * qi;
      }
    }
  }
  double v[1] = {pq}, tot[1];
  if (reduce_last<1>(v, scr + kOffPart, &st->ticket, tot) && threadIdx.x == 0) {
    if (!(tot[0] > 0.0) || !isfinite(tot[0])) {
      st->status = isfinite(tot[0]) ? HFX_ERR_BREAKDOWN : HFX_ERR_NAN;
      st->done = 1;
    } else {
      st->alpha = st->rz / tot[0];
    }
  }
}

// x += alpha p, r -= alpha q, z = M^{-1} r; beta and the convergence test
__global__ void __launch_bounds__(kThreads) nk_update(NoallocSys A, double* scr, double* x, double tol2) {
  CgState* st = (CgState*)(scr + kOffState);
  if (st->done) return;
  const int NF = A.NF;
  double *r = scr + kMaxDofs, *z = scr + 2 * kMaxDofs, *p = scr + 3 * kMaxDofs, *q = scr + 4 * kMaxDofs;
  const double* pc = scr + kOffPc;
  const double alpha = st->alpha;
  double rz = 0.0, rr = 0.0;
  for (int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; f < A.nFaces; f += (int64_t)gridDim.x * blockDim.x) {
    double rl[kMaxNF];
    for (int a = 0; a < NF; ++a) {
      int64_t i = f * NF + a;
      x[i] += alpha * p[i];
      rl[a] = r[i] - alpha * q[i];
      r[i] = rl[a];
      rr += rl[a] * rl[a];
    }
    for (int a = 0; a < NF; ++a) {
      double zi = 0.0;
      for (int b = 0; b < NF; ++b) zi += pc[(f * NF + a) * NF + b] * rl[b];
      z[f * NF + a] = zi;
      rz += rl[a] * zi;
    }
  }
  double v[2] = {rz, rr}, tot[2];
  if (reduce_last<2>(v, scr + kOffPart, &st->ticket, tot) && threadIdx.x == 0) {
    st->iters += 1;
    st->rr = tot[1];
    if (!isfinite(tot[0]) || !isfinite(tot[1])) {
      st->status = HFX_ERR_NAN;
      st->done = 1;
    } else {
      st->beta = tot[0] / st->rz;
      st->rz = tot[0];
      if (tot[1] <= tol2) st->done = 1;
      else if (st->iters >= st->maxits) {
        st->status = HFX_ERR_NOT_CONVERGED;
        st->done = 1;
      }
    }
  }
}

__global__ void nk_pupdate(NoallocSys A, double* scr) {
  CgState* st = (CgState*)(scr + kOffState);
  if (st->done) return;
  const double beta = st->beta;
  const double* z = scr + 2 * kMaxDofs;
  double* p = scr + 3 * kMaxDofs;
  const int64_t n = A.nFaces * A.NF;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    p[i] = z[i] + beta * p[i];
}

// ||b - A x||^2 of the stored system (Dirichlet identity rows included)
__global__ void __launch_bounds__(kThreads) nk_residual(NoallocSys A, double* scr, const double* x) {
  CgState* st = (CgState*)(scr + kOffState);
  const int NF = A.NF;
  const int lane = threadIdx.x & 31;
  double rr = 0.0;
  for (int64_t f = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; f < A.nFaces;
       f += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    const int64_t b0 = A.browptr[f];
    const int nb = (int)(A.browptr[f + 1] - b0), npos = nb * NF;
    for (int a = 0; a < NF; ++a) {
      const double* row = A.val + b0 * NF * NF + (int64_t)a * npos;
      double acc = 0.0;
      for (int m = lane; m < npos; m += 32) acc += row[m] * x[(int64_t)A.bcol[b0 + m / NF] * NF + m % NF];
      for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
      if (lane == 0) {
        double ri = A.rhs[f * NF + a] - acc;
        rr += ri * ri;
      }
    }
  }
  double v[1] = {rr}, tot[1];
  if (reduce_last<1>(v, scr + kOffPart, &st->ticket, tot) && threadIdx.x == 0) st->res_rr = tot[0];
}

std::mutex g_mutex;
double* g_dev_ptr[64] = {};

}  // namespace
}  // namespace hfx

using namespace hfx;

extern "C" int hfx_trace_solve_noalloc(int dim, int nodesPerFace, int nFaces, const int64_t* browptr, const int* bcol,
                                       const unsigned char* isBoundary, const double* val, const double* rhs,
                                       double* x, double rtol, int maxits, void* stream, hfx_solve_info* info) {
  auto fail = [&](int code) {
    if (info) {
      info->status = code;
      info->iterations = 0;
      info->refinements = 0;
      info->rel_residual = 0.0;
      info->solve_ms = 0.0;
      info->fallback = 0;
      info->coarse_degree = 0;
    }
    return code;
  };
  if (dim < 2 || dim > 3 || nodesPerFace < 1 || nodesPerFace > kMaxNF || nFaces < 1 ||
      (int64_t)nFaces * nodesPerFace > kMaxDofs)
    return fail(HFX_ERR_ARG);  // beyond HFX_NOALLOC_MAX_DOFS / HFX_NOALLOC_MAX_NF
  if (!browptr || !bcol || !isBoundary || !val || !rhs || !x || !(rtol > 0.0) || maxits < 1) return fail(HFX_ERR_ARG);
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return fail(HFX_ERR_CUDA);
  double* scr = nullptr;
  {
    // set-up once per device, with that device current: the device address of
    // the scratch array (its host-side name is not a device address)
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_dev_ptr[dev]) {
      void* ptr = nullptr;
      if (cudaGetSymbolAddress(&ptr, g_noalloc_scratch) != cudaSuccess) return fail(HFX_ERR_CUDA);
      g_dev_ptr[dev] = (double*)ptr;
    }
    scr = g_dev_ptr[dev];
  }
  cudaStream_t s = (cudaStream_t)stream;
  auto t0 = std::chrono::steady_clock::now();
  NoallocSys A{nFaces, nodesPerFace, dim == 2 ? 5 : 7, browptr, bcol, isBoundary, val, rhs};
  CgState* st = (CgState*)(scr + kOffState);
  CgState init{};
  init.maxits = maxits;
  // clear the state (ticket, flags, counters) the previous call left behind
  if (cudaMemcpyAsync(st, &init, sizeof(CgState), cudaMemcpyHostToDevice, s) != cudaSuccess) return fail(HFX_ERR_CUDA);
  int nsm = 0;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  int gridF = (int)std::min<int64_t>(kMaxBlocks, std::max<int64_t>(1, ((int64_t)nFaces * 32 + kThreads - 1) / kThreads));
  int gridV = (int)std::min<int64_t>(kMaxBlocks, std::max<int64_t>(1, ((int64_t)nFaces + kThreads - 1) / kThreads));
  gridF = std::min(gridF, 4 * nsm);
  gridV = std::min(gridV, 4 * nsm);
  nk_start<<<gridV, kThreads, 0, s>>>(A, scr, x);
  CgState h;
  if (cudaMemcpyAsync(&h, st, sizeof(CgState), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return fail(HFX_ERR_CUDA);
  const double tol2 = rtol * rtol * h.bb;
  if (h.rr > tol2) {
    while (true) {
      for (int k = 0; k < 25; ++k) {
        nk_spmv<<<gridF, kThreads, 0, s>>>(A, scr);
        nk_update<<<gridV, kThreads, 0, s>>>(A, scr, x, tol2);
        nk_pupdate<<<gridV, kThreads, 0, s>>>(A, scr);
      }
      if (cudaMemcpyAsync(&h, st, sizeof(CgState), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
          cudaStreamSynchronize(s) != cudaSuccess)
        return fail(HFX_ERR_CUDA);
      if (h.done) break;
    }
  }
  nk_residual<<<gridF, kThreads, 0, s>>>(A, scr, x);
  if (cudaMemcpyAsync(&h, st, sizeof(CgState), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return fail(HFX_ERR_CUDA);
  if (cudaGetLastError() != cudaSuccess) return fail(HFX_ERR_CUDA);
  if (info) {
    info->status = h.status;
    info->iterations = h.iters;
    info->refinements = 0;
    info->rel_residual = h.bb > 0 ? std::sqrt(h.res_rr / h.bb) : std::sqrt(h.res_rr);
    info->solve_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    info->fallback = 0;
    info->coarse_degree = 0;
  }
  return h.status;
}
