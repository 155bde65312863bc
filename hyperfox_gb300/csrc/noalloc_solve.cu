// CG solve of a small trace system that allocates no device memory.
//
// Some callers cannot call cudaMalloc: code inside a framework whose caching
// allocator owns all device memory (a raw cudaMalloc would fragment its pool
// or break its memory budget), and real-time loops that cannot take the
// latency or the possible failure of an allocation in the middle of a step.
// They own their device buffers and hand this entry point the system and the
// solution buffer; the solver's own working memory (the CG vectors, the
// block-Jacobi inverses, the reduction partials and the solver state) lives in
// one file-scope __device__ array of fixed size, resident on every GPU that
// loads the library until the process exits.
//
// The computation is the FP64 CG + per-face block-Jacobi solve of hfx_solve
// (HFX_KSP_CG, HFX_PC_BLOCK_JACOBI): the Dirichlet rows are eliminated
// symmetrically and the interior block negated, and the result is the
// solution of the stored system. CG needs a symmetric system: the entry point
// measures the symmetry of the interior block first and refuses a
// non-symmetric one (HFX_ERR_ARG), as hfx_solve refuses CG there. A face
// whose block row holds no diagonal block is refused the same way. Limits: at
// most HFX_NOALLOC_MAX_DOFS trace DOFs and HFX_NOALLOC_MAX_NF nodes per face.
//
// The host drives the iteration: it synchronises the caller's stream and reads
// the solver state between batches of iterations, and returns after the solve.
//
// The first call on a device, with that device current, looks up the device
// address of the scratch array (cudaGetSymbolAddress; the array's name in host
// code is only a host-side stand-in) and keeps it for later calls: make that
// first call before any stream capture.
//
// Every call shares the scratch array and leaves the last call's contents in
// it; the entry point clears what must start at zero itself (a one-thread
// kernel resets the solver state). Calls that overlap on the GPU (two streams,
// two host threads) race on the scratch and must be serialised by the caller.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
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
// scratch layout (doubles): bS, r, z, p, q | inverse face blocks | partials | state |
// pattern check words (max |A - A^T| and max |A| of the interior block as the bit patterns
// of non-negative doubles, which order as the doubles do; a bad-pattern flag)
constexpr int64_t kOffPc = 5 * kMaxDofs;
constexpr int64_t kOffPart = kOffPc + kMaxDofs * kMaxNF;
constexpr int64_t kOffState = kOffPart + 3 * kMaxBlocks;
constexpr int64_t kOffCheck = kOffState + kStateDoubles;
constexpr int64_t kScratchDoubles = kOffCheck + 8;
// relative asymmetry above which CG is refused (a symmetric HDG trace system is
// symmetric to the rounding of its element matrices, about 1e-15)
constexpr double kSymTol = 1e-10;

static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

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

__device__ inline void max_bits(unsigned long long* w, double v) {
  atomicMax(w, (unsigned long long)__double_as_longlong(fabs(v)));
}

// clears the solver state and the pattern-check words the previous call left behind
__global__ void nk_reset(double* scr, int maxits) {
  if (threadIdx.x != 0) return;
  CgState* st = (CgState*)(scr + kOffState);
  CgState init{};
  init.maxits = maxits;
  *st = init;
  unsigned long long* chk = (unsigned long long*)(scr + kOffCheck);
  for (int k = 0; k < 3; ++k) chk[k] = 0ull;
}

// b' (Dirichlet lift, sign flip), inverse diagonal face blocks, x0 = [0, g],
// r0 = b' - A' x0, z0 = M^{-1} r0, p0 = z0; sums r.z, r.r, ||b||^2. Also
// measures the interior block's asymmetry (each interior block (f, g) against
// the transpose of block (g, f)) and flags a row without its diagonal block or
// a block without its transposed partner.
__global__ void __launch_bounds__(kThreads) nk_start(NoallocSys A, double* scr, double* x) {
  const int NF = A.NF;
  double *bS = scr, *r = scr + kMaxDofs, *z = scr + 2 * kMaxDofs, *p = scr + 3 * kMaxDofs;
  double* pc = scr + kOffPc;
  CgState* st = (CgState*)(scr + kOffState);
  unsigned long long* chk = (unsigned long long*)(scr + kOffCheck);
  double rz = 0.0, rr = 0.0, bb = 0.0, asym = 0.0, amax = 0.0;
  bool bad = false;
  for (int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; f < A.nFaces; f += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b0 = A.browptr[f];
    const int nb = (int)(A.browptr[f + 1] - b0), npos = nb * NF;
    const bool rb = A.isBnd[f];
    double B[kMaxNF][kMaxNF], Bi[kMaxNF][kMaxNF];
    int kd = -1;
    bool inRange = true;
    for (int k = 0; k < nb; ++k) {
      const int g = A.bcol[b0 + k];
      if (g == (int)f) kd = k;
      if (g < 0 || g >= A.nFaces) inRange = false;
    }
    if (kd < 0 || !inRange) {  // malformed pattern: no diagonal block, or a column outside the system
      bad = true;
      continue;
    }
    if (!rb) {
      for (int k = 0; k < nb; ++k) {
        const int g = A.bcol[b0 + k];
        if (A.isBnd[g]) continue;
        const int64_t c0 = A.browptr[g];
        const int nbg = (int)(A.browptr[g + 1] - c0), nposg = nbg * NF;
        int kt = -1;
        for (int k2 = 0; k2 < nbg; ++k2)
          if (A.bcol[c0 + k2] == (int)f) kt = k2;
        if (kt < 0) {
          bad = true;
          continue;
        }
        for (int a = 0; a < NF; ++a)
          for (int b = 0; b < NF; ++b) {
            const double v = A.val[b0 * NF * NF + (int64_t)a * npos + k * NF + b];
            const double vt = A.val[c0 * NF * NF + (int64_t)b * nposg + kt * NF + a];
            asym = fmax(asym, fabs(v - vt));
            amax = fmax(amax, fabs(v));
          }
      }
    }
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
  if (asym > 0.0) max_bits(&chk[0], asym);
  if (amax > 0.0) max_bits(&chk[1], amax);
  if (bad) atomicExch(&chk[2], 1ull);
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

template <class T>
struct Same {
  using type = T;
};

// launches through cudaLaunchKernel, whose return code belongs to this launch
// alone (cudaGetLastError would also report, and clear, an earlier error of the
// caller's)
template <class... KArgs>
cudaError_t launch(void (*kernel)(KArgs...), int grid, int block, cudaStream_t s, typename Same<KArgs>::type... args) {
  void* ptrs[] = {(void*)&args...};
  return cudaLaunchKernel((const void*)kernel, dim3(grid), dim3(block), ptrs, 0, s);
}

struct HostCheck {
  CgState st;
  unsigned long long chk[3];
};

cudaError_t read_state(HostCheck* h, const double* scr, cudaStream_t s) {
  cudaError_t e = cudaMemcpyAsync(&h->st, scr + kOffState, sizeof(CgState), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(h->chk, scr + kOffCheck, sizeof(h->chk), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return e;
}

}  // namespace
}  // namespace hfx

using namespace hfx;

extern "C" int hfx_trace_solve_noalloc(int dim, int nodesPerFace, int nFaces, const int64_t* browptr, const int* bcol,
                                       const unsigned char* isBoundary, const double* val, const double* rhs,
                                       double* x, double rtol, int maxits, void* stream, hfx_solve_info* info) {
  auto report = [&](int code, int iters, double relres, double ms) {
    if (info) {
      info->status = code;
      info->iterations = iters;
      info->refinements = 0;
      info->rel_residual = relres;
      info->solve_ms = ms;
      info->fallback = 0;
      info->coarse_degree = 0;
    }
    return code;
  };
  auto fail = [&](int code) { return report(code, 0, 0.0, 0.0); };
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
  int nsm = 0;
  if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return fail(HFX_ERR_CUDA);
  int gridF = (int)std::min<int64_t>(kMaxBlocks, std::max<int64_t>(1, ((int64_t)nFaces * 32 + kThreads - 1) / kThreads));
  int gridV = (int)std::min<int64_t>(kMaxBlocks, std::max<int64_t>(1, ((int64_t)nFaces + kThreads - 1) / kThreads));
  gridF = std::min(gridF, 4 * nsm);
  gridV = std::min(gridV, 4 * nsm);
  if (launch(nk_reset, 1, 32, s, scr, maxits) != cudaSuccess) return fail(HFX_ERR_CUDA);
  if (launch(nk_start, gridV, kThreads, s, A, scr, x) != cudaSuccess) return fail(HFX_ERR_CUDA);
  HostCheck h;
  if (read_state(&h, scr, s) != cudaSuccess) return fail(HFX_ERR_CUDA);
  double asym, amax;
  memcpy(&asym, &h.chk[0], sizeof(double));
  memcpy(&amax, &h.chk[1], sizeof(double));
  // a malformed pattern, or an interior block that is not symmetric: CG does not apply
  if (h.chk[2] != 0ull || asym > kSymTol * amax) return fail(HFX_ERR_ARG);
  const double tol2 = rtol * rtol * h.st.bb;
  if (h.st.rr > tol2) {
    while (true) {
      for (int k = 0; k < 25; ++k) {
        if (launch(nk_spmv, gridF, kThreads, s, A, scr) != cudaSuccess ||
            launch(nk_update, gridV, kThreads, s, A, scr, x, tol2) != cudaSuccess ||
            launch(nk_pupdate, gridV, kThreads, s, A, scr) != cudaSuccess)
          return fail(HFX_ERR_CUDA);
      }
      if (read_state(&h, scr, s) != cudaSuccess) return fail(HFX_ERR_CUDA);
      if (h.st.done) break;
    }
  }
  if (launch(nk_residual, gridF, kThreads, s, A, (double*)scr, (const double*)x) != cudaSuccess)
    return fail(HFX_ERR_CUDA);
  if (read_state(&h, scr, s) != cudaSuccess) return fail(HFX_ERR_CUDA);
  const double relres = h.st.bb > 0 ? std::sqrt(h.st.res_rr / h.st.bb) : std::sqrt(h.st.res_rr);
  const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return report(h.st.status, h.st.iters, relres, ms);
}
