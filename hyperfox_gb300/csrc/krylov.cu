// Krylov solve of the condensed trace system on the device (replaces
// PetscInterface::solve / KSPSolve, PetscInterface.cpp:222-247).
//
// HyperFox's trace system has identity rows for Dirichlet DOFs with their
// columns left in place (HDGSolver.cpp:493-501), so it is not symmetric; its
// interior block is symmetric negative definite. The solver works on the
// equivalent SPD system
//     A' = [ -A_II  0 ]   b' = [ -(b_I - A_ID g) ]
//          [  0     I ]        [        g        ]
// whose solution is the reference system's solution. The FP64 operator is
// applied from the reference values on the fly (face-level masks), so no
// second FP64 copy of the matrix is stored; the mixed-precision path keeps an
// FP32 copy of A' for the inner solves and refines in FP64 against A'.
//
// Values are stored per face block-row, block by block in the sorted column
// order, each NF x NF block column-major (entry (a, b) of block k at
// k*NF*NF + b*NF + a). hfx_get_csr converts to PETSc's row-major AIJ order.
//
// CG per iteration is two kernels:
//   K1: p = z + beta*p_old (computed on the fly for every gathered entry),
//       q = A' p, partial p.q, and in the last block alpha = rz / p.q;
//   K2: x += alpha p, r -= alpha q, z = M^{-1} r, partial r.z and r.r, and in
//       the last block beta, the convergence test and the iteration count.
// Reductions are deterministic: per-block partials in fixed order, summed by
// the last block to finish (atomic ticket, no spin-waits). Once converged (or
// broken down) every later kernel returns at entry, so the host may queue
// many iterations between checks.
#include <algorithm>
#include <climits>
#include <type_traits>
#include <cmath>
#include <cstdio>
#include <vector>

#include "hdg_mixed.h"
#include "hfx_device.h"
#include "krylov.h"

namespace hfx {
namespace {

constexpr int kThreads = 256;

template <typename T>
__device__ __forceinline__ T fma_t(T a, T b, T c);
template <>
__device__ __forceinline__ double fma_t<double>(double a, double b, double c) { return fma(a, b, c); }
template <>
__device__ __forceinline__ float fma_t<float>(float a, float b, float c) { return fmaf(a, b, c); }

// Block-sum then last-block-done total of one or two values; the block that
// takes the last ticket writes the totals (fixed summation order).
template <int NV>
__device__ bool block_reduce_last(double (&v)[NV], double* partials, unsigned* ticket, double (&tot)[NV]) {
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
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[k][w];
      partials[(size_t)k * gridDim.x + blockIdx.x] = s;
    }
    __threadfence();
    unsigned t = atomicAdd(ticket, 1u);
    amLast = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!amLast) return false;
  __threadfence();
  // the last block sums all partials in block order
  for (int k = 0; k < NV; ++k) {
    double s = 0.0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x)
      s += ((volatile double*)partials)[(size_t)k * gridDim.x + b];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) red[k][wid] = s;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 0; k < NV; ++k) {
      double s = 0.0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[k][w];
      tot[k] = s;
    }
    *ticket = 0u;
  }
  return true;
}

// Thread-per-row mapping: the NF threads of a face slot each own one scalar
// row; a warp holds FPW = 32/NF faces. Values are stored block by block in CSR
// order, each NF x NF block column-major, so for a fixed column position the
// NF threads of a face read NF consecutive values, and each thread computes
// its whole row: one FMA per stored value and no cross-lane reductions (the
// reductions' adds, not the FMAs, bounded the FP64 pipe otherwise).
template <int NF, int NBMAX>
struct RowCfg {
  static constexpr int FPW = 32 / NF;
  static constexpr int NPOS = NBMAX * NF;
};

#define HFX_FACE_SLOTS(NF)                                                                     \
  constexpr int FPW = RowCfg<NF, NBMAX>::FPW;                                                  \
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;                                  \
  const int slot = lane / NF, a = lane % NF;                                                   \
  const bool laneUsed = slot < FPW;                                                            \
  const int64_t faceStride = (int64_t)gridDim.x * (kThreads / 32) * FPW;

// Gather x for the face: thread a loads column a of every neighbour block.
template <typename T, int NF, int NBMAX, bool MASKED, bool PUPD>
__device__ __forceinline__ void gather_x(const TraceView& A, int64_t b0, int nb, bool rowBnd, int a, T beta,
                                         const T* __restrict__ z, const T* __restrict__ pold, T* xs) {
  for (int k = 0; k < nb; ++k) {
    int g = A.bcol[b0 + k];
    int64_t j = (int64_t)g * NF + a;
    T v = PUPD ? fma_t<T>(beta, pold[j], z[j]) : z[j];
    if (MASKED && (rowBnd || A.isBnd[g])) v = T(0);
    xs[k * NF + a] = v;
  }
}

// gather_x from the fixed-width rows: the (block column, block location) pairs of the face
// come from one row of the ELL table, so the x loads need no row pointer first (the
// residual replacement's value loads still take the row pointer, in parallel).
template <typename T, int NF, int NBMAX>
__device__ __forceinline__ void gather_x_ell(const TraceView& A, int64_t f, bool rowBnd, int a,
                                             const T* __restrict__ x, T* xs) {
  int2 e2[NBMAX];
#pragma unroll
  for (int k = 0; k < NBMAX; ++k) e2[k] = __ldg(A.ell + f * NBMAX + k);
#pragma unroll
  for (int k = 0; k < NBMAX; ++k) {
    if (e2[k].y == INT_MIN) continue;
    const int g = e2[k].x;
    T v = x[(int64_t)g * NF + a];
    if (rowBnd || A.isBnd[g]) v = T(0);
    xs[k * NF + a] = v;
  }
}

// One row of the face block-row: sum over the nb neighbour blocks.
template <typename T, int NF>
__device__ __forceinline__ T row_dot(const T* __restrict__ val, int64_t b0, int nb, int a, const T* xs) {
  const T* base = val + b0 * NF * NF + a;
  T acc = T(0);
  for (int k = 0; k < nb; ++k) {
    const T* blk = base + (int64_t)k * NF * NF;
#pragma unroll
    for (int b = 0; b < NF; ++b) acc = fma_t<T>(__ldg(blk + b * NF), xs[k * NF + b], acc);
  }
  return acc;
}

// Layout of one NF x NF block of the FP32 half storage. NF even and at least 8: 2 x 2 tiles
// (rows 2i, 2i+1 by columns 2j, 2j+1, row-major inside the 16-byte tile), tiles in
// column-major order; otherwise plain column-major. With tiles a lane's row of a block
// (the stored orientation) is NF/2 8-byte pairs from NF/2 consecutive tiles, the lanes of
// a face reading 8*NF contiguous bytes per instruction, and a lane's column (the mirrored
// orientation) NF/2 tiles read whole, of which it keeps one column; column-major needs NF
// scalar loads for a row and NF/2 pairs at a 4*NF-byte lane stride for a column. Measured
// (launch tuner, 40^3x6 p=3, NF = 10): the bulk-copy kernel 0.294 ms per launch with tiles
// against 0.318 ms column-major, the load-based kernels slower with tiles (0.355 against
// 0.319 ms for paired loads); at NF = 6 (60^3x6 p=2) every kernel was slower with tiles
// (best 0.58 against 0.495 ms), hence tiles only for NF >= 8. The element order of a
// block's products does not change.
template <int NF>
__host__ __device__ constexpr bool tiled_blocks() {
  return NF >= 8 && NF % 2 == 0;
}
template <int NF>
__host__ __device__ __forceinline__ int hblk(int r, int c) {
  if constexpr (tiled_blocks<NF>())
    return 4 * ((r >> 1) + (NF / 2) * (c >> 1)) + 2 * (r & 1) + (c & 1);
  else
    return r + c * NF;
}
// v[b] = S(a, b): row a (GLOBAL: read-only global loads, else generic, e.g. shared memory)
template <int NF, bool GLOBAL>
__device__ __forceinline__ void blk_row(const float* blk, int a, float (&v)[NF]) {
  if constexpr (tiled_blocks<NF>()) {
#pragma unroll
    for (int j = 0; j < NF / 2; ++j) {
      const float2* p = reinterpret_cast<const float2*>(blk + 4 * ((a >> 1) + (NF / 2) * j) + 2 * (a & 1));
      const float2 w = GLOBAL ? __ldg(p) : *p;
      v[2 * j] = w.x;
      v[2 * j + 1] = w.y;
    }
  } else {
#pragma unroll
    for (int b = 0; b < NF; ++b) v[b] = GLOBAL ? __ldg(blk + b * NF + a) : blk[b * NF + a];
  }
}
// v[b] = S(b, a): column a
template <int NF, bool GLOBAL>
__device__ __forceinline__ void blk_col(const float* blk, int a, float (&v)[NF]) {
  if constexpr (tiled_blocks<NF>()) {
    const bool odd = a & 1;
#pragma unroll
    for (int i = 0; i < NF / 2; ++i) {
      const float4* p = reinterpret_cast<const float4*>(blk + 4 * (i + (NF / 2) * (a >> 1)));
      const float4 t = GLOBAL ? __ldg(p) : *p;
      v[2 * i] = odd ? t.y : t.x;
      v[2 * i + 1] = odd ? t.w : t.z;
    }
  } else if constexpr (NF % 2 == 0) {
    // column-major: the lane's column is NF consecutive values, loaded as 8-byte pairs (the
    // block starts 16-byte aligned, the column 8-byte aligned)
#pragma unroll
    for (int j = 0; j < NF / 2; ++j) {
      const float2* p = reinterpret_cast<const float2*>(blk + a * NF + 2 * j);
      const float2 w = GLOBAL ? __ldg(p) : *p;
      v[2 * j] = w.x;
      v[2 * j + 1] = w.y;
    }
  } else {
#pragma unroll
    for (int b = 0; b < NF; ++b) v[b] = GLOBAL ? __ldg(blk + a * NF + b) : blk[a * NF + b];
  }
}

// Row of the face block-row from the symmetric half storage: stored blocks are
// read by column (stride NF), mirrored ones by row (stride 1, the 400-byte block
// comes through L1 once). All block indices are loaded first and every block's
// NF values are issued before use, so the loads of a row are in flight together.
template <int NF, int NBMAX>
__device__ __forceinline__ float row_dot_half(const float* __restrict__ valh, const int* __restrict__ hidx, int64_t b0,
                                              int nb, int a, const float* xs) {
  int hh[NBMAX];
#pragma unroll
  for (int k = 0; k < NBMAX; ++k) hh[k] = k < nb ? __ldg(hidx + b0 + k) : 0;
  float acc = 0.f;
#pragma unroll
  for (int k = 0; k < NBMAX; ++k) {
    if (k < nb) {
      const int h = hh[k];
      float v[NF];
      if (h >= 0)
        blk_row<NF, true>(valh + (int64_t)h * NF * NF, a, v);
      else
        blk_col<NF, true>(valh + (int64_t)(-h - 1) * NF * NF, a, v);
#pragma unroll
      for (int b = 0; b < NF; ++b) acc = fmaf(v[b], xs[k * NF + b], acc);
    }
  }
  return acc;
}

// K1 of CG on the FP32 half storage (mixed precision, symmetric A').
template <int NF, int NBMAX>
__global__ void __launch_bounds__(kThreads) cg_spmv_half(TraceView A, const float* __restrict__ valh,
                                                         const float* __restrict__ z, const float* __restrict__ pold,
                                                         float* __restrict__ pnew, float* __restrict__ q, CgState* st,
                                                         double* partials, int first) {
  __shared__ float xsh[kThreads / 32][RowCfg<NF, NBMAX>::FPW][RowCfg<NF, NBMAX>::NPOS];
  if (st->done) return;
  const float beta = first ? 0.f : (float)st->beta;
  HFX_FACE_SLOTS(NF)
  double pq = 0.0;
  for (int64_t fb = ((int64_t)blockIdx.x * (kThreads / 32) + warp) * FPW; fb < A.nFaces; fb += faceStride) {
    const int64_t f = fb + slot;
    const bool act = laneUsed && f < A.nFaces;
    const int64_t b0 = act ? A.browptr[f] : 0;
    const int nb = act ? (int)(A.browptr[f + 1] - b0) : 0;
    float* xs = laneUsed ? xsh[warp][slot] : nullptr;
    if (act) gather_x<float, NF, NBMAX, false, true>(A, b0, nb, false, a, beta, z, pold, xs);
    __syncwarp();
    if (act) {
      const float y = row_dot_half<NF, NBMAX>(valh, A.hidx, b0, nb, a, xs);
      const int64_t i = f * NF + a;
      const float pi = fmaf(beta, pold[i], z[i]);
      pnew[i] = pi;
      q[i] = y;
      pq += (double)pi * (double)y;
    }
    __syncwarp();
  }
  double v[1] = {pq}, tot[1];
  if (block_reduce_last<1>(v, partials, &st->ticket, tot) && threadIdx.x == 0) {
    double pAp = tot[0];
    if (!(pAp > 0.0) || !isfinite(pAp)) {
      st->status = isfinite(pAp) ? 6 : 7;
      st->done = 1;
    } else {
      st->alpha = st->rz / pAp;
    }
  }
}

// cg_spmv_half over the fixed-width rows: the (block column, block location)
// pairs of a face are one 8-byte load per slot at f * NBMAX + k, so no row
// pointer has to arrive before the gather and the value loads can start; the
// products are the same, in the same order. At most six 256-thread blocks per
// SM keep the register count of the row-pointer version (five with whole-tile loads,
// whose values in flight need more registers).
//
// PAIRED: the block values are loaded as whole pairs and tiles of the block layout (hblk:
// with tiles NF/2 8-byte pairs for a row and NF/2 16-byte tiles for a column; column-major
// with NF even, NF/2 pairs for a column); otherwise one scalar load per value.
// XV: the gathered x of each block is stored with a row of NF rounded up to a multiple of
// four and read back as float4s: a quarter of the shared-memory wavefronts of the scalar
// reads (those wavefronts share the L1 data pipe with the value loads, which bound the
// kernel). The products and their order do not change.
template <int NF, int NBMAX, bool PAIRED = false, bool XV = false>
__global__ void __launch_bounds__(kThreads, PAIRED && tiled_blocks<NF>() ? 5 : 6) cg_spmv_half_ell(TraceView A, const float* __restrict__ valh,
                                                                const float* __restrict__ z,
                                                                const float* __restrict__ pold,
                                                                float* __restrict__ pnew, float* __restrict__ q,
                                                                CgState* st, double* partials, int first) {
  constexpr int XR = XV ? (NF + 3) / 4 * 4 : NF;  // stride of a block's gathered x
  __shared__ __align__(16) float xsh[kThreads / 32][RowCfg<NF, NBMAX>::FPW][NBMAX * XR];
  if (st->done) return;
  const float beta = first ? 0.f : (float)st->beta;
  HFX_FACE_SLOTS(NF)
  double pq = 0.0;
  for (int64_t fb = ((int64_t)blockIdx.x * (kThreads / 32) + warp) * FPW; fb < A.nFaces; fb += faceStride) {
    const int64_t f = fb + slot;
    const bool act = laneUsed && f < A.nFaces;
    float* xs = laneUsed ? xsh[warp][slot] : nullptr;
    int hh[NBMAX];
#pragma unroll
    for (int k = 0; k < NBMAX; ++k) hh[k] = INT_MIN;
    if (act) {
      const int2* row = A.ell + f * NBMAX;
      for (int k = 0; k < NBMAX; ++k) {
        const int2 e2 = __ldg(row + k);
        hh[k] = e2.y;
        if (e2.y != INT_MIN) {
          const int64_t j = (int64_t)e2.x * NF + a;
          xs[k * XR + a] = fmaf(beta, pold[j], z[j]);
        }
      }
    }
    __syncwarp();
    if (act) {
      float acc = 0.f;
#pragma unroll
      for (int k = 0; k < NBMAX; ++k) {
        const int h = hh[k];
        if (h != INT_MIN) {
          const float* blk = valh + (int64_t)(h >= 0 ? h : -h - 1) * NF * NF;
          float v[NF];
          if (PAIRED) {
            if (h >= 0)
              blk_row<NF, true>(blk, a, v);
            else
              blk_col<NF, true>(blk, a, v);
          } else {
#pragma unroll
            for (int b = 0; b < NF; ++b) v[b] = __ldg(blk + (h >= 0 ? hblk<NF>(a, b) : hblk<NF>(b, a)));
          }
          if (XV) {
            float xv[XR];
            const float4* x4 = reinterpret_cast<const float4*>(xs + k * XR);
#pragma unroll
            for (int c = 0; c < XR / 4; ++c) {
              const float4 w = x4[c];
              xv[4 * c] = w.x;
              xv[4 * c + 1] = w.y;
              xv[4 * c + 2] = w.z;
              xv[4 * c + 3] = w.w;
            }
#pragma unroll
            for (int b = 0; b < NF; ++b) acc = fmaf(v[b], xv[b], acc);
          } else {
#pragma unroll
            for (int b = 0; b < NF; ++b) acc = fmaf(v[b], xs[k * XR + b], acc);
          }
        }
      }
      const int64_t i = f * NF + a;
      const float pi = fmaf(beta, pold[i], z[i]);
      pnew[i] = pi;
      q[i] = acc;
      pq += (double)pi * (double)acc;
    }
    __syncwarp();
  }
  double v[1] = {pq}, tot[1];
  if (block_reduce_last<1>(v, partials, &st->ticket, tot) && threadIdx.x == 0) {
    double pAp = tot[0];
    if (!(pAp > 0.0) || !isfinite(pAp)) {
      st->status = isfinite(pAp) ? 6 : 7;
      st->done = 1;
    } else {
      st->alpha = st->rz / pAp;
    }
  }
}

// The same K1 with the blocks staged in shared memory by the copy engine. The values of a
// face group (FPW faces, NBMAX blocks each, NF x NF floats per block) are fetched by
// cp.async.bulk, one 16-byte-aligned copy per block, completing on a per-warp mbarrier.
// STAGES = 2: each warp keeps two groups in flight (while it computes one group from
// shared memory the next group's blocks are being copied), four warps per CTA; STAGES = 1:
// one group per warp, eight warps per CTA, the other warps cover the copy latency (both
// fit three CTAs per SM at NF = 10). The value stream then never goes
// through the L1 tag stage (whose sector lookups, two to three per value byte for the
// transposed reads, bound the load-based kernels), and the bytes in flight do not depend
// on registers. The x gather, the products and their order are those of
// cg_spmv_half_ell, so q is the same. Needs NF even (16-byte block size).
// Every wait on an mbarrier is bounded: a wait that runs out waits (bounded) for the
// warp's other copies, sets status HFX_ERR_CUDA and stops the solve.
constexpr int kTmaStages = 1;
constexpr uint32_t kTmaWait = 1u << 22;  // mbarrier polls before a wait is abandoned

template <int NF, int NBMAX, int STAGES = kTmaStages>
struct TmaCfg {
  static constexpr int WARPS = STAGES == 2 ? 4 : 8;
  static constexpr int THREADS = 32 * WARPS;
  static constexpr int FPW = 32 / NF;
  static constexpr int NBLK = FPW * NBMAX;     // blocks staged per face group
  static constexpr int BLK = NF * NF;          // floats per block
  static constexpr int NFP = (NF + 3) / 4 * 4;  // gathered x per block, padded for float4 reads
  static constexpr int BUF = NBLK * BLK;       // floats per stage
  static constexpr int XS = FPW * NBMAX * NFP;
  static constexpr int NCH = (NBLK + 31) / 32;  // copy rounds of 32 lanes
  static constexpr int WARP_BYTES = (STAGES * BUF + XS) * 4 + 16;
  static constexpr int CTA_BYTES = WARP_BYTES * WARPS;
};

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// all lanes poll; the answer is made warp-uniform (a lane that gave up fails the warp)
__device__ __forceinline__ bool tma_wait(uint32_t bar, uint32_t parity) {
  uint32_t done = 0;
  for (uint32_t it = 0; it < kTmaWait && !done; ++it)
    asm volatile("{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
                 : "=r"(done)
                 : "r"(bar), "r"(parity)
                 : "memory");
  return __all_sync(0xffffffffu, done != 0);
}

// Copies of the blocks of face group g into buf: lane t takes block t (face t / NBMAX of the
// group, slot t % NBMAX); the byte count is announced on the mbarrier before any copy starts.
template <int NF, int NBMAX>
__device__ __forceinline__ void tma_issue_group(const TraceView& A, const float* __restrict__ valh, int64_t g,
                                                float* buf, uint32_t bar, int lane) {
  using C = TmaCfg<NF, NBMAX>;
  int hs[C::NCH];
  uint32_t nblk = 0;
#pragma unroll
  for (int c = 0; c < C::NCH; ++c) {
    const int t = c * 32 + lane;
    int h = INT_MIN;
    if (t < C::NBLK) {
      const int64_t f = g * C::FPW + t / NBMAX;
      if (f < A.nFaces) h = __ldg(A.ell + f * NBMAX + t % NBMAX).y;
    }
    hs[c] = h;
    nblk += __popc(__ballot_sync(0xffffffffu, h != INT_MIN));
  }
  if (lane == 0)
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(nblk * C::BLK * 4u)
                 : "memory");
  __syncwarp();
#pragma unroll
  for (int c = 0; c < C::NCH; ++c) {
    const int h = hs[c];
    if (h != INT_MIN) {
      const int t = c * 32 + lane;
      const float* src = valh + (int64_t)(h >= 0 ? h : -h - 1) * C::BLK;
      asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                       smem_addr(buf + t * C::BLK)),
                   "l"(src), "r"((uint32_t)(C::BLK * 4)), "r"(bar)
                   : "memory");
    }
  }
}

template <int NF, int NBMAX, int STAGES = kTmaStages>
__global__ void __launch_bounds__(TmaCfg<NF, NBMAX, STAGES>::THREADS)
    cg_spmv_half_tma(TraceView A, const float* __restrict__ valh,
                                                                const float* __restrict__ z,
                                                                const float* __restrict__ pold,
                                                                float* __restrict__ pnew, float* __restrict__ q,
                                                                CgState* st, double* partials, int first) {
  static_assert(NF % 2 == 0, "blocks of 16-byte multiples only");
  using C = TmaCfg<NF, NBMAX, STAGES>;
  constexpr int FPW = C::FPW, NFP = C::NFP;
  extern __shared__ __align__(16) unsigned char tma_smem[];
  if (st->done) return;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float* buf0 = reinterpret_cast<float*>(tma_smem + warp * C::WARP_BYTES);
  float* buf1 = buf0 + (STAGES == 2 ? C::BUF : 0);
  float* xsw = buf0 + STAGES * C::BUF;
  uint64_t* bars = reinterpret_cast<uint64_t*>(xsw + C::XS);
  const uint32_t bar0 = smem_addr(&bars[0]), bar1 = smem_addr(&bars[1]);
  if (lane == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar0));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar1));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncwarp();
  const float beta = first ? 0.f : (float)st->beta;
  const int slot = lane / NF, a = lane % NF;
  const bool laneUsed = slot < FPW;
  float* xs = xsw + (laneUsed ? slot : 0) * NBMAX * NFP;
  const int64_t nGroups = ((int64_t)A.nFaces + FPW - 1) / FPW;
  const int64_t warps = (int64_t)gridDim.x * C::WARPS;
  int64_t g = (int64_t)blockIdx.x * C::WARPS + warp;
  double pq = 0.0;
  bool bad = false;
  uint32_t u = 0;
  if (STAGES == 2 && g < nGroups) tma_issue_group<NF, NBMAX>(A, valh, g, buf0, bar0, lane);
  for (; g < nGroups; g += warps, ++u) {
    const int stg = STAGES == 2 ? (int)(u & 1) : 0;
    const float* buf = stg ? buf1 : buf0;
    const uint32_t bar = stg ? bar1 : bar0;
    // the buffer about to be filled was last read by an earlier group (generic loads,
    // finished at its __syncwarp): order those reads before the copy engine's writes
    if (STAGES == 1) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      tma_issue_group<NF, NBMAX>(A, valh, g, buf0, bar0, lane);
    } else if (g + warps < nGroups) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      tma_issue_group<NF, NBMAX>(A, valh, g + warps, stg ? buf0 : buf1, stg ? bar0 : bar1, lane);
    }
    const int64_t f = g * FPW + slot;
    const bool act = laneUsed && f < A.nFaces;
    int hh[NBMAX];
#pragma unroll
    for (int k = 0; k < NBMAX; ++k) hh[k] = INT_MIN;
    if (act) {
      const int2* row = A.ell + f * NBMAX;
#pragma unroll
      for (int k = 0; k < NBMAX; ++k) {
        const int2 e2 = __ldg(row + k);
        hh[k] = e2.y;
        if (e2.y != INT_MIN) {
          const int64_t j = (int64_t)e2.x * NF + a;
          xs[k * NFP + a] = fmaf(beta, pold[j], z[j]);
        }
      }
    }
    __syncwarp();
    if (!tma_wait(bar, STAGES == 2 ? (u >> 1) & 1u : u & 1u)) {
      bad = true;
      if (STAGES == 2 && g + warps < nGroups) tma_wait(stg ? bar0 : bar1, ((u + 1) >> 1) & 1u);
      break;
    }
    if (act) {
      float acc = 0.f;
#pragma unroll
      for (int k = 0; k < NBMAX; ++k) {
        const int h = hh[k];
        if (h != INT_MIN) {
          const float* blk = buf + (slot * NBMAX + k) * C::BLK;
          float v[NF], xv[NFP];
          if (h >= 0)
            blk_row<NF, false>(blk, a, v);
          else
            blk_col<NF, false>(blk, a, v);
          const float4* x4 = reinterpret_cast<const float4*>(xs + k * NFP);
#pragma unroll
          for (int c = 0; c < NFP / 4; ++c) {
            const float4 w = x4[c];
            xv[4 * c] = w.x;
            xv[4 * c + 1] = w.y;
            xv[4 * c + 2] = w.z;
            xv[4 * c + 3] = w.w;
          }
#pragma unroll
          for (int b = 0; b < NF; ++b) acc = fmaf(v[b], xv[b], acc);
        }
      }
      const int64_t i = f * NF + a;
      const float pi = fmaf(beta, pold[i], z[i]);
      pnew[i] = pi;
      q[i] = acc;
      pq += (double)pi * (double)acc;
    }
    __syncwarp();
  }
  // (done is set by the last block: a block that has not started yet must still take its ticket)
  if (bad && lane == 0) st->status = 3;  // HFX_ERR_CUDA: a block copy did not arrive
  double v[1] = {pq}, tot[1];
  if (block_reduce_last<1>(v, partials, &st->ticket, tot) && threadIdx.x == 0) {
    double pAp = tot[0];
    if (st->status != 0) {
      st->done = 1;
    } else if (!(pAp > 0.0) || !isfinite(pAp)) {
      st->status = isfinite(pAp) ? 6 : 7;
      st->done = 1;
    } else {
      st->alpha = st->rz / pAp;
    }
  }
}

// Grid of cg_spmv_half_tma (every CTA resident, no more than the face groups need); 0 where
// the kernel does not apply (NF odd) or cannot be resident.
template <int NF, int NBMAX>
int tma_grid(int64_t nFaces) {
  if constexpr (NF % 2 != 0) {
    return 0;
  } else {
    using C = TmaCfg<NF, NBMAX>;
    int dev = 0, nsm = 0, perSM = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (cudaFuncSetAttribute(cg_spmv_half_tma<NF, NBMAX>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             C::CTA_BYTES) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, cg_spmv_half_tma<NF, NBMAX>, C::THREADS,
                                                      C::CTA_BYTES) != cudaSuccess ||
        perSM < 1) {
      cudaGetLastError();
      return 0;
    }
    const int64_t groups = (nFaces + C::FPW - 1) / C::FPW;
    const int64_t need = (groups + C::WARPS - 1) / C::WARPS;
    return (int)std::max<int64_t>(1, std::min<int64_t>(need, (int64_t)nsm * perSM));
  }
}

template <int NF, int NBMAX>
void launch_spmv_tma(int grid, cudaStream_t s, const TraceView& A, const float* valh, const float* z,
                     const float* pold, float* pnew, float* q, CgState* st, double* partials, int first) {
  if constexpr (NF % 2 == 0)
    cg_spmv_half_tma<NF, NBMAX><<<grid, TmaCfg<NF, NBMAX>::THREADS, TmaCfg<NF, NBMAX>::CTA_BYTES, s>>>(
        A, valh, z, pold, pnew, q, st, partials, first);
}

// K1 of CG (see the file comment).
template <typename T, int NF, int NBMAX, bool MASKED>
__global__ void __launch_bounds__(kThreads) cg_spmv(TraceView A, const T* __restrict__ val,
                                                    const T* __restrict__ z, const T* __restrict__ pold,
                                                    T* __restrict__ pnew, T* __restrict__ q, CgState* st,
                                                    double* partials, int first) {
  __shared__ T xsh[kThreads / 32][RowCfg<NF, NBMAX>::FPW][RowCfg<NF, NBMAX>::NPOS];
  if (st->done) return;
  const T beta = first ? T(0) : (T)st->beta;
  HFX_FACE_SLOTS(NF)
  double pq = 0.0;
  for (int64_t fb = ((int64_t)blockIdx.x * (kThreads / 32) + warp) * FPW; fb < A.nFaces; fb += faceStride) {
    const int64_t f = fb + slot;
    const bool act = laneUsed && f < A.nFaces;
    const int64_t b0 = act ? A.browptr[f] : 0;
    const int nb = act ? (int)(A.browptr[f + 1] - b0) : 0;
    const bool rowBnd = MASKED && act && A.isBnd[f];
    T* xs = laneUsed ? xsh[warp][slot] : nullptr;
    if (act) gather_x<T, NF, NBMAX, MASKED, true>(A, b0, nb, rowBnd, a, beta, z, pold, xs);
    __syncwarp();
    if (act) {
      T y = row_dot<T, NF>(val, b0, nb, a, xs);
      int64_t i = f * NF + a;
      T pi = fma_t<T>(beta, pold[i], z[i]);
      T yi = MASKED ? (rowBnd ? pi : -y) : y;
      pnew[i] = pi;
      q[i] = yi;
      pq += (double)pi * (double)yi;
    }
    __syncwarp();
  }
  double v[1] = {pq}, tot[1];
  if (block_reduce_last<1>(v, partials, &st->ticket, tot) && threadIdx.x == 0) {
    double pAp = tot[0];
    if (!(pAp > 0.0) || !isfinite(pAp)) {
      st->status = isfinite(pAp) ? 6 : 7;  // HFX_ERR_BREAKDOWN / HFX_ERR_NAN
      st->done = 1;
    } else {
      st->alpha = st->rz / pAp;
    }
  }
}

// K2 of CG. PC: 0 none, 1 Jacobi (pc = inverse diagonal), 2 block Jacobi
// (pc = inverse face blocks, column-major NF x NF). Thread per row, the NF
// threads of a face exchange their residual rows through shared memory.
template <typename T, int NF, int PC>
__global__ void __launch_bounds__(kThreads) cg_update(int64_t nFaces, T* __restrict__ x, T* __restrict__ r,
                                                      T* __restrict__ z, const T* __restrict__ p,
                                                      const T* __restrict__ q, const T* __restrict__ pc,
                                                      CgState* st, double* partials, double tol2) {
  constexpr int FPW = 32 / NF;
  __shared__ T rsh[kThreads / 32][FPW][NF];
  if (st->done) return;
  const T alpha = (T)st->alpha;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int slot = lane / NF, a = lane % NF;
  const bool laneUsed = slot < FPW;
  const int64_t stride = (int64_t)gridDim.x * (kThreads / 32) * FPW;
  double rz = 0.0, rr = 0.0;
  for (int64_t fb = ((int64_t)blockIdx.x * (kThreads / 32) + warp) * FPW; fb < nFaces; fb += stride) {
    const int64_t f = fb + slot;
    const bool act = laneUsed && f < nFaces;
    T ra = T(0);
    if (act) {
      int64_t i = f * NF + a;
      x[i] = fma_t<T>(alpha, p[i], x[i]);
      ra = fma_t<T>(-alpha, q[i], r[i]);
      r[i] = ra;
      rr += (double)ra * (double)ra;
      if (PC == 2) rsh[warp][slot][a] = ra;
    }
    if (PC == 2) __syncwarp();
    if (act) {
      int64_t i = f * NF + a;
      T zi;
      if (PC == 0) zi = ra;
      else if (PC == 1) zi = pc[i] * ra;
      else {
        zi = T(0);
        const T* B = pc + f * NF * NF + a;
#pragma unroll
        for (int b = 0; b < NF; ++b) zi = fma_t<T>(B[b * NF], rsh[warp][slot][b], zi);
      }
      z[i] = zi;
      rz += (double)ra * (double)zi;
    }
    if (PC == 2) __syncwarp();
  }
  double v[2] = {rz, rr}, tot[2];
  if (block_reduce_last<2>(v, partials, &st->ticket, tot) && threadIdx.x == 0) {
    double rzn = tot[0];
    st->iters += 1;
    st->rr = tot[1];
    if (!isfinite(rzn) || !isfinite(tot[1])) {
      st->status = 7;
      st->done = 1;
    } else {
      st->beta = rzn / st->rz;
      st->rz = rzn;
      if (tot[1] <= tol2) st->done = 1;
      else if (st->iters >= st->maxits) {
        st->status = 5;  // HFX_ERR_NOT_CONVERGED
        st->done = 1;
      }
    }
  }
}

// K2 of CG with the two-level preconditioner, first half: x += alpha p,
// r -= alpha q, ||r||^2 and the convergence test. z follows in tl_apply once the
// coarse solve of the new residual is done.
template <typename T, int NF>
__global__ void __launch_bounds__(kThreads) cg_update_r(int64_t nFaces, T* __restrict__ x, T* __restrict__ r,
                                                        const T* __restrict__ p, const T* __restrict__ q,
                                                        CgState* st, double* partials, double tol2) {
  if (st->done) return;
  const T alpha = (T)st->alpha;
  const int64_t n = nFaces * NF;
  double rr = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * kThreads + threadIdx.x; i < n; i += (int64_t)gridDim.x * kThreads) {
    x[i] = fma_t<T>(alpha, p[i], x[i]);
    T ra = fma_t<T>(-alpha, q[i], r[i]);
    r[i] = ra;
    rr += (double)ra * (double)ra;
  }
  double v[1] = {rr}, tot[1];
  if (block_reduce_last<1>(v, partials, &st->ticket, tot) && threadIdx.x == 0) {
    st->iters += 1;
    st->rr = tot[0];
    if (!isfinite(tot[0])) {
      st->status = 7;
      st->done = 1;
    } else if (tot[0] <= tol2) {
      st->done = 1;
    } else if (st->iters >= st->maxits) {
      st->status = 5;
      st->done = 1;
    }
  }
}

// z = B^{-1} r + P yc (face-block Jacobi plus the prolongated coarse solution),
// r.z; init = 1 stores r.z only (start of CG), else beta = r.z / previous r.z.
template <typename T, int NF>
__global__ void __launch_bounds__(kThreads) tl_apply(int64_t nFaces, const T* __restrict__ r, T* __restrict__ z,
                                                     const T* __restrict__ pc, CoarseDev cd, CgState* st,
                                                     double* partials, int init) {
  constexpr int FPW = 32 / NF;
  __shared__ T rsh[kThreads / 32][FPW][NF];
  if (st->done) return;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int slot = lane / NF, a = lane % NF;
  const bool laneUsed = slot < FPW;
  const int64_t stride = (int64_t)gridDim.x * (kThreads / 32) * FPW;
  const int d = cd.dim;
  double rz = 0.0;
  for (int64_t fb = ((int64_t)blockIdx.x * (kThreads / 32) + warp) * FPW; fb < nFaces; fb += stride) {
    const int64_t f = fb + slot;
    const bool act = laneUsed && f < nFaces;
    T ra = T(0);
    if (act) {
      ra = r[f * NF + a];
      rsh[warp][slot][a] = ra;
    }
    __syncwarp();
    if (act) {
      T zi = T(0);
      const T* B = pc + f * NF * NF + a;
#pragma unroll
      for (int b = 0; b < NF; ++b) zi = fma_t<T>(B[b * NF], rsh[warp][slot][b], zi);
      if (!cd.isBnd[f]) {
        float s = 0.f;
        for (int k = 0; k < d; ++k) s = fmaf(cd.Wf[a * d + k], cd.yc[cd.faceV[f * d + k]], s);
        zi += (T)s;
      }
      z[f * NF + a] = zi;
      rz += (double)ra * (double)zi;
    }
    __syncwarp();
  }
  double v[1] = {rz}, tot[1];
  if (block_reduce_last<1>(v, partials, &st->ticket, tot) && threadIdx.x == 0) {
    if (!isfinite(tot[0])) {
      st->status = 7;
      st->done = 1;
    } else if (init) {
      st->rz = tot[0];
    } else {
      st->beta = tot[0] / st->rz;
      st->rz = tot[0];
    }
  }
}

// r = b' - A' x (FP64, masked reference values) and its norm; also z = M^{-1} r
// and r.z to start CG. Writes the squared norms to st (||b||^2 of the reference rhs).
template <int NF, int NBMAX, int PC>
__global__ void __launch_bounds__(kThreads) cg_start(TraceView A, const double* __restrict__ val,
                                                     const double* __restrict__ bS, const double* __restrict__ bref,
                                                     const double* __restrict__ x, double* __restrict__ r,
                                                     double* __restrict__ z, const double* __restrict__ pc, CgState* st,
                                                     double* partials) {
  __shared__ double xsh[kThreads / 32][RowCfg<NF, NBMAX>::FPW][RowCfg<NF, NBMAX>::NPOS];
  HFX_FACE_SLOTS(NF)
  double rr = 0.0, rz = 0.0, bb = 0.0;
  for (int64_t fb = ((int64_t)blockIdx.x * (kThreads / 32) + warp) * FPW; fb < A.nFaces; fb += faceStride) {
    const int64_t f = fb + slot;
    const bool act = laneUsed && f < A.nFaces;
    const int64_t b0 = act ? A.browptr[f] : 0;
    const int nb = act ? (int)(A.browptr[f + 1] - b0) : 0;
    const bool rowBnd = act && A.isBnd[f];
    double* xs = laneUsed ? xsh[warp][slot] : nullptr;
    if (act) gather_x<double, NF, NBMAX, true, false>(A, b0, nb, rowBnd, a, 0.0, x, x, xs);
    __syncwarp();
    double ra = 0.0;
    if (act) {
      double y = row_dot<double, NF>(val, b0, nb, a, xs);
      int64_t i = f * NF + a;
      double ax = rowBnd ? x[i] : -y;
      ra = bS[i] - ax;
      r[i] = ra;
      rr += ra * ra;
      bb += bref[i] * bref[i];
    }
    __syncwarp();
    // z for the face needs all NF residual rows: pass them through shared memory
    if (act) xs[a] = ra;
    __syncwarp();
    if (act) {
      int64_t i = f * NF + a;
      double zi;
      if (PC == 0) zi = ra;
      else if (PC == 1) zi = pc[i] * ra;
      else {
        zi = 0.0;
        for (int b = 0; b < NF; ++b) zi += pc[f * NF * NF + b * NF + a] * xs[b];
      }
      z[i] = zi;
      rz += ra * zi;
    }
    __syncwarp();
  }
  double v[3] = {rr, rz, bb}, tot[3];
  if (block_reduce_last<3>(v, partials, &st->ticket, tot) && threadIdx.x == 0) {
    st->rr = tot[0];
    st->rz = tot[1];
    st->bb = tot[2];
  }
}

// Residual of the reference system: res = b - A x with the stored values as
// they are (Dirichlet identity rows included); totals ||b-Ax||^2, ||b||^2.
template <int NF, int NBMAX>
__global__ void __launch_bounds__(kThreads) ref_residual(TraceView A, const double* __restrict__ val,
                                                         const double* __restrict__ b, const double* __restrict__ x,
                                                         CgState* st, double* partials) {
  __shared__ double xsh[kThreads / 32][RowCfg<NF, NBMAX>::FPW][RowCfg<NF, NBMAX>::NPOS];
  HFX_FACE_SLOTS(NF)
  double rr = 0.0, bb = 0.0;
  for (int64_t fb = ((int64_t)blockIdx.x * (kThreads / 32) + warp) * FPW; fb < A.nFaces; fb += faceStride) {
    const int64_t f = fb + slot;
    const bool act = laneUsed && f < A.nFaces;
    const int64_t b0 = act ? A.browptr[f] : 0;
    const int nb = act ? (int)(A.browptr[f + 1] - b0) : 0;
    double* xs = laneUsed ? xsh[warp][slot] : nullptr;
    if (act) gather_x<double, NF, NBMAX, false, false>(A, b0, nb, false, a, 0.0, x, x, xs);
    __syncwarp();
    if (act) {
      double ri = b[f * NF + a] - row_dot<double, NF>(val, b0, nb, a, xs);
      rr += ri * ri;
      bb += b[f * NF + a] * b[f * NF + a];
    }
    __syncwarp();
  }
  double v[2] = {rr, bb}, tot[2];
  if (block_reduce_last<2>(v, partials, &st->ticket, tot) && threadIdx.x == 0) {
    st->res_rr = tot[0];
    st->res_bb = tot[1];
  }
}

// b' and the FP32 copy of A' (optional), thread per row.
template <int NF, int NBMAX>
__global__ void __launch_bounds__(kThreads) prepare_system(TraceView A, const double* __restrict__ val,
                                                           const double* __restrict__ b, double* __restrict__ bS,
                                                           float* __restrict__ val32, float* __restrict__ val32h = nullptr) {
  HFX_FACE_SLOTS(NF)
  for (int64_t fb = ((int64_t)blockIdx.x * (kThreads / 32) + warp) * FPW; fb < A.nFaces; fb += faceStride) {
    const int64_t f = fb + slot;
    if (!(laneUsed && f < A.nFaces)) continue;
    const int64_t b0 = A.browptr[f];
    const int nb = (int)(A.browptr[f + 1] - b0);
    const bool rowBnd = A.isBnd[f];
    double lift = 0.0;
    for (int k = 0; k < nb; ++k) {
      int g = A.bcol[b0 + k];
      for (int c = 0; c < NF; ++c) {
        int64_t idx = (b0 + k) * NF * NF + (int64_t)c * NF + a;
        double v = val[idx];
        if (!rowBnd && A.isBnd[g]) lift += v * b[(int64_t)g * NF + c];
        if (val32 || val32h) {
          float w;
          if (rowBnd) w = (g == (int)f && c == a) ? 1.0f : 0.0f;
          else w = A.isBnd[g] ? 0.0f : (float)(-v);
          if (val32) val32[idx] = w;
          if (val32h) {
            const int h = A.hidx[b0 + k];
            if (h >= 0) val32h[(int64_t)h * NF * NF + hblk<NF>(a, c)] = w;
          }
        }
      }
    }
    int64_t i = f * NF + a;
    bS[i] = rowBnd ? b[i] : -(b[i] - lift);
  }
}

// Inverse diagonal / inverse diagonal face blocks of A' (FP64 and FP32 copies).
// TM: arithmetic of the inversion (float when only the FP32 copy is wanted).
// Block-Jacobi inverses of the diagonal face blocks, one face per NF lanes
// (three faces per warp at NF = 10): lane a holds row a of [B | I] in
// registers and every Gauss-Jordan step takes the pivot row from its lane by
// shuffles (SPD blocks: no pivoting). Lane a reads row a of the stored
// column-major block, coalesced with the face's other rows.
template <int NF, typename TM = double>
__global__ void __launch_bounds__(kThreads) build_precond(TraceView A, const double* __restrict__ val, int pcType,
                                                          double* pc64, float* pc32) {
  constexpr int NBMAX = 1;  // only the face slots of the row layout are used here
  HFX_FACE_SLOTS(NF)
  const int base = (laneUsed ? slot : 0) * NF;  // spare lanes follow the first face
  for (int64_t fb = ((int64_t)blockIdx.x * (kThreads / 32) + warp) * FPW; fb < A.nFaces; fb += faceStride) {
    const int64_t f = fb + slot;
    const bool act = laneUsed && f < A.nFaces;
    int64_t bd = 0;  // the diagonal block
    bool bnd = false;
    if (act) {
      const int64_t b0 = A.browptr[f];
      const int nb = (int)(A.browptr[f + 1] - b0);
      bd = b0;
      for (int k = 0; k < nb; ++k)
        if (A.bcol[b0 + k] == (int)f) bd = b0 + k;
      bnd = A.isBnd[f] != 0;
    }
    TM row[2 * NF];
#pragma unroll
    for (int b = 0; b < NF; ++b) {
      row[b] = (!act || bnd) ? TM(a == b ? 1 : 0) : -(TM)val[bd * NF * NF + (int64_t)b * NF + a];
      row[NF + b] = TM(a == b ? 1 : 0);
    }
    if (pcType == 1) {
      if (act) {
        TM d = TM(0);  // row[a] without a dynamic index (keeps row in registers)
#pragma unroll
        for (int b = 0; b < NF; ++b)
          if (b == a) d = row[b];
        const TM v = d != TM(0) ? TM(1) / d : TM(1);
        if (pc64) pc64[f * NF + a] = (double)v;
        if (pc32) pc32[f * NF + a] = (float)v;
      }
      continue;
    }
#pragma unroll
    for (int k = 0; k < NF; ++k) {
      TM piv[2 * NF];
#pragma unroll
      for (int j = 0; j < 2 * NF; ++j) piv[j] = __shfl_sync(0xffffffffu, row[j], base + k);
      const TM inv = TM(1) / piv[k];
      if (laneUsed && a == k) {
#pragma unroll
        for (int j = 0; j < 2 * NF; ++j) row[j] = piv[j] * inv;
      } else {
        const TM l = row[k] * inv;
#pragma unroll
        for (int j = 0; j < 2 * NF; ++j) row[j] -= l * piv[j];
      }
    }
    if (act)
#pragma unroll
      for (int b = 0; b < NF; ++b) {  // column-major inverse
        if (pc64) pc64[f * NF * NF + b * NF + a] = (double)row[NF + b];
        if (pc32) pc32[f * NF * NF + b * NF + a] = (float)row[NF + b];
      }
  }
}

template <int NF>
unsigned precond_grid(int64_t nFaces) {
  const int64_t perBlock = (kThreads / 32) * (32 / NF);
  int64_t g = (nFaces + perBlock - 1) / perBlock;
  if (g > 152 * 8) g = 152 * 8;
  return (unsigned)(g < 1 ? 1 : g);
}

// Reliable update of the mixed-precision CG: the true residual
// r = b' - A' x (FP64, masked reference values) replaces the FP32 recursive
// residual; writes r32 = (float) r, z32 = M^{-1} r32 and the sums ||r||^2 (FP64)
// and r32.z32 into st. The FP32 search direction is kept.
template <int NF, int NBMAX, int PC>
__global__ void __launch_bounds__(kThreads) cg_replace(TraceView A, const double* __restrict__ val,
                                                       const double* __restrict__ bS, const double* __restrict__ bref,
                                                       const double* __restrict__ x, float* __restrict__ r32,
                                                       float* __restrict__ z32, const float* __restrict__ pc,
                                                       CgState* st, double* partials) {
  __shared__ double xsh[kThreads / 32][RowCfg<NF, NBMAX>::FPW][RowCfg<NF, NBMAX>::NPOS];
  __shared__ float rsh[kThreads / 32][RowCfg<NF, NBMAX>::FPW][NF];
  HFX_FACE_SLOTS(NF)
  double rr = 0.0, rz = 0.0, bb = 0.0;
  for (int64_t fb = ((int64_t)blockIdx.x * (kThreads / 32) + warp) * FPW; fb < A.nFaces; fb += faceStride) {
    const int64_t f = fb + slot;
    const bool act = laneUsed && f < A.nFaces;
    const int64_t b0 = act ? A.browptr[f] : 0;
    const int nb = act ? (int)(A.browptr[f + 1] - b0) : 0;
    const bool rowBnd = act && A.isBnd[f];
    double* xs = laneUsed ? xsh[warp][slot] : nullptr;
    if (act) {
      if (A.ell && A.ellWidth == NBMAX) gather_x_ell<double, NF, NBMAX>(A, f, rowBnd, a, x, xs);
      else gather_x<double, NF, NBMAX, true, false>(A, b0, nb, rowBnd, a, 0.0, x, x, xs);
    }
    __syncwarp();
    float ra = 0.f;
    if (act) bb += bref[f * NF + a] * bref[f * NF + a];
    if (act) {
      double y = row_dot<double, NF>(val, b0, nb, a, xs);
      int64_t i = f * NF + a;
      double r = bS[i] - (rowBnd ? x[i] : -y);
      rr += r * r;
      ra = (float)r;
      r32[i] = ra;
      rsh[warp][slot][a] = ra;
    }
    __syncwarp();
    if (act) {
      int64_t i = f * NF + a;
      float zi;
      if (PC == 0) zi = ra;
      else if (PC == 1) zi = pc[i] * ra;
      else {
        zi = 0.f;
        const float* B = pc + f * NF * NF + a;
#pragma unroll
        for (int b = 0; b < NF; ++b) zi = fmaf(B[b * NF], rsh[warp][slot][b], zi);
      }
      z32[i] = zi;
      rz += (double)ra * (double)zi;
    }
    __syncwarp();
  }
  double v[3] = {rr, rz, bb}, tot[3];
  if (block_reduce_last<3>(v, partials, &st->ticket, tot) && threadIdx.x == 0) {
    st->rr = tot[0];
    st->rz = tot[1];
    st->bb = tot[2];
  }
}

// x64 += y32, y32 = 0
__global__ void accum_x(int64_t n, float* __restrict__ y, double* __restrict__ x) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    x[i] += (double)y[i];
    y[i] = 0.f;
  }
}

// Start of an inner FP32 CG from d = 0: r = rhs, z = M^{-1} r, r.z, r.r.
template <int NF, int PC>
__global__ void __launch_bounds__(kThreads) cg_start_zero_f32(int64_t nFaces, const float* __restrict__ rhs,
                                                              float* __restrict__ x, float* __restrict__ r,
                                                              float* __restrict__ z, const float* __restrict__ pc,
                                                              CgState* st, double* partials) {
  double rr = 0.0, rz = 0.0;
  for (int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; f < nFaces; f += (int64_t)gridDim.x * blockDim.x) {
    float rl[NF];
    for (int a = 0; a < NF; ++a) {
      int64_t i = f * NF + a;
      rl[a] = rhs[i];
      r[i] = rl[a];
      x[i] = 0.0f;
      rr += (double)rl[a] * rl[a];
    }
    for (int a = 0; a < NF; ++a) {
      int64_t i = f * NF + a;
      float zi;
      if (PC == 0) zi = rl[a];
      else if (PC == 1) zi = pc[i] * rl[a];
      else {
        zi = 0.0f;
        for (int b = 0; b < NF; ++b) zi = fmaf(pc[f * NF * NF + b * NF + a], rl[b], zi);
      }
      z[i] = zi;
      rz += (double)rl[a] * zi;
    }
  }
  double v[2] = {rr, rz}, tot[2];
  if (block_reduce_last<2>(v, partials, &st->ticket, tot) && threadIdx.x == 0) {
    st->rr = tot[0];
    st->rz = tot[1];
    st->bb = tot[0];
  }
}

template <int NF>
__global__ void copy_dirichlet(TraceView A, const double* __restrict__ bS, double* __restrict__ x) {
  for (int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; f < A.nFaces; f += (int64_t)gridDim.x * blockDim.x)
    if (A.isBnd[f])
      for (int a = 0; a < NF; ++a) x[f * NF + a] = bS[f * NF + a];
}

// b' = [-(b_I - A_ID b_D) ; b_D] from raw values of any precision (thread per row)
template <typename T, int NF, int NBMAX>
__global__ void __launch_bounds__(kThreads) prepare_rhs_t(TraceView A, const T* __restrict__ val,
                                                          const T* __restrict__ b, T* __restrict__ bS) {
  HFX_FACE_SLOTS(NF)
  for (int64_t fb = ((int64_t)blockIdx.x * (kThreads / 32) + warp) * FPW; fb < A.nFaces; fb += faceStride) {
    const int64_t f = fb + slot;
    if (!(laneUsed && f < A.nFaces)) continue;
    const int64_t b0 = A.browptr[f];
    const int nb = (int)(A.browptr[f + 1] - b0);
    const bool rowBnd = A.isBnd[f];
    double lift = 0.0;
    if (!rowBnd)
      for (int k = 0; k < nb; ++k) {
        int g = A.bcol[b0 + k];
        if (!A.isBnd[g]) continue;
        for (int c = 0; c < NF; ++c)
          lift += (double)val[(b0 + k) * NF * NF + (int64_t)c * NF + a] * (double)b[(int64_t)g * NF + c];
      }
    int64_t i = f * NF + a;
    bS[i] = rowBnd ? b[i] : (T)(-((double)b[i] - lift));
  }
}

template <typename T, int NF>
__global__ void build_precond_t(TraceView A, const T* __restrict__ val, int pcType, T* pc) {
  for (int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; f < A.nFaces; f += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b0 = A.browptr[f];
    const int nb = (int)(A.browptr[f + 1] - b0);
    int kd = 0;
    for (int k = 0; k < nb; ++k)
      if (A.bcol[b0 + k] == (int)f) kd = k;
    double B[NF][2 * NF];
    for (int a = 0; a < NF; ++a)
      for (int b = 0; b < NF; ++b) {
        B[a][b] = A.isBnd[f] ? (a == b ? 1.0 : 0.0) : -(double)val[(b0 + kd) * NF * NF + (int64_t)b * NF + a];
        B[a][NF + b] = (a == b) ? 1.0 : 0.0;
      }
    if (pcType == 1) {
      for (int a = 0; a < NF; ++a) pc[f * NF + a] = (T)(B[a][a] != 0.0 ? 1.0 / B[a][a] : 1.0);
      continue;
    }
    for (int k = 0; k < NF; ++k) {
      double inv = 1.0 / B[k][k];
      for (int j = 0; j < 2 * NF; ++j) B[k][j] *= inv;
      for (int i = 0; i < NF; ++i) {
        if (i == k) continue;
        double l = B[i][k];
        for (int j = 0; j < 2 * NF; ++j) B[i][j] -= l * B[k][j];
      }
    }
    for (int a = 0; a < NF; ++a)
      for (int b = 0; b < NF; ++b) pc[f * NF * NF + b * NF + a] = (T)B[a][NF + b];  // column-major
  }
}

template <typename KernelT>
int grid_of(KernelT k, int threads) {
  int dev = 0, nsm = 0, perSM = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, k, threads, 0);
  if (perSM < 1) perSM = 1;
  return nsm * perSM;
}

// ------------------------------------------------------------------ driver
template <int NF, int NBMAX>
struct Driver {
  static int run(const TraceSolveArgs& a, TraceSolveResult* out) {
    cudaStream_t s = a.stream;
    const TraceView& A = a.A;
    const int64_t n = (int64_t)A.nFaces * NF;
    // 0 none, 1 Jacobi, 2 block Jacobi, 3 two-level (block Jacobi + coarse space)
    const bool twoLevel = a.precond == 3 && a.coarse && a.coarse->ready;
    const int pcT = a.precond == 3 ? 2 : a.precond;  // the block-Jacobi part
    auto fail = [&](cudaError_t e) {
      out->cudaErr = e;
      return 3;
    };
    cudaError_t err;
    // grids: the resident CTAs, but no more than the work needs (every kernel is a
    // grid-stride loop; on small systems the extra CTAs would only add launch and
    // reduction cost): face-slot kernels take 32 / NF faces per warp, vector kernels a
    // trace value per thread
    const int64_t slotThreads = ((int64_t)A.nFaces + RowCfg<NF, NBMAX>::FPW - 1) / RowCfg<NF, NBMAX>::FPW * 32;
    auto cap = [](int g, int64_t threads) {
      const int64_t need = (threads + kThreads - 1) / kThreads;
      return (int)std::max<int64_t>(1, std::min<int64_t>(g, need));
    };
    const int gridF = cap(grid_of(cg_spmv<double, NF, NBMAX, true>, kThreads), slotThreads);
    const int gridF32 = cap(grid_of(cg_spmv<float, NF, NBMAX, false>, kThreads), slotThreads);
    const int gridE = cap(grid_of(cg_spmv_half_ell<NF, NBMAX>, kThreads), slotThreads);
    const int gridU = cap(grid_of(cg_update<double, NF, 2>, kThreads), slotThreads);
    const int gridS = cap(grid_of(prepare_system<NF, NBMAX>, kThreads), slotThreads);
    const int gridR1 = cap(grid_of(cg_update_r<double, NF>, kThreads), n);
    const int gridT = cap(grid_of(tl_apply<double, NF>, kThreads), slotThreads);
    double* partials = a.ws.partials;
    CgState* st = a.ws.state;
    CgState hst;
    KernelTimer* tm = a.timer;
    // two-level second half of K2 (coarse solve of r, then z and r.z)
    int coarseApplies = 0;
    auto coarse_z = [&](auto* rv, auto* zv, const auto* pcv, int init) {
      using T = std::remove_cv_t<std::remove_pointer_t<decltype(rv)>>;
      tm->begin(K_COARSE, s);
      coarse_apply<T>(*a.coarse, rv, &st->done, s);
      tm->end(K_COARSE, s);
      if (a.sampleBuf && a.sampleCount && coarseApplies % std::max(1, a.sampleStride) == 0 &&
          *a.sampleCount < a.sampleCap) {
        const int64_t nV = a.coarse->dev.nV;
        cudaMemcpyAsync(a.sampleBuf + (int64_t)(*a.sampleCount) * nV, a.coarse->dev.rc, sizeof(float) * nV,
                        cudaMemcpyDeviceToDevice, s);
        ++*a.sampleCount;
      }
      ++coarseApplies;
      tm->begin(K_UPDATE, s);
      tl_apply<T, NF><<<gridT, kThreads, 0, s>>>(A.nFaces, rv, zv, pcv, a.coarse->dev, st, partials, init);
      tm->end(K_UPDATE, s);
    };
    // 1. system b', FP32 values if needed, preconditioner
    tm->begin(K_OTHER, s);
    const bool half = a.mixed && A.hidx && a.ws.val32h;  // FP32 operator in symmetric half storage
    prepare_system<NF, NBMAX><<<gridS, kThreads, 0, s>>>(A, a.val, a.rhs, a.ws.bS,
                                                           a.mixed && !half ? a.ws.val32 : nullptr,
                                                           half ? a.ws.val32h : nullptr);
    if (pcT > 0) {
      // the mixed-precision solve only applies the FP32 copy: invert in FP32
      if (a.mixed)
        build_precond<NF, float><<<precond_grid<NF>(A.nFaces), kThreads, 0, s>>>(A, a.val, pcT, nullptr,
                                                                                       a.ws.pc32);
      else
        build_precond<NF><<<precond_grid<NF>(A.nFaces), kThreads, 0, s>>>(A, a.val, pcT, a.ws.pc64, nullptr);
    }
    tm->end(K_OTHER, s);
    if ((err = cudaGetLastError()) != cudaSuccess) return fail(err);
    double* x = a.x;
    if (!a.use_initial_guess) {
      // interior 0, Dirichlet rows g (b' holds g there)
      cudaMemsetAsync(x, 0, sizeof(double) * n, s);
    }
    auto reset_state = [&](int maxits) {
      CgState init{};
      init.maxits = maxits;
      return cudaMemcpyAsync(st, &init, sizeof(CgState), cudaMemcpyHostToDevice, s);
    };
    int totalIters = 0, refinements = 0, status = 0;
    if (!a.mixed) {
      if ((err = reset_state(a.maxits)) != cudaSuccess) return fail(err);
      if (!a.use_initial_guess) {
        // Dirichlet rows start exact: x_D = g
        set_dirichlet_start(A, a.ws.bS, x, s);
      }
      tm->begin(K_OTHER, s);
      launch_start(A, a, x, st, partials, pcT, gridF, s);
      tm->end(K_OTHER, s);
      if (twoLevel && a.coarse_guess && !a.use_initial_guess) {
        // initial guess: x0 = [P q(A_c) P^T b'; g], then the residual again
        tm->begin(K_COARSE, s);
        coarse_apply<double>(*a.coarse, a.ws.r, nullptr, s);
        coarse_prolong_add<double>(*a.coarse, x, s);
        tm->end(K_COARSE, s);
        if ((err = reset_state(a.maxits)) != cudaSuccess) return fail(err);
        tm->begin(K_OTHER, s);
        launch_start(A, a, x, st, partials, pcT, gridF, s);
        tm->end(K_OTHER, s);
      }
      if (twoLevel) coarse_z(a.ws.r, a.ws.z, (const double*)a.ws.pc64, 1);
      if ((err = cudaMemcpyAsync(&hst, st, sizeof(CgState), cudaMemcpyDeviceToHost, s)) != cudaSuccess) return fail(err);
      cudaStreamSynchronize(s);
      double tol2 = a.rtol * a.rtol * hst.bb;
      if (hst.rr <= tol2) {
        // already converged
      } else {
        double *r = a.ws.r, *z = a.ws.z, *p0 = a.ws.p0, *p1 = a.ws.p1, *q = a.ws.q;
        int it = 0;
        // the two-level solve converges in tens of iterations: check more often
        const int batch = twoLevel ? std::min(a.check_every, 10) : a.check_every;
        while (true) {
          for (int k = 0; k < batch; ++k, ++it) {
            double* pold = (it & 1) ? p1 : p0;
            double* pnew = (it & 1) ? p0 : p1;
            tm->begin(K_SPMV64, s);
            cg_spmv<double, NF, NBMAX, true><<<gridF, kThreads, 0, s>>>(A, a.val, z, pold, pnew, q, st, partials, it == 0);
            tm->end(K_SPMV64, s);
            if (twoLevel) {
              tm->begin(K_UPDATE, s);
              cg_update_r<double, NF><<<gridR1, kThreads, 0, s>>>(A.nFaces, x, r, pnew, q, st, partials, tol2);
              tm->end(K_UPDATE, s);
              coarse_z(r, z, (const double*)a.ws.pc64, 0);
            } else {
              tm->begin(K_UPDATE, s);
              launch_update<double>(A.nFaces, x, r, z, pnew, q, pcT >= 1 ? a.ws.pc64 : nullptr, st, partials, tol2,
                                    pcT, gridU, s);
              tm->end(K_UPDATE, s);
            }
          }
          if ((err = cudaGetLastError()) != cudaSuccess) return fail(err);
          cudaMemcpyAsync(&hst, st, sizeof(CgState), cudaMemcpyDeviceToHost, s);
          cudaStreamSynchronize(s);
          if (hst.done) break;
        }
        status = hst.status;
        totalIters = hst.iters;
      }
    } else {
      // Mixed-precision CG with reliable updates: one FP32 CG on the FP32 copy
      // of A' whose recursive residual is replaced by the true FP64 residual
      // b' - A' x64 whenever it has dropped by delta since the last
      // replacement; the iterate is accumulated in FP32 between replacements
      // and added to x64 in FP64. The search direction is never restarted, so
      // the iteration count stays close to FP64 CG's.
      float *r32 = a.ws.r32, *z32 = a.ws.z32, *p032 = a.ws.p032, *p132 = a.ws.p132, *q32 = a.ws.q32;
      float* y32 = a.ws.d32;
      // launch tuner: the first mixed solve on a system layout times the FP32 operator
      // kernels (three launches each, after one warm-up, on this system's own values; the
      // state is cleared before each launch so that every launch runs in full) and keeps the
      // fastest for this and later solves (*a.spmvChoice: 0 row per lane, 1 blocks staged in
      // shared memory by bulk copies (NF even; elsewhere kernel 0 runs), 2 row per lane with
      // paired loads of the transposed blocks, 3 the same with the gathered x read as float4s)
      const bool ellOk = half && A.ell && A.ellWidth == NBMAX;
      const int gridTma = tma_grid<NF, NBMAX>(A.nFaces);
      const int gridP = cap(grid_of(cg_spmv_half_ell<NF, NBMAX, true>, kThreads), slotThreads);
      int variant = 0;
      if (ellOk && a.spmvChoice) {
        if (*a.spmvChoice < 0) {
          cudaEvent_t e0, e1;
          cudaEventCreate(&e0);
          cudaEventCreate(&e1);
          float best[4] = {0.f, 1e30f, 0.f, 0.f};
          for (int v = 0; v < 4; ++v) {
            if (v == 1 && gridTma == 0) continue;
            float tmin = 1e30f;
            for (int rep = 0; rep < 4; ++rep) {
              cudaMemsetAsync(st, 0, sizeof(CgState), s);
              cudaEventRecord(e0, s);
              if (v == 0)
                cg_spmv_half_ell<NF, NBMAX><<<gridE, kThreads, 0, s>>>(A, a.ws.val32h, z32, p032, p132, q32, st,
                                                                        partials, 1);
              else if (v == 1)
                launch_spmv_tma<NF, NBMAX>(gridTma, s, A, a.ws.val32h, z32, p032, p132, q32, st, partials, 1);
              else if (v == 2)
                cg_spmv_half_ell<NF, NBMAX, true><<<gridP, kThreads, 0, s>>>(A, a.ws.val32h, z32, p032, p132, q32,
                                                                              st, partials, 1);
              else
                cg_spmv_half_ell<NF, NBMAX, true, true><<<gridP, kThreads, 0, s>>>(A, a.ws.val32h, z32, p032, p132,
                                                                                    q32, st, partials, 1);
              cudaEventRecord(e1, s);
              cudaEventSynchronize(e1);
              float ms = 0.f;
              cudaEventElapsedTime(&ms, e0, e1);
              if (rep > 0) tmin = std::min(tmin, ms);
            }
            best[v] = tmin;
          }
          cudaEventDestroy(e0);
          cudaEventDestroy(e1);
          if ((err = cudaGetLastError()) != cudaSuccess) return fail(err);
          int bestK = 0;
          for (int v = 1; v < 4; ++v)
            if (best[v] < best[bestK]) bestK = v;
          *a.spmvChoice = bestK;
          if (a.spmvTimes)
            for (int v = 0; v < 4; ++v) a.spmvTimes[v] = best[v] < 1e29f ? best[v] : 0.f;
        }
        variant = *a.spmvChoice;
      }
      // replace the residual after every inner_rtol of FP32 reduction (two
      // decades by default); FP32 rounding bounds how far a stretch can go
      const double delta = std::min(0.5, std::max(1e-4, a.inner_rtol));
      const int gridR = cap(grid_of(cg_replace<NF, NBMAX, 2>, kThreads), slotThreads);
      if (!a.use_initial_guess) set_dirichlet_start(A, a.ws.bS, x, s);
      cudaMemsetAsync(y32, 0, sizeof(float) * n, s);
      // true residual of x (and ||b||^2 of the reference rhs for the tolerance)
      auto replace = [&]() {
        tm->begin(K_OTHER, s);
        // with the two-level preconditioner tl_apply forms z and r.z right after:
        // the replacement skips its own block-Jacobi product
        switch (twoLevel ? 0 : pcT) {
          case 0: cg_replace<NF, NBMAX, 0><<<gridR, kThreads, 0, s>>>(A, a.val, a.ws.bS, a.rhs, x, r32, z32, a.ws.pc32, st, partials); break;
          case 1: cg_replace<NF, NBMAX, 1><<<gridR, kThreads, 0, s>>>(A, a.val, a.ws.bS, a.rhs, x, r32, z32, a.ws.pc32, st, partials); break;
          default: cg_replace<NF, NBMAX, 2><<<gridR, kThreads, 0, s>>>(A, a.val, a.ws.bS, a.rhs, x, r32, z32, a.ws.pc32, st, partials); break;
        }
        tm->end(K_OTHER, s);
        if (twoLevel) coarse_z(r32, z32, (const float*)a.ws.pc32, 1);
        cudaMemcpyAsync(&hst, st, sizeof(CgState), cudaMemcpyDeviceToHost, s);
        return cudaStreamSynchronize(s);
      };
      if ((err = reset_state(a.maxits)) != cudaSuccess) return fail(err);
      if ((err = replace()) != cudaSuccess) return fail(err);
      if (twoLevel && a.coarse_guess && !a.use_initial_guess) {
        tm->begin(K_COARSE, s);
        coarse_apply<float>(*a.coarse, r32, nullptr, s);
        coarse_prolong_add<double>(*a.coarse, x, s);
        tm->end(K_COARSE, s);
        if ((err = reset_state(a.maxits)) != cudaSuccess) return fail(err);
        if ((err = replace()) != cudaSuccess) return fail(err);
      }
      const double tol2 = a.rtol * a.rtol * hst.bb;
      double lastR2 = hst.rr;
      int lastStretch = 0;
      bool first = true;
      while (hst.rr > tol2) {
        if (!std::isfinite(hst.rr)) {
          status = 7;
          break;
        }
        if (totalIters >= a.maxits) {
          status = 5;
          break;
        }
        // the FP32 recurrence runs until its residual has dropped by delta
        // since the last replacement (never below the final tolerance)
        const double stretch2 = std::max(delta * delta * lastR2, tol2);
        hst.done = 0;
        hst.iters = 0;
        hst.maxits = a.maxits - totalIters;
        hst.status = 0;
        hst.ticket = 0;
        cudaMemcpyAsync(st, &hst, sizeof(CgState), cudaMemcpyHostToDevice, s);
        int it = totalIters;  // the ping-pong parity follows completed iterations
        // iterations queued before the host checks: one more than the last stretch took (the
        // first stretch: one more than the first stretch of the previous solve on this system
        // layout, else 8), then short batches. Iterations queued past the stretch's end return
        // at entry, but each still costs its launches.
        const int hint = a.stretchHint && *a.stretchHint > 0 ? *a.stretchHint + 1 : 8;
        int batch = std::max(3, std::min(a.check_every, lastStretch > 0 ? lastStretch + 1 : hint));
        while (true) {
          for (int k = 0; k < batch; ++k, ++it) {
            float* pold = (it & 1) ? p132 : p032;
            float* pnew = (it & 1) ? p032 : p132;
            tm->begin(K_SPMV32, s);
            if (ellOk && variant == 1 && gridTma > 0)
              launch_spmv_tma<NF, NBMAX>(gridTma, s, A, a.ws.val32h, z32, pold, pnew, q32, st, partials, first ? 1 : 0);
            else if (ellOk && variant == 2)
              cg_spmv_half_ell<NF, NBMAX, true><<<gridP, kThreads, 0, s>>>(A, a.ws.val32h, z32, pold, pnew, q32, st,
                                                                            partials, first ? 1 : 0);
            else if (ellOk && variant == 3)
              cg_spmv_half_ell<NF, NBMAX, true, true><<<gridP, kThreads, 0, s>>>(A, a.ws.val32h, z32, pold, pnew, q32,
                                                                                  st, partials, first ? 1 : 0);
            else if (ellOk)
              cg_spmv_half_ell<NF, NBMAX><<<gridE, kThreads, 0, s>>>(A, a.ws.val32h, z32, pold, pnew, q32, st,
                                                                      partials, first ? 1 : 0);
            else if (half)
              cg_spmv_half<NF, NBMAX><<<gridF32, kThreads, 0, s>>>(A, a.ws.val32h, z32, pold, pnew, q32, st, partials,
                                                                    first ? 1 : 0);
            else
              cg_spmv<float, NF, NBMAX, false><<<gridF32, kThreads, 0, s>>>(A, a.ws.val32, z32, pold, pnew, q32, st,
                                                                            partials, first ? 1 : 0);
            tm->end(K_SPMV32, s);
            first = false;
            if (twoLevel) {
              tm->begin(K_UPDATE, s);
              cg_update_r<float, NF><<<gridR1, kThreads, 0, s>>>(A.nFaces, y32, r32, pnew, q32, st, partials, stretch2);
              tm->end(K_UPDATE, s);
              coarse_z(r32, z32, (const float*)a.ws.pc32, 0);
            } else {
              tm->begin(K_UPDATE, s);
              launch_update<float>(A.nFaces, y32, r32, z32, pnew, q32, a.ws.pc32, st, partials, stretch2, pcT, gridU, s);
              tm->end(K_UPDATE, s);
            }
          }
          if ((err = cudaGetLastError()) != cudaSuccess) return fail(err);
          cudaMemcpyAsync(&hst, st, sizeof(CgState), cudaMemcpyDeviceToHost, s);
          cudaStreamSynchronize(s);
          if (hst.done) break;
          batch = std::max(2, batch / 4);
        }
        if (a.stretchHint && lastStretch == 0 && hst.iters > 0) *a.stretchHint = hst.iters;
        totalIters += hst.iters;
        lastStretch = hst.iters;
        if (hst.status != 0 && hst.status != 5) {
          status = hst.status;
          break;
        }
        // r.z of the iteration before the last one: beta = rz_new / rz_prev
        const double rzPrev = hst.beta != 0.0 ? hst.rz / hst.beta : 0.0;
        // reliable update: x += y (FP64), r = b' - A' x (FP64), direction kept
        accum_x<<<gridU, kThreads, 0, s>>>(n, y32, x);
        hst.ticket = 0;
        hst.done = 0;  // the stretch's stop flag would make the two-level z of the replacement return at entry
        cudaMemcpyAsync(st, &hst, sizeof(CgState), cudaMemcpyHostToDevice, s);
        if ((err = replace()) != cudaSuccess) return fail(err);
        refinements += 1;
        lastR2 = hst.rr;
        hst.beta = rzPrev > 0.0 ? hst.rz / rzPrev : 0.0;
        if (hst.iters == 0) first = true;  // nothing ran: restart the direction
      }
    }
    if (a.mixed && status == 0) {
      // the last reliable update computed the true residual of the eliminated
      // system, whose norm equals the reference system's (Dirichlet rows exact)
      out->iterations = totalIters;
      out->refinements = refinements;
      out->rel_residual = hst.bb > 0 ? std::sqrt(hst.rr / hst.bb) : std::sqrt(hst.rr);
      return status;
    }
    // final residual of the reference system
    CgState init{};
    cudaMemcpyAsync(st, &init, sizeof(CgState), cudaMemcpyHostToDevice, s);
    tm->begin(K_OTHER, s);
    ref_residual<NF, NBMAX><<<gridF, kThreads, 0, s>>>(A, a.val, a.rhs, x, st, partials);
    tm->end(K_OTHER, s);
    if ((err = cudaGetLastError()) != cudaSuccess) return fail(err);
    cudaMemcpyAsync(&hst, st, sizeof(CgState), cudaMemcpyDeviceToHost, s);
    if ((err = cudaStreamSynchronize(s)) != cudaSuccess) return fail(err);
    out->iterations = totalIters;
    out->refinements = refinements;
    out->rel_residual = hst.res_bb > 0 ? std::sqrt(hst.res_rr / hst.res_bb) : std::sqrt(hst.res_rr);
    return status;
  }

  static void set_dirichlet_start(const TraceView& A, const double* bS, double* x, cudaStream_t s) {
    copy_dirichlet<NF><<<(unsigned)((A.nFaces + 255) / 256), 256, 0, s>>>(A, bS, x);
  }
  static void launch_start(const TraceView& A, const TraceSolveArgs& a, double* x, CgState* st, double* partials,
                           int pcT, int grid, cudaStream_t s) {
    const double* pc = a.ws.pc64;
    switch (pcT) {
      case 0: cg_start<NF, NBMAX, 0><<<grid, kThreads, 0, s>>>(A, a.val, a.ws.bS, a.rhs, x, a.ws.r, a.ws.z, pc, st, partials); break;
      case 1: cg_start<NF, NBMAX, 1><<<grid, kThreads, 0, s>>>(A, a.val, a.ws.bS, a.rhs, x, a.ws.r, a.ws.z, pc, st, partials); break;
      default: cg_start<NF, NBMAX, 2><<<grid, kThreads, 0, s>>>(A, a.val, a.ws.bS, a.rhs, x, a.ws.r, a.ws.z, pc, st, partials); break;
    }
  }
  static void launch_start_f32(int64_t nFaces, const float* rhs, float* x, float* r, float* z, const float* pc,
                               CgState* st, double* partials, int pcT, int grid, cudaStream_t s) {
    switch (pcT) {
      case 0: cg_start_zero_f32<NF, 0><<<grid, kThreads, 0, s>>>(nFaces, rhs, x, r, z, pc, st, partials); break;
      case 1: cg_start_zero_f32<NF, 1><<<grid, kThreads, 0, s>>>(nFaces, rhs, x, r, z, pc, st, partials); break;
      default: cg_start_zero_f32<NF, 2><<<grid, kThreads, 0, s>>>(nFaces, rhs, x, r, z, pc, st, partials); break;
    }
  }
  template <typename T>
  static void launch_update(int64_t nFaces, T* x, T* r, T* z, const T* p, const T* q, const T* pc, CgState* st,
                            double* partials, double tol2, int pcT, int grid, cudaStream_t s) {
    switch (pcT) {
      case 0: cg_update<T, NF, 0><<<grid, kThreads, 0, s>>>(nFaces, x, r, z, p, q, pc, st, partials, tol2); break;
      case 1: cg_update<T, NF, 1><<<grid, kThreads, 0, s>>>(nFaces, x, r, z, p, q, pc, st, partials, tol2); break;
      default: cg_update<T, NF, 2><<<grid, kThreads, 0, s>>>(nFaces, x, r, z, p, q, pc, st, partials, tol2); break;
    }
  }
};

}  // namespace

int trace_solve(const TraceSolveArgs& a, TraceSolveResult* out) {
  const int NF = a.A.NF;
  if (a.dim == 2) {
    switch (NF) {
      case 2: return Driver<2, 5>::run(a, out);
      case 3: return Driver<3, 5>::run(a, out);
      case 4: return Driver<4, 5>::run(a, out);
      case 5: return Driver<5, 5>::run(a, out);
      case 6: return Driver<6, 5>::run(a, out);
    }
  } else if (a.dim == 3) {
    switch (NF) {
      case 3: return Driver<3, 7>::run(a, out);
      case 6: return Driver<6, 7>::run(a, out);
      case 10: return Driver<10, 7>::run(a, out);
    }
  }
  return 9;  // HFX_ERR_UNSUPPORTED
}

size_t trace_partials_needed() { return 64 * 152 * 32; }

template <int NF, int NBMAX>
static void prepare_t(const TraceSolveArgs& a) {
  cudaStream_t s = a.stream;
  const int gridS = grid_of(prepare_system<NF, NBMAX>, kThreads);
  a.timer->begin(K_OTHER, s);
  prepare_system<NF, NBMAX><<<gridS, kThreads, 0, s>>>(a.A, a.val, a.rhs, a.ws.bS, a.mixed ? a.ws.val32 : nullptr);
  if (a.precond > 0)
    build_precond<NF><<<precond_grid<NF>(a.A.nFaces), kThreads, 0, s>>>(a.A, a.val, a.precond, a.ws.pc64,
                                                                           a.mixed ? a.ws.pc32 : nullptr);
  a.timer->end(K_OTHER, s);
}

template <int NF, int NBMAX>
static void residual_t(const TraceSolveArgs& a, TraceSolveResult* out) {
  cudaStream_t s = a.stream;
  CgState init{}, hst;
  cudaMemcpyAsync(a.ws.state, &init, sizeof(CgState), cudaMemcpyHostToDevice, s);
  const int gridF = grid_of(ref_residual<NF, NBMAX>, kThreads);
  a.timer->begin(K_OTHER, s);
  ref_residual<NF, NBMAX><<<gridF, kThreads, 0, s>>>(a.A, a.val, a.rhs, a.x, a.ws.state, a.ws.partials);
  a.timer->end(K_OTHER, s);
  cudaMemcpyAsync(&hst, a.ws.state, sizeof(CgState), cudaMemcpyDeviceToHost, s);
  cudaStreamSynchronize(s);
  out->rel_residual = hst.res_bb > 0 ? std::sqrt(hst.res_rr / hst.res_bb) : std::sqrt(hst.res_rr);
}

#define HFX_DISPATCH_NF(fn, ...)                                            \
  do {                                                                      \
    const int NF_ = a.A.NF;                                                 \
    if (a.dim == 2) {                                                       \
      if (NF_ == 2) fn<2, 5>(__VA_ARGS__);                                  \
      else if (NF_ == 3) fn<3, 5>(__VA_ARGS__);                             \
      else if (NF_ == 4) fn<4, 5>(__VA_ARGS__);                             \
      else if (NF_ == 5) fn<5, 5>(__VA_ARGS__);                             \
      else if (NF_ == 6) fn<6, 5>(__VA_ARGS__);                             \
    } else {                                                                \
      if (NF_ == 3) fn<3, 7>(__VA_ARGS__);                                  \
      else if (NF_ == 6) fn<6, 7>(__VA_ARGS__);                             \
      else if (NF_ == 10) fn<10, 7>(__VA_ARGS__);                           \
    }                                                                       \
  } while (0)

// The same dispatch with the vector (Burgers) trace blocks of 2D cells, Nf*dim = 8, 10, 12
// (p = 3, 4, 5), which only the FP64 GMRES path uses.
#define HFX_DISPATCH_NF_VEC(fn, ...)                                        \
  do {                                                                      \
    const int NFV_ = a.A.NF;                                                \
    if (a.dim == 2 && NFV_ == 8) fn<8, 5>(__VA_ARGS__);                     \
    else if (a.dim == 2 && NFV_ == 10) fn<10, 5>(__VA_ARGS__);              \
    else if (a.dim == 2 && NFV_ == 12) fn<12, 5>(__VA_ARGS__);              \
    else HFX_DISPATCH_NF(fn, __VA_ARGS__);                                  \
  } while (0)

void trace_prepare(const TraceSolveArgs& a) { HFX_DISPATCH_NF_VEC(prepare_t, a); }

template <int NF, int NBMAX>
static void prepare_f32_t(const TraceView& A, const float* val, const float* rhs, float* bS, int pcType, float* pc,
                          cudaStream_t s) {
  prepare_rhs_t<float, NF, NBMAX><<<grid_of(prepare_rhs_t<float, NF, NBMAX>, kThreads), kThreads, 0, s>>>(A, val, rhs, bS);
  if (pcType > 0 && pc)
    build_precond_t<float, NF><<<(unsigned)((A.nFaces + 127) / 128), 128, 0, s>>>(A, val, pcType, pc);
}

void trace_prepare_f32(int dim, const TraceView& A, const float* val, const float* rhs, float* bS, int pcType,
                       float* pc, cudaStream_t s) {
  struct {
    int dim;
    TraceView A;
  } a{dim, A};
  HFX_DISPATCH_NF(prepare_f32_t, A, val, rhs, bS, pcType, pc, s);
}

// FP32 CG on the eliminated system from raw FP32 values (masked on the fly).
template <int NF, int NBMAX>
static void cg_f32_t(const F32SolveArgs& a, int* its, int* status) {
  cudaStream_t s = a.stream;
  const TraceView& A = a.A;
  KernelTimer* tm = a.timer;
  const int gridF = grid_of(cg_spmv<float, NF, NBMAX, true>, kThreads);
  const int gridU = grid_of(cg_update<float, NF, 2>, kThreads);
  tm->begin(K_OTHER, s);
  prepare_f32_t<NF, NBMAX>(A, a.val, a.rhs, a.ws.bS32, a.rebuildPrecond ? a.precond : 0, a.ws.pc32, s);
  CgState init{}, hst;
  init.maxits = a.maxits;
  cudaMemcpyAsync(a.ws.state, &init, sizeof(CgState), cudaMemcpyHostToDevice, s);
  switch (a.precond) {
    case 0: cg_start_zero_f32<NF, 0><<<gridU, kThreads, 0, s>>>(A.nFaces, a.ws.bS32, a.x, a.ws.r32, a.ws.z32, a.ws.pc32, a.ws.state, a.ws.partials); break;
    case 1: cg_start_zero_f32<NF, 1><<<gridU, kThreads, 0, s>>>(A.nFaces, a.ws.bS32, a.x, a.ws.r32, a.ws.z32, a.ws.pc32, a.ws.state, a.ws.partials); break;
    default: cg_start_zero_f32<NF, 2><<<gridU, kThreads, 0, s>>>(A.nFaces, a.ws.bS32, a.x, a.ws.r32, a.ws.z32, a.ws.pc32, a.ws.state, a.ws.partials); break;
  }
  tm->end(K_OTHER, s);
  cudaMemcpyAsync(&hst, a.ws.state, sizeof(CgState), cudaMemcpyDeviceToHost, s);
  cudaStreamSynchronize(s);
  const double tol2 = a.rtol * a.rtol * hst.rr;
  *status = 0;
  if (!(hst.rr > tol2)) return;
  int it = 0;
  while (true) {
    for (int k = 0; k < 25; ++k, ++it) {
      float* pold = (it & 1) ? a.ws.p132 : a.ws.p032;
      float* pnew = (it & 1) ? a.ws.p032 : a.ws.p132;
      tm->begin(K_SPMV32, s);
      cg_spmv<float, NF, NBMAX, true><<<gridF, kThreads, 0, s>>>(A, a.val, a.ws.z32, pold, pnew, a.ws.q32, a.ws.state,
                                                                  a.ws.partials, it == 0);
      tm->end(K_SPMV32, s);
      tm->begin(K_UPDATE, s);
      switch (a.precond) {
        case 0: cg_update<float, NF, 0><<<gridU, kThreads, 0, s>>>(A.nFaces, a.x, a.ws.r32, a.ws.z32, pnew, a.ws.q32, a.ws.pc32, a.ws.state, a.ws.partials, tol2); break;
        case 1: cg_update<float, NF, 1><<<gridU, kThreads, 0, s>>>(A.nFaces, a.x, a.ws.r32, a.ws.z32, pnew, a.ws.q32, a.ws.pc32, a.ws.state, a.ws.partials, tol2); break;
        default: cg_update<float, NF, 2><<<gridU, kThreads, 0, s>>>(A.nFaces, a.x, a.ws.r32, a.ws.z32, pnew, a.ws.q32, a.ws.pc32, a.ws.state, a.ws.partials, tol2); break;
      }
      tm->end(K_UPDATE, s);
    }
    cudaMemcpyAsync(&hst, a.ws.state, sizeof(CgState), cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    if (hst.done) break;
  }
  *its += hst.iters;
  *status = hst.status;
}

int trace_solve_f32(const F32SolveArgs& a, int* its) {
  if (a.gmres) return trace_gmres_f32(a, its);
  int status = 9;
  HFX_DISPATCH_NF(cg_f32_t, a, its, &status);
  return status;
}
void trace_ref_residual(const TraceSolveArgs& a, TraceSolveResult* out) { HFX_DISPATCH_NF_VEC(residual_t, a, out); }

}  // namespace hfx
