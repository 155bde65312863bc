// Vertex coarse space of the two-level trace preconditioner (see coarse.h):
// host construction of the coarse pattern and of the contribution lists, the
// Galerkin coarse operator from the element matrices, a Lanczos estimate of its
// Jacobi-scaled spectrum, the Chebyshev coarse solve, restriction and
// prolongation. Every sum runs in a fixed order (no atomics), so the coarse
// operator and the preconditioner are bitwise reproducible.
#include "coarse.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <numeric>

namespace hfx {

// ------------------------------------------------------------------ host

// Barycentric coordinates of a reference point w.r.t. the reference vertices
// (nodes 0..dim): solve sum_m l_m V_m = x, sum_m l_m = 1.
static void barycentric(const RefEl& re, const double* x, double* lam) {
  const int d = re.dim;
  double A[4][5];
  for (int r = 0; r <= d; ++r) {
    for (int m = 0; m <= d; ++m) A[r][m] = (r < d) ? re.nodes[m * d + r] : 1.0;
    A[r][d + 1] = (r < d) ? x[r] : 1.0;
  }
  const int n = d + 1;
  for (int k = 0; k < n; ++k) {
    int piv = k;
    for (int i = k + 1; i < n; ++i)
      if (std::fabs(A[i][k]) > std::fabs(A[piv][k])) piv = i;
    for (int j = 0; j <= n; ++j) std::swap(A[k][j], A[piv][j]);
    for (int i = 0; i < n; ++i) {
      if (i == k) continue;
      double l = A[i][k] / A[k][k];
      for (int j = k; j <= n; ++j) A[i][j] -= l * A[k][j];
    }
  }
  for (int m = 0; m < n; ++m) lam[m] = A[m][n] / A[m][m];
}

bool coarse_weight_tables(const RefEl& re, std::vector<double>* Wf, std::vector<double>* Wc, std::string* err) {
  const int d = re.dim, F = re.nFaces, NF = re.nNodesFace, NV1 = d + 1;
  Wc->assign((size_t)F * NF * NV1, 0.0);
  Wf->assign((size_t)NF * d, 0.0);
  for (int i = 0; i < F; ++i) {
    const int* fn = &re.faceNodes[(size_t)i * NF];
    for (int k = 0; k < d; ++k)
      if (fn[k] > d) {
        *err = "coarse space: face vertices are not the first face nodes";
        return false;
      }
    for (int j = 0; j < NF; ++j) {
      double lam[4];
      barycentric(re, &re.nodes[(size_t)fn[j] * d], lam);
      for (int m = 0; m < NV1; ++m) (*Wc)[((size_t)i * NF + j) * NV1 + m] = std::fabs(lam[m]) < 1e-14 ? 0.0 : lam[m];
      for (int k = 0; k < d; ++k) {
        double w = lam[fn[k]];
        if (std::fabs(w) < 1e-14) w = 0.0;
        if (i == 0) (*Wf)[(size_t)j * d + k] = w;
        else if (std::fabs((*Wf)[(size_t)j * d + k] - w) > 1e-12) {
          *err = "coarse space: face weight table differs between faces";
          return false;
        }
      }
    }
  }
  return true;
}

bool build_coarse_host(const RefEl& re, int nCells, const int* cellVerts, const Topology& t, CoarseHost* out,
                       std::string* err) {
  const int d = re.dim, F = re.nFaces, NF = re.nNodesFace, NV1 = d + 1;
  CoarseHost h;
  h.dim = d;
  h.NF = NF;
  h.F = F;
  h.LL = F * NF;
  h.NV1 = NV1;
  std::vector<double> Wf, Wc;
  if (!coarse_weight_tables(re, &Wf, &Wc, err)) return false;
  h.Wf.assign(Wf.begin(), Wf.end());
  h.Wc.assign(Wc.begin(), Wc.end());
  // coarse ids of the distinct cell vertices, in order of first appearance
  int maxNode = 0;
  for (int64_t i = 0; i < (int64_t)nCells * NV1; ++i) maxNode = std::max(maxNode, cellVerts[i]);
  std::vector<int> cv((size_t)maxNode + 1, -1);
  h.cellV.resize((size_t)nCells * NV1);
  for (int e = 0; e < nCells; ++e)
    for (int m = 0; m < NV1; ++m) {
      int node = cellVerts[(int64_t)e * NV1 + m];
      if (cv[node] < 0) {
        cv[node] = h.nV++;
        h.vertexNode.push_back(node);
      }
      h.cellV[(size_t)e * NV1 + m] = cv[node];
    }
  h.faceV.resize((size_t)t.nFaces * d);
  for (int f = 0; f < t.nFaces; ++f)
    for (int k = 0; k < d; ++k) {
      int node = t.faces[(size_t)f * NF + k];
      if (node > maxNode || cv[node] < 0) {
        *err = "coarse space: face vertex is not a cell vertex";
        return false;
      }
      h.faceV[(size_t)f * d + k] = cv[node];
    }
  // pattern: vertices sharing a cell; counting sort of (row, col) pairs
  const int nV = h.nV;
  std::vector<int64_t> cnt((size_t)nV + 1, 0);
  for (int e = 0; e < nCells; ++e)
    for (int m = 0; m < NV1; ++m) cnt[h.cellV[(size_t)e * NV1 + m] + 1] += NV1;
  for (int v = 0; v < nV; ++v) cnt[v + 1] += cnt[v];
  std::vector<int> pairs((size_t)cnt[nV]);   // column per (row, contribution)
  std::vector<int> pairSrc((size_t)cnt[nV]);  // contribution index e*NV1^2 + m*NV1 + m2
  {
    std::vector<int64_t> pos(cnt.begin(), cnt.end() - 1);
    for (int e = 0; e < nCells; ++e)
      for (int m = 0; m < NV1; ++m) {
        int v = h.cellV[(size_t)e * NV1 + m];
        for (int m2 = 0; m2 < NV1; ++m2) {
          int64_t p = pos[v]++;
          pairs[p] = h.cellV[(size_t)e * NV1 + m2];
          pairSrc[p] = (e * NV1 + m) * NV1 + m2;
        }
      }
  }
  h.rowptr.assign((size_t)nV + 1, 0);
  h.cptr.push_back(0);
  std::vector<int> order;
  for (int v = 0; v < nV; ++v) {
    const int64_t b = cnt[v], n = cnt[v + 1] - b;
    order.resize(n);
    std::iota(order.begin(), order.end(), 0);
    // stable by column, then by contribution index (fixed summation order)
    std::sort(order.begin(), order.end(), [&](int x, int y) {
      if (pairs[b + x] != pairs[b + y]) return pairs[b + x] < pairs[b + y];
      return pairSrc[b + x] < pairSrc[b + y];
    });
    int last = -1;
    for (int64_t j = 0; j < n; ++j) {
      int c = pairs[b + order[j]];
      if (c != last) {
        if (last >= 0) h.cptr.push_back((int)h.cidx.size());
        h.col.push_back(c);
        last = c;
      }
      h.cidx.push_back(pairSrc[b + order[j]]);
    }
    if (last >= 0) h.cptr.push_back((int)h.cidx.size());
    h.rowptr[v + 1] = (int)h.col.size();
  }
  if ((int64_t)nCells * NV1 * NV1 > 2147483647LL) {
    *err = "coarse space: too many cells for 32-bit contribution indices";
    return false;
  }
  // ELL copy (column-major by slot): coalesced, fixed-width rows for the Chebyshev steps
  for (int v = 0; v < nV; ++v) h.ellW = std::max(h.ellW, h.rowptr[v + 1] - h.rowptr[v]);
  h.ellW = (h.ellW + 7) / 8 * 8;  // whole batches of 8 loads in flight, no serial tail
  h.ellCol.assign((size_t)h.ellW * nV, 0);
  h.ellSrc.assign((size_t)h.ellW * nV, -1);
  for (int v = 0; v < nV; ++v)
    for (int k = 0; k < h.ellW; ++k) {
      const int q = h.rowptr[v] + k;
      const bool in = q < h.rowptr[v + 1];
      h.ellCol[(size_t)k * nV + v] = in ? h.col[q] : v;
      h.ellSrc[(size_t)k * nV + v] = in ? q : -1;
    }
  // restriction lists: faces incident to each vertex
  h.rptr.assign((size_t)nV + 1, 0);
  for (int f = 0; f < t.nFaces; ++f)
    for (int k = 0; k < d; ++k) h.rptr[h.faceV[(size_t)f * d + k] + 1]++;
  for (int v = 0; v < nV; ++v) h.rptr[v + 1] += h.rptr[v];
  h.ridx.resize((size_t)h.rptr[nV]);
  {
    std::vector<int> pos(h.rptr.begin(), h.rptr.end() - 1);
    for (int f = 0; f < t.nFaces; ++f)
      for (int k = 0; k < d; ++k) h.ridx[pos[h.faceV[(size_t)f * d + k]]++] = f * d + k;
  }
  *out = std::move(h);
  return true;
}

// ------------------------------------------------------------------ device

namespace {

constexpr int kT = 256;

unsigned blocks_for(int64_t n, int threads = kT) {
  int64_t g = (n + threads - 1) / threads;
  if (g > 152 * 32) g = 152 * 32;
  return (unsigned)(g < 1 ? 1 : g);
}

// C_e = -W_m^T S_e W_m, W_m = cell weights with the rows of Dirichlet faces
// zeroed (A' = -A on interior rows). One warp per cell; lanes run over rows of
// S_e (column-major, coalesced), FP32 arithmetic on the stored values.
template <typename T, int NV1>
__global__ void coarse_elem(CoarseDev c, const T* __restrict__ S) {
  const int lane = threadIdx.x & 31;
  const int64_t warpId = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nWarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int LL = c.LL, NF = c.NF;
  for (int64_t e = warpId; e < c.nCells; e += nWarps) {
    const T* Se = S + e * (int64_t)LL * LL;
    unsigned fmask = 0;  // bit i: face i of the cell is interior
    for (int i = 0; i < c.F; ++i)
      if (!c.isBnd[c.cell2face[e * c.F + i]]) fmask |= 1u << i;
    float acc[NV1][NV1];
#pragma unroll
    for (int m = 0; m < NV1; ++m)
#pragma unroll
      for (int m2 = 0; m2 < NV1; ++m2) acc[m][m2] = 0.f;
    for (int r = lane; r < LL; r += 32) {
      const float maskR = (fmask >> (r / NF)) & 1u ? 1.f : 0.f;
      float t[NV1];
#pragma unroll
      for (int m2 = 0; m2 < NV1; ++m2) t[m2] = 0.f;
#pragma unroll 8
      for (int col = 0; col < LL; ++col) {  // unrolled: eight rows of S in flight per lane
        const float mc = (fmask >> (col / NF)) & 1u ? 1.f : 0.f;
        const float s = (float)Se[r + (int64_t)col * LL] * mc;
#pragma unroll
        for (int m2 = 0; m2 < NV1; ++m2) t[m2] = fmaf(s, c.Wc[col * NV1 + m2], t[m2]);
      }
#pragma unroll
      for (int m = 0; m < NV1; ++m) {
        const float w = c.Wc[r * NV1 + m] * maskR;
#pragma unroll
        for (int m2 = 0; m2 < NV1; ++m2) acc[m][m2] = fmaf(w, t[m2], acc[m][m2]);
      }
    }
#pragma unroll
    for (int m = 0; m < NV1; ++m)
#pragma unroll
      for (int m2 = 0; m2 < NV1; ++m2) {
        float x = acc[m][m2];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
        if (lane == 0) c.Ce[e * NV1 * NV1 + m * NV1 + m2] = -x;
      }
  }
}

// Coarse values by gathering the element contributions in fixed order, and the
// inverse diagonal (0 marks a coarse DOF that touches no interior face).
__global__ void coarse_gather(CoarseDev c) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < c.nV; v += (int64_t)gridDim.x * blockDim.x) {
    float diag = 0.f;
    for (int k = c.rowptr[v]; k < c.rowptr[v + 1]; ++k) {
      float s = 0.f;
      for (int j = c.cptr[k]; j < c.cptr[k + 1]; ++j) s += c.Ce[c.cidx[j]];
      c.val[k] = s;
      if (c.col[k] == v) diag = s;
    }
    c.dinv[v] = diag > 0.f ? 1.f / diag : 0.f;
  }
}

__global__ void coarse_fill_ell(CoarseDev c) {
  const int64_t n = (int64_t)c.ellW * c.nV;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int q = c.ellSrc[i];
    c.ellVal[i] = q >= 0 ? c.val[q] : 0.f;
  }
}

// y_v = sum_k ell[k][v] x[col] with up to 8 loads in flight (x read through L2:
// other blocks write it between grid barriers)
__device__ __forceinline__ float ell_row(const CoarseDev& c, int64_t v, const float* x) {
  float y = 0.f;
  const int W = c.ellW;
  int k = 0;
  for (; k + 8 <= W; k += 8) {
    int cc[8];
    float aa[8], xx[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      cc[u] = c.ellCol[(int64_t)(k + u) * c.nV + v];
      aa[u] = c.ellVal[(int64_t)(k + u) * c.nV + v];
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) xx[u] = __ldcg(x + cc[u]);
#pragma unroll
    for (int u = 0; u < 8; ++u) y = fmaf(aa[u], xx[u], y);
  }
  for (; k < W; ++k) y = fmaf(c.ellVal[(int64_t)k * c.nV + v], __ldcg(x + c.ellCol[(int64_t)k * c.nV + v]), y);
  return y;
}

// ---- Lanczos on D^{-1/2} A_c D^{-1/2} (eigenvalue bounds for Chebyshev)

__device__ __forceinline__ float coarse_row_sym(const CoarseDev& c, int64_t v, const float* __restrict__ x) {
  const float sv = sqrtf(c.dinv[v]);
  float y = 0.f;
  for (int k = c.rowptr[v]; k < c.rowptr[v + 1]; ++k) {
    const int w = c.col[k];
    y = fmaf(c.val[k] * sqrtf(c.dinv[w]), x[w], y);
  }
  return sv * y;
}

__device__ void block_partial(double v, double* partials, int slot) {
  __shared__ double red[kT / 32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
    partials[(size_t)slot * gridDim.x + blockIdx.x] = s;
  }
  __syncthreads();
}

// start vector: deterministic pseudo-random entries on active DOFs; norm^2
__global__ void lanczos_init(CoarseDev c, float* v, double* partials) {
  double ss = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < c.nV; i += (int64_t)gridDim.x * blockDim.x) {
    uint32_t h = (uint32_t)i * 2654435761u + 12345u;
    h ^= h >> 13;
    h *= 0x5bd1e995u;
    h ^= h >> 15;
    float x = c.dinv[i] > 0.f ? 0.5f + (float)(h & 0xffff) / 65536.f : 0.f;
    v[i] = x;
    ss += (double)x * x;
  }
  block_partial(ss, partials, 0);
}

__global__ void lanczos_scale(int64_t n, float* v, float s) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    v[i] *= s;
}

// w = A v - beta v_prev; partials alpha = w . v, |w|^2 and |v|^2. The next beta is
// |w - alpha v| = sqrt(|w|^2 - alpha^2 (2 - |v|^2)), with the computed |v|^2: assuming
// |v| = 1 instead multiplies the norm error of v by about (alpha / beta)^2 every step,
// and within 15-30 steps the tridiagonal's eigenvalues leave the spectrum.
__global__ void lanczos_apply(CoarseDev c, const float* v, const float* vprev, float beta, float* w,
                              double* partials) {
  double a = 0.0, ww = 0.0, vv = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < c.nV; i += (int64_t)gridDim.x * blockDim.x) {
    float y = c.dinv[i] > 0.f ? coarse_row_sym(c, i, v) : 0.f;
    y -= beta * vprev[i];
    w[i] = y;
    const float vi = v[i];
    a += (double)y * vi;
    ww += (double)y * y;
    vv += (double)vi * vi;
  }
  block_partial(a, partials, 0);
  block_partial(ww, partials, 1);
  block_partial(vv, partials, 2);
}

// v_next = (w - alpha v) / beta
__global__ void lanczos_next(int64_t n, const float* v, float alpha, float ib, float* w) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    w[i] = (w[i] - alpha * v[i]) * ib;
}

// Absolute row sum of row v of D^{-1/2} A_c D^{-1/2} (0 for an inactive row). Its maximum
// over the rows, the matrix's infinity norm, bounds the spectral radius from above.
__device__ __forceinline__ double coarse_row_abs(const CoarseDev& c, int64_t v) {
  const float dv = c.dinv[v];
  if (!(dv > 0.f)) return 0.0;
  double y = 0.0;
  for (int k = c.rowptr[v]; k < c.rowptr[v + 1]; ++k) y += fabs((double)c.val[k]) * sqrt((double)c.dinv[c.col[k]]);
  return y * sqrt((double)dv);
}

__device__ void block_max(double v, double* partials, int slot) {
  __shared__ double red[kT / 32];
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s = fmax(s, red[w]);
    partials[(size_t)slot * gridDim.x + blockIdx.x] = s;
  }
  __syncthreads();
}

// per-block maxima of the absolute row sums (slot 0)
__global__ void coarse_row_bound(CoarseDev c, double* partials) {
  double g = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < c.nV; i += (int64_t)gridDim.x * blockDim.x)
    g = fmax(g, coarse_row_abs(c, i));
  block_max(g, partials, 0);
}


// ---- coarse solve

// rc = P^T r (interior faces); Chebyshev start: cr = rc, d0 = D^{-1} rc / theta, yc = 0
template <typename T>
__global__ void coarse_restrict(CoarseDev c, const T* __restrict__ r, const int* skip, float d0scale) {
  if (skip && *skip) return;
  const int d = c.dim, NF = c.NF;
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < c.nV; v += (int64_t)gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int j = c.rptr[v]; j < c.rptr[v + 1]; ++j) {
      const int fk = c.ridx[j];
      const int64_t f = fk / d;
      const int k = fk - (int)f * d;
      if (c.isBnd[f]) continue;
      const T* rf = r + f * NF;
      for (int a = 0; a < NF; ++a) s = fmaf(c.Wf[a * d + k], (float)rf[a], s);
    }
    c.rc[v] = s;
    c.cr[v] = s;
    c.yc[v] = 0.f;
    c.cd0[v] = c.dinv[v] * s * d0scale;
  }
}

// One Chebyshev step: yc += d_k, r -= A d_k, d_{k+1} = c1 d_k + c2 D^{-1} r
__global__ void coarse_cheb_step(CoarseDev c, const float* __restrict__ dk, float* __restrict__ dn, float c1, float c2,
                                 int last, const int* skip) {
  if (skip && *skip) return;
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < c.nV; v += (int64_t)gridDim.x * blockDim.x) {
    const float dv = dk[v];
    c.yc[v] += dv;
    if (last) continue;
    const float y = ell_row(c, v, dk);
    const float r = c.cr[v] - y;
    c.cr[v] = r;
    dn[v] = c1 * dv + c2 * c.dinv[v] * r;
  }
}

// ---- one-launch coarse solve: restriction and all Chebyshev steps in a
// cooperative kernel (every block resident), separated by a grid barrier.

constexpr int kMaxDegree = 64;
constexpr long long kBarrierSpin = 1LL << 22;  // about a second: then the error flag

struct ChebSchedule {
  float c1[kMaxDegree], c2[kMaxDegree];
  float d0scale;
  int degree;
};

// Grid-wide barrier with a bounded wait. The arrival counter starts each launch
// at 0 and only grows within it: the k-th barrier completes when it reaches
// k * gridDim.x. Arrival is a release add, the wait an acquire load; a wait that
// runs out sets *error and returns (never spins forever).
__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void red_release_add(unsigned* p, unsigned v) {
  asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Once any wait has run out (*error set) the later barriers of the solve return
// at once: its iterates are invalid anyway and the host restarts without them.
// withhold: this block does not arrive (the test hook that makes the wait run out).
__device__ __forceinline__ void grid_barrier(unsigned* count, unsigned target, int* error, bool withhold = false) {
  __syncthreads();
  if (threadIdx.x == 0) {
    if (!withhold) red_release_add(count, 1u);
    long long it = 0;
    while ((int)(ld_acquire(count) - target) < 0) {
      if (*(volatile int*)error) break;
      if (++it > kBarrierSpin) {
        atomicExch(error, 1);
        break;
      }
    }
  }
  __syncthreads();
}

// CLUSTER: the grid is one thread-block cluster (small coarse spaces: at most 8 CTAs of
// 1024 threads) and the steps are separated by the hardware cluster barrier (release /
// acquire at cluster scope, so the global writes of one step are visible to every CTA of
// the cluster in the next; vectors written in the launch are read through L2, __ldcg).
// Every thread reaches every barrier: the only early exit is the skip flag, which is the
// same for all (set before the launch).
__device__ __forceinline__ void cluster_sync_all() {
  __syncwarp();  // the .aligned barrier wants the warp converged
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// Four lanes per coarse row: the restriction splits the row's incident faces
// and every step splits the ELL slots between them (a shuffle sum joins them),
// which shortens each lane's chain of dependent L2 loads four-fold.
constexpr int kCoarseLanes = 4;
template <typename T, bool CLUSTER = false>
__global__ void __launch_bounds__(CLUSTER ? 1024 : 512) coarse_solve_coop(CoarseDev c, const T* __restrict__ r,
                                                                          const int* skip, ChebSchedule cs) {
  if (skip && *skip) return;  // the same value for every block: set before this launch
  // barrier[0] counts arrivals and starts every launch at 0: the last block to
  // leave (counted in barrier[1]) resets both, after every wait has finished
  const int d = c.dim, NF = c.NF;
  const int sub = threadIdx.x % kCoarseLanes;
  const int64_t groups = (int64_t)gridDim.x * (blockDim.x / kCoarseLanes);
  const int64_t g0 = (int64_t)blockIdx.x * (blockDim.x / kCoarseLanes) + threadIdx.x / kCoarseLanes;
  // rows are walked in whole warps so that every lane reaches the shuffles
  const int64_t nVr = (c.nV + 7) / 8 * 8;
  for (int64_t v = g0; v < nVr; v += groups) {
    float s = 0.f;
    if (v < c.nV)
      for (int j = c.rptr[v] + sub; j < c.rptr[v + 1]; j += kCoarseLanes) {
        const int fk = c.ridx[j];
        const int64_t f = fk / d;
        const int k = fk - (int)f * d;
        if (c.isBnd[f]) continue;
        const T* rf = r + f * NF;
        for (int a = 0; a < NF; ++a) s = fmaf(c.Wf[a * d + k], (float)rf[a], s);
      }
    s += __shfl_xor_sync(0xffffffffu, s, 1);
    s += __shfl_xor_sync(0xffffffffu, s, 2);
    if (sub == 0 && v < c.nV) {
      c.rc[v] = s;
      c.cr[v] = s;
      c.yc[v] = 0.f;
      c.cd0[v] = c.dinv[v] * s * cs.d0scale;
    }
  }
  float* dk = c.cd0;
  float* dn = c.cd1;
  bool withhold = false;
  if (!CLUSTER && c.testHold && blockIdx.x == 0 && threadIdx.x == 0) withhold = atomicExch(c.testHold, 0) != 0;
  for (int k = 0; k < cs.degree; ++k) {
    if (CLUSTER)
      cluster_sync_all();
    else
      grid_barrier(c.barrier, (unsigned)(k + 1) * gridDim.x, c.error, k == 0 && withhold);
    const bool last = k + 1 == cs.degree;
    for (int64_t v = g0; v < nVr; v += groups) {
      float y = 0.f;
      if (!last && v < c.nV) {
        int cc[4];
        float aa[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int slot = sub + u * kCoarseLanes;
          const bool in = slot < c.ellW;
          cc[u] = in ? c.ellCol[(int64_t)slot * c.nV + v] : (int)v;
          aa[u] = in ? c.ellVal[(int64_t)slot * c.nV + v] : 0.f;
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) y = fmaf(aa[u], __ldcg(dk + cc[u]), y);
        for (int slot = sub + 16; slot < c.ellW; slot += kCoarseLanes)
          y = fmaf(c.ellVal[(int64_t)slot * c.nV + v], __ldcg(dk + c.ellCol[(int64_t)slot * c.nV + v]), y);
      }
      y += __shfl_xor_sync(0xffffffffu, y, 1);
      y += __shfl_xor_sync(0xffffffffu, y, 2);
      if (sub == 0 && v < c.nV) {
        const float dv = __ldcg(dk + v);
        c.yc[v] += dv;
        if (!last) {
          const float rr = c.cr[v] - y;
          c.cr[v] = rr;
          dn[v] = cs.c1[k] * dv + cs.c2[k] * c.dinv[v] * rr;
        }
      }
    }
    float* t = dk;
    dk = dn;
    dn = t;
  }
  if (CLUSTER) return;  // yc is complete at the end of the launch (kernel boundary)
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned left = atomicAdd(c.barrier + 1, 1u) + 1u;
    if (left == gridDim.x) {
      atomicExch(c.barrier, 0u);
      atomicExch(c.barrier + 1, 0u);
    }
  }
}

// The Lanczos steps of coarse_setup in one cooperative launch, one grid barrier per step.
// Step j reads w_{j-1} and v_{j-1} (written by every block in step j-1) and forms
// v_j = (w_{j-1} - alpha_{j-1} v_{j-1}) / beta_{j-1} where it needs it, on the fly for
// the neighbour columns of its rows; it writes its rows of v_j and
// w_j = A v_j - beta_{j-1} v_{j-1} into the other pair of buffers, with the partial
// sums of w_j . v_j, |w_j|^2 and |v_j|^2 (the next beta as in lanczos_apply). The
// vectors are stored times D^{-1/2} (A here is D^{-1/2} A_c D^{-1/2}), so a row gathers
// its neighbours' stored values and multiplies the ELL row of A_c by them. The partial
// sums alternate between two sets by step parity, so a set is rewritten only after every
// block has passed the next barrier, i.e. has read it. Vectors written by other blocks are
// read through L2 (__ldcg). out: alpha[m], beta[m], the step count, the start norm and the
// row-sum bound.

// totals of three consecutive slots of block partials (gridDim.x values each), summed by
// every thread of the block in the same order
__device__ __forceinline__ void grid_sum3(const double* p, double* t0, double* t1, double* t2) {
  __shared__ double red[3][kT / 32];
  const unsigned g = gridDim.x;
  double a0 = 0.0, a1 = 0.0, a2 = 0.0;
  for (unsigned b = threadIdx.x; b < g; b += blockDim.x) {
    a0 += __ldcg(p + b);
    a1 += __ldcg(p + g + b);
    a2 += __ldcg(p + 2 * g + b);
  }
  for (int o = 16; o > 0; o >>= 1) {
    a0 += __shfl_down_sync(0xffffffffu, a0, o);
    a1 += __shfl_down_sync(0xffffffffu, a1, o);
    a2 += __shfl_down_sync(0xffffffffu, a2, o);
  }
  if ((threadIdx.x & 31) == 0) {
    red[0][threadIdx.x >> 5] = a0;
    red[1][threadIdx.x >> 5] = a1;
    red[2][threadIdx.x >> 5] = a2;
  }
  __syncthreads();
  double s0 = 0.0, s1 = 0.0, s2 = 0.0;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
    s0 += red[0][w];
    s1 += red[1][w];
    s2 += red[2][w];
  }
  __syncthreads();  // red is rewritten by the next call
  *t0 = s0;
  *t1 = s1;
  *t2 = s2;
}

// total of one slot of block partials, by every thread of the block
__device__ __forceinline__ double grid_sum1(const double* p) {
  __shared__ double red[kT / 32];
  double a = 0.0;
  for (unsigned b = threadIdx.x; b < gridDim.x; b += blockDim.x) a += __ldcg(p + b);
  for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = a;
  __syncthreads();
  double r = 0.0;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) r += red[w];
  __syncthreads();
  return r;
}

// maximum of one slot of block partials, by every thread of the block
__device__ __forceinline__ double grid_max1(const double* p) {
  __shared__ double red[kT / 32];
  double a = 0.0;
  for (unsigned b = threadIdx.x; b < gridDim.x; b += blockDim.x) a = fmax(a, __ldcg(p + b));
  for (int o = 16; o > 0; o >>= 1) a = fmax(a, __shfl_down_sync(0xffffffffu, a, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = a;
  __syncthreads();
  double r = 0.0;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) r = fmax(r, red[w]);
  __syncthreads();
  return r;
}

__device__ void block_partial3(double a, double b, double c, double* p) {
  __shared__ double red[3][kT / 32];
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, o);
    b += __shfl_down_sync(0xffffffffu, b, o);
    c += __shfl_down_sync(0xffffffffu, c, o);
  }
  if ((threadIdx.x & 31) == 0) {
    red[0][threadIdx.x >> 5] = a;
    red[1][threadIdx.x >> 5] = b;
    red[2][threadIdx.x >> 5] = c;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double s0 = 0.0, s1 = 0.0, s2 = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      s0 += red[0][w];
      s1 += red[1][w];
      s2 += red[2][w];
    }
    p[blockIdx.x] = s0;
    p[gridDim.x + blockIdx.x] = s1;
    p[2 * gridDim.x + blockIdx.x] = s2;
  }
  __syncthreads();
}

// partials: 6 gridDim.x values (two sets of three slots)
__global__ void __launch_bounds__(kT) lanczos_coop(CoarseDev c, int m, float* va, float* vb, float* wa, float* wb,
                                                   double* out) {
  unsigned nb = 0;  // barriers passed in this launch
  const int64_t i0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, stride = (int64_t)gridDim.x * blockDim.x;
  double* const P0 = c.partials;
  double* const P1 = c.partials + 3 * (size_t)gridDim.x;
  // step -1: w = the start vector (wa), v = 0 (vb), alpha = 0, beta = its norm
  double ss = 0.0, gmax = 0.0;
  for (int64_t i = i0; i < c.nV; i += stride) {
    uint32_t h = (uint32_t)i * 2654435761u + 12345u;
    h ^= h >> 13;
    h *= 0x5bd1e995u;
    h ^= h >> 15;
    const float x = c.dinv[i] > 0.f ? 0.5f + (float)(h & 0xffff) / 65536.f : 0.f;
    wa[i] = x * sqrtf(c.dinv[i]);
    vb[i] = 0.f;
    ss += (double)x * x;
    gmax = fmax(gmax, coarse_row_abs(c, i));
  }
  // the start vector's sums in set 1: the first write to set 1 (step 1) follows the
  // barrier of step 0, which every block reaches after reading them
  block_partial(ss, P1, 0);
  block_max(gmax, P1, 1);
  grid_barrier(c.barrier, ++nb * gridDim.x, c.error);
  const double nrm = sqrt(grid_sum1(P1));
  if (blockIdx.x == 0) {
    const double g = grid_max1(P1 + gridDim.x);
    if (threadIdx.x == 0) out[2 * m + 2] = g;
  }
  int steps = 0;
  if (nrm > 0.0) {
    double alpha = 0.0, beta = nrm;
    const float *wr = wa, *vr = vb;  // w_{j-1}, v_{j-1}
    float *wn = wb, *vn = va;        // w_j, v_j
    for (int j = 0; j < m; ++j) {
      const float fa = (float)alpha, ib = (float)(1.0 / beta), fb = (float)beta;
      double a = 0.0, ww = 0.0, vv = 0.0;
      for (int64_t i = i0; i < c.nV; i += stride) {
        float y = 0.f, vi = 0.f, vti = 0.f, si = 0.f;
        if (c.dinv[i] > 0.f) {
          si = sqrtf(c.dinv[i]);
          // the row from the ELL copy, eight neighbours' loads in flight at a time
          const int W = c.ellW;
          int k = 0;
          for (; k + 8 <= W; k += 8) {
            int cc[8];
            float aa[8], xx[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
              cc[u] = c.ellCol[(int64_t)(k + u) * c.nV + i];
              aa[u] = c.ellVal[(int64_t)(k + u) * c.nV + i];
            }
#pragma unroll
            for (int u = 0; u < 8; ++u) xx[u] = (__ldcg(wr + cc[u]) - fa * __ldcg(vr + cc[u])) * ib;
#pragma unroll
            for (int u = 0; u < 8; ++u) y = fmaf(aa[u], xx[u], y);
          }
          for (; k < W; ++k) {
            const int cc = c.ellCol[(int64_t)k * c.nV + i];
            y = fmaf(c.ellVal[(int64_t)k * c.nV + i], (__ldcg(wr + cc) - fa * __ldcg(vr + cc)) * ib, y);
          }
          const float is = 1.f / si;
          vti = (__ldcg(wr + i) - fa * __ldcg(vr + i)) * ib;
          vi = vti * is;
          y = y * si - fb * (__ldcg(vr + i) * is);
        }
        wn[i] = y * si;
        vn[i] = vti;
        a += (double)y * vi;
        ww += (double)y * y;
        vv += (double)vi * vi;
      }
      double* const P = (j & 1) ? P1 : P0;
      block_partial3(a, ww, vv, P);
      grid_barrier(c.barrier, ++nb * gridDim.x, c.error);
      double al, wsum, vsum;
      grid_sum3(P, &al, &wsum, &vsum);
      if (blockIdx.x == 0 && threadIdx.x == 0) out[j] = al;
      steps = j + 1;
      // |w - alpha v| with the computed |v|^2 (lanczos_apply)
      const double bn = sqrt(fmax(wsum - al * al * (2.0 - vsum), 0.0));
      if (j + 1 == m || bn < 1e-6 * sqrt(wsum)) break;
      if (blockIdx.x == 0 && threadIdx.x == 0) out[m + j] = bn;
      alpha = al;
      beta = bn;
      const float *tw = wr, *tv = vr;
      wr = wn;
      vr = vn;
      wn = const_cast<float*>(tw);
      vn = const_cast<float*>(tv);
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    out[2 * m] = (double)steps;
    out[2 * m + 1] = nrm;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned left = atomicAdd(c.barrier + 1, 1u) + 1u;
    if (left == gridDim.x) {
      atomicExch(c.barrier, 0u);
      atomicExch(c.barrier + 1, 0u);
    }
  }
}

template <typename T>
__global__ void coarse_prolong(CoarseDev c, T* __restrict__ x) {
  const int d = c.dim, NF = c.NF;
  const int64_t n = c.nFaces * NF;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t f = i / NF;
    const int a = (int)(i - f * NF);
    if (c.isBnd[f]) continue;
    float s = 0.f;
    for (int k = 0; k < d; ++k) s = fmaf(c.Wf[a * d + k], c.yc[c.faceV[f * d + k]], s);
    x[i] += (T)s;
  }
}

// ---- learned coarse polynomial: forward and backward kernels.
// Samples and every intermediate are [S][nV] (sample s contiguous). The model
// propagates coarse errors U through the Richardson steps,
// U_{k+1} = U_k - theta_k D^{-1} A_c U_k, and the loss is their energy after K
// steps, L = sum_s w_s U_K[s]^T A_c U_K[s], w_s = 1 / (S U_0[s]^T A_c U_0[s]):
// the A_c-norm error reduction of the coarse solve on the solver's own coarse
// errors (U_0 = A_c^{-1} P^T r from its Krylov residuals r).

__device__ __forceinline__ float ell_row_plain(const CoarseDev& c, int64_t v, const float* x) {
  float y = 0.f;
  for (int k = 0; k < c.ellW; ++k)
    y = fmaf(c.ellVal[(int64_t)k * c.nV + v], x[c.ellCol[(int64_t)k * c.nV + v]], y);
  return y;
}

__device__ __forceinline__ void block_sum_to(double v, double* out) {
  __shared__ double red[kT / 32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
    *out = t;
  }
  __syncthreads();
}

// grid (Gx, S). AX = A X; partials of X . AX per sample at partials[s * Gx + bx]
__global__ void learn_energy(CoarseDev c, const float* X, float* AX, double* partials) {
  const int sm = blockIdx.y;
  const float* x = X + (int64_t)sm * c.nV;
  double acc = 0.0;
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < c.nV; v += (int64_t)gridDim.x * blockDim.x) {
    const float y = c.dinv[v] > 0.f ? ell_row_plain(c, v, x) : 0.f;
    AX[(int64_t)sm * c.nV + v] = y;
    acc += (double)x[v] * y;
  }
  block_sum_to(acc, partials + (int64_t)sm * gridDim.x + blockIdx.x);
}

// Y = D^{-1} A X, Xn = X - theta Y
__global__ void learn_fwd(CoarseDev c, const float* X, float* Y, float* Xn, float theta) {
  const int sm = blockIdx.y;
  const float* x = X + (int64_t)sm * c.nV;
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < c.nV; v += (int64_t)gridDim.x * blockDim.x) {
    const float y = c.dinv[v] > 0.f ? c.dinv[v] * ell_row_plain(c, v, x) : 0.f;
    Y[(int64_t)sm * c.nV + v] = y;
    Xn[(int64_t)sm * c.nV + v] = x[v] - theta * y;
  }
}

// loss partials w_s U . AU and the adjoint seed G = 2 w_s AU (AU from learn_energy)
__global__ void learn_seed(CoarseDev c, const float* U, const float* AU, const double* w, float* G, double* partials) {
  const int sm = blockIdx.y;
  const double ws = w[sm];
  double acc = 0.0;
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < c.nV; v += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = (int64_t)sm * c.nV + v;
    acc += ws * (double)U[i] * AU[i];
    G[i] = (float)(2.0 * ws * AU[i]);
  }
  block_sum_to(acc, partials + (int64_t)sm * gridDim.x + blockIdx.x);
}

// dL/dtheta_k partials = -sum G_{k+1} . Y_k, and G_k = G_{k+1} - theta_k A_c D^{-1} G_{k+1}
__global__ void learn_bwd(CoarseDev c, const float* G, const float* Yk, float* Gn, float theta, double* partials) {
  const int sm = blockIdx.y;
  const float* g = G + (int64_t)sm * c.nV;
  double acc = 0.0;
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < c.nV; v += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = (int64_t)sm * c.nV + v;
    acc -= (double)g[v] * Yk[i];
    float ag = 0.f;
    if (c.dinv[v] > 0.f)
      for (int k = 0; k < c.ellW; ++k) {
        const int col = c.ellCol[(int64_t)k * c.nV + v];
        ag = fmaf(c.ellVal[(int64_t)k * c.nV + v] * c.dinv[col], g[col], ag);
      }
    Gn[i] = g[v] - theta * ag;
  }
  block_sum_to(acc, partials + (int64_t)sm * gridDim.x + blockIdx.x);
}

// batched Chebyshev step on coarse vectors (errors of the training samples):
// Y += D_k; R -= A D_k; D_{k+1} = c1 D_k + c2 D^{-1} R
__global__ void learn_cheb(CoarseDev c, const float* Dk, float* Dn, float* R, float* Y, float c1, float c2, int last) {
  const int sm = blockIdx.y;
  const float* d = Dk + (int64_t)sm * c.nV;
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < c.nV; v += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = (int64_t)sm * c.nV + v;
    Y[i] += d[v];
    if (last) continue;
    const float ad = c.dinv[v] > 0.f ? ell_row_plain(c, v, d) : 0.f;
    const float r = R[i] - ad;
    R[i] = r;
    Dn[i] = c1 * d[v] + c2 * c.dinv[v] * r;
  }
}

__global__ void learn_cheb_start(CoarseDev c, const float* R, float* D0, float* Y, float scale) {
  const int sm = blockIdx.y;
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < c.nV; v += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = (int64_t)sm * c.nV + v;
    D0[i] = c.dinv[v] * R[i] * scale;
    Y[i] = 0.f;
  }
}

struct LearnWork {
  float *E, *Y, *G0, *G1;
  double *w, *part;
  int Gx;
};

// Forward and backward pass for theta (unscaled): loss and dL/dtheta.
cudaError_t learn_pass(const CoarseDev& c, const LearnWork& lw, int S, int K, const double* theta, double* loss,
                       double* grad, std::vector<double>& hp, cudaStream_t s) {
  const int64_t nV = c.nV;
  const dim3 grid(lw.Gx, S);
  for (int k = 0; k < K; ++k)
    learn_fwd<<<grid, kT, 0, s>>>(c, lw.E + (int64_t)k * S * nV, lw.Y + (int64_t)k * S * nV,
                                  lw.E + (int64_t)(k + 1) * S * nV, (float)theta[k]);
  // A U_K into G1, then the loss and the seed G0
  learn_energy<<<grid, kT, 0, s>>>(c, lw.E + (int64_t)K * S * nV, lw.G1, lw.part);
  learn_seed<<<grid, kT, 0, s>>>(c, lw.E + (int64_t)K * S * nV, lw.G1, lw.w, lw.G0, lw.part);
  float *g = lw.G0, *gn = lw.G1;
  for (int k = K - 1; k >= 0; --k) {
    learn_bwd<<<grid, kT, 0, s>>>(c, g, lw.Y + (int64_t)k * S * nV, gn, (float)theta[k],
                                  lw.part + (int64_t)(k + 1) * S * lw.Gx);
    std::swap(g, gn);
  }
  const size_t np = (size_t)(K + 1) * S * lw.Gx;
  hp.resize(np);
  cudaError_t e = cudaMemcpyAsync(hp.data(), lw.part, sizeof(double) * np, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return e;
  const size_t slot = (size_t)S * lw.Gx;
  double L = 0.0;
  for (size_t i = 0; i < slot; ++i) L += hp[i];
  *loss = L;
  for (int k = 0; k < K; ++k) {
    double gk = 0.0;
    for (size_t i = 0; i < slot; ++i) gk += hp[(k + 1) * slot + i];
    grad[k] = gk;
  }
  return cudaSuccess;
}

// Work buffers; E_0 = the error samples [S][nV] and their weights.
cudaError_t learn_setup(const CoarseDev& c, const float* samples, int S, int K, LearnWork* lw, cudaStream_t s) {
  const int64_t nV = c.nV;
  lw->Gx = (int)std::min<int64_t>((nV + kT - 1) / kT, 64);
  cudaError_t e;
  if ((e = cudaMalloc(&lw->E, sizeof(float) * (size_t)(K + 1) * S * nV)) != cudaSuccess) return e;
  if ((e = cudaMalloc(&lw->Y, sizeof(float) * (size_t)std::max(K, 1) * S * nV)) != cudaSuccess) return e;
  if ((e = cudaMalloc(&lw->G0, sizeof(float) * (size_t)S * nV)) != cudaSuccess) return e;
  if ((e = cudaMalloc(&lw->G1, sizeof(float) * (size_t)S * nV)) != cudaSuccess) return e;
  if ((e = cudaMalloc(&lw->w, sizeof(double) * S)) != cudaSuccess) return e;
  if ((e = cudaMalloc(&lw->part, sizeof(double) * (size_t)(K + 1) * S * lw->Gx)) != cudaSuccess) return e;
  cudaMemcpyAsync(lw->E, samples, sizeof(float) * (size_t)S * nV, cudaMemcpyDeviceToDevice, s);
  learn_energy<<<dim3(lw->Gx, S), kT, 0, s>>>(c, lw->E, lw->G1, lw->part);
  std::vector<double> hp((size_t)S * lw->Gx), w(S);
  cudaMemcpyAsync(hp.data(), lw->part, sizeof(double) * hp.size(), cudaMemcpyDeviceToHost, s);
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
  for (int sm = 0; sm < S; ++sm) {
    double t = 0.0;
    for (int b = 0; b < lw->Gx; ++b) t += hp[(size_t)sm * lw->Gx + b];
    w[sm] = t > 0.0 ? 1.0 / (t * S) : 0.0;  // every sample weighs 1/S
  }
  cudaMemcpyAsync(lw->w, w.data(), sizeof(double) * S, cudaMemcpyHostToDevice, s);
  return cudaGetLastError();
}

void learn_free(LearnWork* lw) {
  cudaFree(lw->E);
  cudaFree(lw->Y);
  cudaFree(lw->G0);
  cudaFree(lw->G1);
  cudaFree(lw->w);
  cudaFree(lw->part);
}

// Soft constraint keeping the residual polynomial below 1 on [0, lhi]: penalty
// P = 100 mean_i relu(q(lambda_i) - 0.999)^2 on a grid and its gradient in theta.
double poly_penalty(const std::vector<double>& theta, double lhi, std::vector<double>* grad) {
  const int K = (int)theta.size(), n = 1024;
  double P = 0.0;
  grad->assign(K, 0.0);
  for (int i = 1; i <= n; ++i) {
    const double l = lhi * i / n;
    double q = 1.0;
    for (double t : theta) q *= 1.0 - t * l;
    const double ex = q - 0.999;
    if (ex <= 0.0) continue;
    P += ex * ex;
    for (int k = 0; k < K; ++k) {
      double dq = -l;  // d/dtheta_k of prod_j (1 - theta_j l)
      for (int j = 0; j < K; ++j)
        if (j != k) dq *= 1.0 - theta[j] * l;
      (*grad)[k] += 2.0 * ex * dq;
    }
  }
  const double sc = 100.0 / n;
  for (auto& g : *grad) g *= sc;
  return P * sc;
}

// max over [0, lhi] of prod_k (1 - theta_k lambda) (the coarse solve stays
// positive semidefinite when this is <= 1 on the spectrum; lhi is the upper
// Chebyshev bound, 1.1 x the largest Lanczos Ritz value)
double poly_max(const std::vector<double>& theta, double lhi) {
  double m = -1e300;
  for (int i = 0; i <= 4096; ++i) {
    const double l = lhi * i / 4096.0;
    double q = 1.0;
    for (double t : theta) q *= 1.0 - t * l;
    m = std::max(m, q);
  }
  return m;
}

// Sturm count: number of eigenvalues of the tridiagonal (a, b) below x.
int sturm_below(const std::vector<double>& a, const std::vector<double>& b, double x) {
  int cnt = 0;
  double q = 1.0;
  for (size_t i = 0; i < a.size(); ++i) {
    double bb = i ? b[i - 1] * b[i - 1] : 0.0;
    q = a[i] - x - (i ? bb / q : 0.0);
    if (q == 0.0) q = 1e-300;
    if (q < 0) ++cnt;
  }
  return cnt;
}

double tridiag_eig(const std::vector<double>& a, const std::vector<double>& b, int k) {
  double lo = 1e300, hi = -1e300;
  for (size_t i = 0; i < a.size(); ++i) {
    double r = (i ? std::fabs(b[i - 1]) : 0.0) + (i + 1 < a.size() ? std::fabs(b[i]) : 0.0);
    lo = std::min(lo, a[i] - r);
    hi = std::max(hi, a[i] + r);
  }
  for (int it = 0; it < 200; ++it) {
    double mid = 0.5 * (lo + hi);
    if (sturm_below(a, b, mid) > k) hi = mid;
    else lo = mid;
  }
  return 0.5 * (lo + hi);
}

double sum_partials(const double* h, int n) {
  double s = 0.0;
  for (int i = 0; i < n; ++i) s += h[i];
  return s;
}

}  // namespace

template <typename T>
cudaError_t coarse_setup(CoarseSolver* cs, const T* S, int maxDegree, double target, cudaStream_t s) {
  CoarseDev* c = &cs->dev;
  cs->ready = false;
  const unsigned gE = blocks_for(c->nCells * 32);
  if (c->NV1 == 3) coarse_elem<T, 3><<<gE, kT, 0, s>>>(*c, S);
  else coarse_elem<T, 4><<<gE, kT, 0, s>>>(*c, S);
  coarse_gather<<<blocks_for(c->nV), kT, 0, s>>>(*c);
  coarse_fill_ell<<<blocks_for((int64_t)c->ellW * c->nV), kT, 0, s>>>(*c);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  // Lanczos, m steps, on D^{-1/2} A_c D^{-1/2}; three partial sums per block fit the partials buffer
  const unsigned g = std::min<unsigned>(blocks_for(c->nV), (152 * 32 + 64) / 3);
  std::vector<double> hp(3 * g);
  float *v = c->cd0, *vprev = c->cd1, *w = c->lz;
  const int m = (int)std::min<int64_t>(30, c->nV);
  std::vector<double> al, be;
  double rowBound = 0.0;  // infinity norm of D^{-1/2} A_c D^{-1/2}
  {
    // one cooperative launch (grid-stride over the rows; six partial sums per block fit the
    // partials buffer) where the device has cooperative launches
    int dev = 0, coop = 0, nsm = 0, perSM = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (coop && c->barrier && c->lanczosOut &&
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, lanczos_coop, kT, 0) == cudaSuccess && perSM >= 1) {
      const unsigned gc = (unsigned)std::min<int64_t>(std::min<int64_t>(g, (152 * 32 + 64) / 6), (int64_t)perSM * nsm);
      CoarseDev cv = *c;
      int mm = m;
      float *a0 = c->cd0, *a1 = c->cd1, *a2 = c->lz, *a3 = c->cr;  // cr: coarse-solve work, free here
      double* o = c->lanczosOut;
      void* args[] = {&cv, &mm, &a0, &a1, &a2, &a3, &o};
      std::vector<double> ho(2 * m + 3);
      int herr = 0;
      const bool launched =
          cudaLaunchCooperativeKernel((const void*)lanczos_coop, dim3(gc), dim3(kT), args, 0, s) == cudaSuccess;
      if (!launched) {
        cudaGetLastError();  // not launched: the launch-per-step loop below does the steps
      } else {
        cudaMemcpyAsync(ho.data(), c->lanczosOut, sizeof(double) * (2 * m + 3), cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(&herr, c->error, sizeof(int), cudaMemcpyDeviceToHost, s);
        if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
      }
      if (launched && herr == 0) {
        const int steps = (int)ho[2 * m];
        if (!(ho[2 * m + 1] > 0)) {
          cs->lmin = cs->lmax = 1.0;
          cs->degree = 0;
          cs->ready = true;
          return cudaSuccess;
        }
        al.assign(ho.begin(), ho.begin() + steps);
        be.assign(ho.begin() + m, ho.begin() + m + std::max(steps - 1, 0));
        rowBound = ho[2 * m + 2];
      } else if (launched) {
        // a barrier wait ran out: clear the flag and redo the steps one launch at a time
        cudaMemsetAsync(c->error, 0, sizeof(int), s);
        cudaMemsetAsync(c->barrier, 0, 2 * sizeof(unsigned), s);
      }
    }
  }
  if (al.empty()) {
  coarse_row_bound<<<g, kT, 0, s>>>(*c, c->partials);
  cudaMemcpyAsync(hp.data(), c->partials, sizeof(double) * g, cudaMemcpyDeviceToHost, s);
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
  rowBound = 0.0;
  for (unsigned b = 0; b < g; ++b) rowBound = std::max(rowBound, hp[b]);
  cudaMemsetAsync(vprev, 0, sizeof(float) * c->nV, s);
  lanczos_init<<<g, kT, 0, s>>>(*c, v, c->partials);
  cudaMemcpyAsync(hp.data(), c->partials, sizeof(double) * g, cudaMemcpyDeviceToHost, s);
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
  double nrm = std::sqrt(sum_partials(hp.data(), g));
  if (!(nrm > 0)) {
    cs->lmin = cs->lmax = 1.0;
    cs->degree = 0;
    cs->ready = true;
    return cudaSuccess;
  }
  lanczos_scale<<<g, kT, 0, s>>>(c->nV, v, (float)(1.0 / nrm));
  double beta = 0.0;
  for (int j = 0; j < m; ++j) {
    // one host round trip per step: alpha, |w|^2 and |v|^2 from the same pass
    lanczos_apply<<<g, kT, 0, s>>>(*c, v, vprev, (float)beta, w, c->partials);
    cudaMemcpyAsync(hp.data(), c->partials, sizeof(double) * 3 * g, cudaMemcpyDeviceToHost, s);
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
    const double alpha = sum_partials(hp.data(), g);
    const double ww = sum_partials(hp.data() + g, g);
    const double vv = sum_partials(hp.data() + 2 * g, g);
    al.push_back(alpha);
    beta = std::sqrt(std::max(ww - alpha * alpha * (2.0 - vv), 0.0));
    if (j + 1 == m || beta < 1e-6 * std::sqrt(ww)) break;
    be.push_back(beta);
    lanczos_next<<<g, kT, 0, s>>>(c->nV, v, (float)alpha, (float)(1.0 / beta), w);
    float* t = vprev;
    vprev = v;
    v = w;
    w = t;
  }
  be.resize(al.size() > 0 ? al.size() - 1 : 0);
  }
  const double tmin = tridiag_eig(al, be, 0), tmax = tridiag_eig(al, be, (int)al.size() - 1);
  // upper bound must cover the spectrum (|p| <= 1 there keeps q(A_c) SPD): the largest
  // Ritz value is below the spectral radius, the row-sum norm above it, so the margin on the
  // Ritz value is capped by the norm; the lower end may be above the true minimum: modes
  // below it are damped less
  cs->ritzMin = tmin;
  cs->ritzMax = tmax;
  cs->rowBound = rowBound;
  cs->lmax = rowBound > 0.0 ? std::min(1.1 * tmax, rowBound) : 1.1 * tmax;
  cs->lmin = std::max(tmin / 1.5, cs->lmax * 1e-6);
  const double th = 0.5 * (cs->lmax + cs->lmin), de = 0.5 * (cs->lmax - cs->lmin);
  const double sig = th / de;
  int K = (int)std::ceil(std::acosh(1.0 / target) / std::acosh(sig));
  K = std::max(1, std::min(K, maxDegree));
  cs->degree = K;
  c->theta = (float)th;
  cs->c1.assign(K, 0.f);
  cs->c2.assign(K, 0.f);
  double rho = 1.0 / sig;
  for (int k = 0; k < K; ++k) {
    double rho1 = 1.0 / (2.0 * sig - rho);
    cs->c1[k] = (float)(rho1 * rho);
    cs->c2[k] = (float)(2.0 * rho1 / de);
    rho = rho1;
  }
  // one-launch solve: every block must be resident (cooperative launch)
  cs->coopGrid = 0;
  int dev = 0, coop = 0, nsm = 0, perSM = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  if (coop && c->barrier && K <= kMaxDegree &&
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, coarse_solve_coop<double>, 512, 0) == cudaSuccess &&
      perSM >= 1) {
    // 128 rows per block of 512 threads; every block must be resident at once
    int64_t want = (c->nV + 127) / 128;
    int g = (int)std::min<int64_t>(want, (int64_t)nsm * std::min(perSM, 2));
    cs->coopGrid = std::max(g, 1);
  }
  // small coarse spaces: one cluster of up to 8 CTAs of 1024 threads (256 rows each per pass,
  // at most two passes per step), hardware cluster barriers between the steps
  cs->clusterGrid = 0;
  int clusterOk = 0;
  cudaDeviceGetAttribute(&clusterOk, cudaDevAttrClusterLaunch, dev);
  if (clusterOk && K <= kMaxDegree && c->nV <= 4096) {
    const int g = (int)std::min<int64_t>(8, (c->nV + 255) / 256);
    cs->clusterGrid = std::max(g, 1);
  }
  cs->ready = true;
  return cudaGetLastError();
}

static ChebSchedule poly_schedule(const CoarseSolver& cs) {
  ChebSchedule sch{};
  if (cs.useLearned && !cs.thetaHat.empty()) {
    // Richardson steps with the learned weights
    const int K = (int)cs.thetaHat.size();
    sch.degree = K;
    sch.d0scale = (float)(cs.thetaHat[0] / cs.lmax);
    for (int k = 0; k < K; ++k) {
      sch.c1[k] = 0.f;
      sch.c2[k] = k + 1 < K ? (float)(cs.thetaHat[k + 1] / cs.lmax) : 0.f;
    }
    return sch;
  }
  sch.degree = cs.degree;
  sch.d0scale = 1.0f / cs.dev.theta;
  for (int k = 0; k < cs.degree; ++k) {
    sch.c1[k] = cs.c1[k];
    sch.c2[k] = cs.c2[k];
  }
  return sch;
}

template <typename T>
cudaError_t coarse_apply(const CoarseSolver& cs, const T* r, const int* skip, cudaStream_t s) {
  const CoarseDev& c = cs.dev;
  const ChebSchedule sch = poly_schedule(cs);
  if (cs.clusterGrid > 0 && !cs.forceCoop && sch.degree <= kMaxDegree) {
    cudaLaunchConfig_t cfg{};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)cs.clusterGrid;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3((unsigned)cs.clusterGrid);
    cfg.blockDim = dim3(1024);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, coarse_solve_coop<T, true>, c, r, skip, sch);
  }
  if (cs.coopGrid > 0 && sch.degree <= kMaxDegree) {
    CoarseDev cv = c;
    const T* rr = r;
    ChebSchedule sc = sch;
    void* args[] = {&cv, (void*)&rr, (void*)&skip, &sc};
    return cudaLaunchCooperativeKernel((const void*)coarse_solve_coop<T>, dim3(cs.coopGrid), dim3(512), args, 0, s);
  }
  const unsigned g = blocks_for(c.nV);
  coarse_restrict<T><<<g, kT, 0, s>>>(c, r, skip, sch.d0scale);
  float *dk = c.cd0, *dn = c.cd1;
  for (int k = 0; k < sch.degree; ++k) {
    coarse_cheb_step<<<g, kT, 0, s>>>(c, dk, dn, sch.c1[k], sch.c2[k], k + 1 == sch.degree, skip);
    std::swap(dk, dn);
  }
  return cudaGetLastError();
}

template <typename T>
cudaError_t coarse_prolong_add(const CoarseSolver& cs, T* x, cudaStream_t s) {
  coarse_prolong<T><<<blocks_for(cs.dev.nFaces * cs.dev.NF), kT, 0, s>>>(cs.dev, x);
  return cudaGetLastError();
}

// Errors of the coarse residual samples: Y ~ A_c^{-1} R by Chebyshev on
// [lmin, lmax] of D^{-1} A_c, degree for a reduction `target` (at most maxDeg).
cudaError_t coarse_errors(const CoarseSolver& cs, const float* R0, int S, double target, int maxDeg, float** out,
                          cudaStream_t s) {
  const CoarseDev& c = cs.dev;
  const int64_t n = (int64_t)S * c.nV;
  float *R = nullptr, *D0 = nullptr, *D1 = nullptr, *Y = nullptr;
  cudaError_t e = cudaMalloc(&R, sizeof(float) * n);
  if (e == cudaSuccess) e = cudaMalloc(&D0, sizeof(float) * n);
  if (e == cudaSuccess) e = cudaMalloc(&D1, sizeof(float) * n);
  if (e == cudaSuccess) e = cudaMalloc(&Y, sizeof(float) * n);
  if (e != cudaSuccess) {
    cudaFree(R);
    cudaFree(D0);
    cudaFree(D1);
    cudaFree(Y);
    return e;
  }
  cudaMemcpyAsync(R, R0, sizeof(float) * n, cudaMemcpyDeviceToDevice, s);
  const double th = 0.5 * (cs.lmax + cs.lmin), de = 0.5 * (cs.lmax - cs.lmin), sig = th / de;
  int K = (int)std::ceil(std::acosh(1.0 / target) / std::acosh(sig));
  K = std::max(1, std::min(K, maxDeg));
  const dim3 grid((unsigned)std::min<int64_t>((c.nV + kT - 1) / kT, 64), S);
  learn_cheb_start<<<grid, kT, 0, s>>>(c, R, D0, Y, (float)(1.0 / th));
  double rho = 1.0 / sig;
  float *dk = D0, *dn = D1;
  for (int k = 0; k < K; ++k) {
    const double rho1 = 1.0 / (2.0 * sig - rho);
    learn_cheb<<<grid, kT, 0, s>>>(c, dk, dn, R, Y, (float)(rho1 * rho), (float)(2.0 * rho1 / de), k + 1 == K);
    rho = rho1;
    std::swap(dk, dn);
  }
  cudaFree(R);
  cudaFree(D0);
  cudaFree(D1);
  *out = Y;
  return cudaGetLastError();
}

cudaError_t coarse_loss_grad(const CoarseSolver& cs, const float* samples, int S, int K, const double* theta,
                             double* loss, double* grad, cudaStream_t s) {
  LearnWork lw{};
  cudaError_t e = learn_setup(cs.dev, samples, S, K, &lw, s);
  std::vector<double> hp;
  if (e == cudaSuccess) e = learn_pass(cs.dev, lw, S, K, theta, loss, grad, hp, s);
  learn_free(&lw);
  return e;
}

cudaError_t coarse_train(CoarseSolver* cs, const float* samples, int S, int K, int steps, double lr, cudaStream_t s,
                         CoarseTrainResult* out, bool feasible) {
  *out = CoarseTrainResult{};
  out->degree = K;
  out->samples = S;
  out->steps = steps;
  auto t0 = std::chrono::steady_clock::now();
  const double lmax = cs->lmax, lmin = cs->lmin;
  // training errors U_0 = A_c^{-1} (P^T r): Chebyshev to 1e-4 on the residual samples
  float* U0 = nullptr;
  cudaError_t e = coarse_errors(*cs, samples, S, 1e-4, 256, &U0, s);
  LearnWork lw{};
  if (e == cudaSuccess) e = learn_setup(cs->dev, U0, S, K, &lw, s);
  cudaFree(U0);
  if (e != cudaSuccess) {
    learn_free(&lw);
    return e;
  }
  // start from Chebyshev of the same degree on [lmin, lmax]: its residual
  // polynomial has the roots lambda_j of T_K mapped to the interval
  std::vector<double> phi(K), theta(K), grad(K), hp, best(K);
  for (int j = 0; j < K; ++j) {
    const double lj = 0.5 * (lmax + lmin) + 0.5 * (lmax - lmin) * std::cos(M_PI * (2 * j + 1) / (2.0 * K));
    phi[j] = std::log(lmax / lj);  // theta_j = e^phi / lmax = 1 / lambda_j
  }
  auto thetas = [&]() {
    for (int k = 0; k < K; ++k) theta[k] = std::exp(phi[k]) / lmax;
  };
  thetas();
  double L = 0.0;
  if ((e = learn_pass(cs->dev, lw, S, K, theta.data(), &L, grad.data(), hp, s)) != cudaSuccess) {
    learn_free(&lw);
    return e;
  }
  out->lossChebyshev = L;
  double bestL = L;
  best = phi;
  std::vector<double> m1(K, 0.0), m2(K, 0.0);
  const double b1 = 0.9, b2 = 0.999;
  std::vector<double> pgrad(K);
  std::vector<double> step(K), trial(K), thTrial(K);
  for (int it = 0; it < steps; ++it) {
    poly_penalty(theta, lmax, &pgrad);
    for (int k = 0; k < K; ++k) {
      const double g = (grad[k] + pgrad[k]) * theta[k];  // d/dphi of loss + penalty
      m1[k] = b1 * m1[k] + (1 - b1) * g;
      m2[k] = b2 * m2[k] + (1 - b2) * g * g;
      const double mh = m1[k] / (1 - std::pow(b1, it + 1)), vh = m2[k] / (1 - std::pow(b2, it + 1));
      step[k] = lr * mh / (std::sqrt(vh) + 1e-12);
    }
    if (feasible) {
      // stay inside the set where the residual polynomial is <= 1 on [0, lmax]: halve
      // the step until it is (twelve halvings at most; otherwise no move this step)
      double sc = 1.0;
      bool ok = false;
      for (int bt = 0; bt < 12 && !ok; ++bt, sc *= 0.5) {
        for (int k = 0; k < K; ++k) {
          trial[k] = phi[k] - sc * step[k];
          thTrial[k] = std::exp(trial[k]) / lmax;
        }
        ok = poly_max(thTrial, lmax) <= 1.0 + 1e-9;
      }
      if (!ok) {
        ++out->rejectedSteps;
        continue;
      }
      phi = trial;
    } else {
      for (int k = 0; k < K; ++k) phi[k] -= step[k];
    }
    thetas();
    if ((e = learn_pass(cs->dev, lw, S, K, theta.data(), &L, grad.data(), hp, s)) != cudaSuccess) break;
    if (it == 0) out->lossFirstStep = L;
    if (std::isfinite(L) && L < bestL) {
      // keep only polynomials that leave the coarse solve positive semidefinite
      std::vector<double> th(K);
      for (int k = 0; k < K; ++k) th[k] = std::exp(phi[k]) / lmax;
      if (poly_max(th, lmax) <= 1.0 + 1e-9) {
        bestL = L;
        best = phi;
        ++out->lowerSteps;
      } else {
        ++out->rejectedSteps;
      }
    }
  }
  learn_free(&lw);
  if (e != cudaSuccess) return e;
  out->lossLearned = bestL;
  out->lossStart = out->lossChebyshev;
  std::vector<double> th(K);
  for (int k = 0; k < K; ++k) th[k] = std::exp(best[k]) / lmax;
  out->maxGain = poly_max(th, lmax);
  out->accepted = bestL < out->lossChebyshev ? 1 : 0;
  if (out->accepted) {
    // Leja order of the roots 1/theta (largest first, then each maximising the
    // product of distances to those already taken): the same polynomial, with
    // bounded growth of the partial products in FP32
    std::vector<double> roots(K), ordered;
    for (int k = 0; k < K; ++k) roots[k] = 1.0 / std::exp(best[k]);  // in units of lmax
    std::vector<bool> used(K, false);
    for (int n = 0; n < K; ++n) {
      int pick = -1;
      double bestScore = -1.0;
      for (int k = 0; k < K; ++k) {
        if (used[k]) continue;
        double score = n == 0 ? std::fabs(roots[k]) : 1.0;
        for (double r : ordered) score *= std::fabs(roots[k] - r);
        if (score > bestScore) {
          bestScore = score;
          pick = k;
        }
      }
      used[pick] = true;
      ordered.push_back(roots[pick]);
    }
    cs->thetaHat.resize(K);
    for (int k = 0; k < K; ++k) cs->thetaHat[k] = 1.0 / ordered[k];  // theta * lmax
  }
  out->ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return cudaSuccess;
}

template cudaError_t coarse_setup<double>(CoarseSolver*, const double*, int, double, cudaStream_t);
template cudaError_t coarse_setup<float>(CoarseSolver*, const float*, int, double, cudaStream_t);
template cudaError_t coarse_apply<double>(const CoarseSolver&, const double*, const int*, cudaStream_t);
template cudaError_t coarse_apply<float>(const CoarseSolver&, const float*, const int*, cudaStream_t);
template cudaError_t coarse_prolong_add<double>(const CoarseSolver&, double*, cudaStream_t);
template cudaError_t coarse_prolong_add<float>(const CoarseSolver&, float*, cudaStream_t);

}  // namespace hfx
