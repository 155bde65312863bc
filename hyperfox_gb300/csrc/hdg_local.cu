// Per-element HDG assembly + static condensation, FP64, sm_103a.
//
// One group of TPE threads owns one element at a time; EPC groups share a CTA
// and the reference tables staged once per CTA in shared memory. The CTA walks
// the elements with a grid-stride loop (grid = resident CTAs on all SMs), so
// the tables are loaded once per CTA, not once per element.
//
// Restates, per element (HyperFox file:line):
//   Jacobians / measures / inverse   Operator.cpp:14-84, HDGModel.cpp:53-85
//   normals                          HDGBase.cpp:34-65
//   tau at face IPs                  HDGBase.cpp:18-32
//   HDGBase blocks                   HDGBase.cpp:67-158
//   HDGDiffusion blocks, kappa       HDGDiffusion.cpp:31-145, HDGDiffusionSource.cpp:60-79
//   Source RHS                       Source.cpp:5-48
//   implicit Euler on the U rows     HDGModel.cpp:39-47, Euler.cpp:18-34
//   condensation U,Q,U0,Q0,S,S0      HDGSolver.cpp:331-348
//   Dirichlet Set on boundary faces  HDGSolver.cpp:361-529, DirichletModel.cpp:19-44
//
// The local matrix is never formed: the kernel builds its non-zero blocks
// (mass M, convection C_d, kappa-weighted K_d, face blocks T_f, E_fd, H_fd) and
// condenses with the structure Sqq = M (x) I_d, so Sqq^{-1} is one N x N
// inverse. Results equal the reference's dense QR condensation up to
// round-off.
#include <cstdio>

#include "hfx_device.h"

namespace hfx {
namespace {

template <typename T_, int D, int P, int TPE, int EPC>
struct Layout {
  using K = Dims<D, P>;
  static constexpr int N = K::N, NF = K::NF, F = K::F, NI = K::NI, NIF = K::NIF, LL = K::LL;
  static constexpr int DM = D - 1;
  // shared tables
  static constexpr int T_PHI = 0;
  static constexpr int T_DPHI = T_PHI + NI * N;
  static constexpr int T_W = T_DPHI + NI * N * D;
  static constexpr int T_FPHI = T_W + NI;
  static constexpr int T_FDPHI = T_FPHI + NIF * NF;
  static constexpr int T_FW = T_FDPHI + NIF * NF * DM;
  static constexpr int TAB = (T_FW + NIF + 3) & ~3;  // whole 16-byte units for the bulk copy
  // per-group region (doubles)
  static constexpr int X = 0;                       // N*D coordinates
  static constexpr int KAPN = X + N * D;            // N*D*D nodal kappa tensor
  static constexpr int TAUL = KAPN + N * D * D;     // F*NF local tau
  static constexpr int DV = TAUL + F * NF;          // NI
  static constexpr int FQ = DV + NI;                // NI source at IPs
  static constexpr int FU = FQ + NI;                // N
  static constexpr int DST = FU + N;                // F*NIF   dS*tau
  static constexpr int DSN = DST + F * NIF;         // F*NIF*D dS*n
  static constexpr int DSKN = DSN + F * NIF * D;    // F*NIF*D dS*kappa*n
  static constexpr int M = DSKN + F * NIF * D;      // N*N mass, later M^{-1}
  static constexpr int C = M + N * N;               // D*N*N convection
  static constexpr int KS = C + D * N * N;          // D*N*N kappa-convection, then Suq
  static constexpr int T = KS + D * N * N;          // F*NF*NF
  static constexpr int E = T + F * NF * NF;         // F*D*NF*NF
  static constexpr int H = E + F * D * NF * NF;     // F*D*NF*NF
  static constexpr int BIG_A = 2 * NI * N * D;      // G and KG
  static constexpr int BIG_B = D * N * LL;          // Xl, later Q
  static constexpr int BIG = H + F * D * NF * NF;
  static constexpr int XU = BIG + (BIG_A > BIG_B ? BIG_A : BIG_B);  // D*N*N; invJ/kq alias before
  static constexpr int XU_SZ = (D * N * N > 2 * NI * D * D) ? D * N * N : 2 * NI * D * D;
  static constexpr int AR = XU + XU_SZ;             // A (N*N) + RHS N*(LL+1); Gauss-Jordan before
  static constexpr int AR_SZ = (N * N + N * (LL + 1) > 2 * N * N) ? N * N + N * (LL + 1) : 2 * N * N;
  static constexpr int Q0 = AR + AR_SZ;             // D*N
  static constexpr int WQ = Q0 + D * N;             // D*N  M^{-1} r_q (residual mode)
  static constexpr int GROUP = (WQ + D * N + 1) & ~1;
  static constexpr int TOTAL_DOUBLES = TAB + EPC * GROUP;
  // per-group ints
  static constexpr int IGROUP = N + 2 * F;          // pivots, face ids, boundary flags
};

template <typename T, int D, int P, int TPE, int EPC>
__global__ void __launch_bounds__(TPE * EPC)
    local_condense(LocalParams p) {
  using L = Layout<T, D, P, TPE, EPC>;
  constexpr int N = L::N, NF = L::NF, F = L::F, NI = L::NI, NIF = L::NIF, LL = L::LL, DM = L::DM;
  constexpr int LU = N, LQ = D * N;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* smem = reinterpret_cast<T*>(smem_raw);
  __shared__ int sFaceNodes[F * NF];
  __shared__ int sOpp[F];
  __shared__ int sPos[F * N];  // position of element node i on face f, -1 if not on it
  __shared__ int sInt[EPC * L::IGROUP];

  const int nthr = TPE * EPC;
  // ---- stage tables once per CTA: one bulk copy (the table in the kernel's precision,
  // padded to whole 16-byte units), completion counted in bytes on an mbarrier
  {
    __shared__ __align__(8) uint64_t tabBar;
    __shared__ int sTabFail;
    const uint32_t bar = (uint32_t)__cvta_generic_to_shared(&tabBar);
    if (threadIdx.x == 0) sTabFail = 0;
    const uint32_t bytes = (uint32_t)(((L::T_FW + NIF) * sizeof(T) + 15) / 16 * 16);
    const void* src = sizeof(T) == 8 ? (const void*)p.tab : (const void*)p.tab32;
    if (threadIdx.x == 0) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar));
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
      asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                       (uint32_t)__cvta_generic_to_shared(smem)),
                   "l"(src), "r"(bytes), "r"(bar)
                   : "memory");
    }
    for (int i = threadIdx.x; i < F * NF; i += nthr) sFaceNodes[i] = p.itab[i];
    for (int i = threadIdx.x; i < F; i += nthr) sOpp[i] = p.itab[F * NF + i];
    for (int i = threadIdx.x; i < F * N; i += nthr) sPos[i] = -1;
    __syncthreads();  // also orders the barrier's initialisation before every thread's wait
    for (int i = threadIdx.x; i < F * NF; i += nthr) sPos[(i / NF) * N + sFaceNodes[i]] = i % NF;
    // bounded wait for the table (phase 0); a wait that runs out reports status 2
    uint32_t done = 0;
    for (uint32_t it = 0; it < (1u << 26) && !done; ++it)
      asm volatile("{ .reg .pred q; mbarrier.try_wait.parity.shared::cta.b64 q, [%1], 0; selp.u32 %0, 1, 0, q; }"
                   : "=r"(done)
                   : "r"(bar)
                   : "memory");
    if (!done) {
      atomicCAS(p.status, 0, 2);
      sTabFail = 1;
    }
    __syncthreads();
    if (sTabFail) return;  // the same value for every thread of the CTA
  }
  const T* phi = smem + L::T_PHI;
  const T* dphi = smem + L::T_DPHI;
  const T* w = smem + L::T_W;
  const T* fphi = smem + L::T_FPHI;
  const T* fdphi = smem + L::T_FDPHI;
  const T* fw = smem + L::T_FW;

  const int grp = threadIdx.x / TPE, t = threadIdx.x % TPE;
  T* R = smem + L::TAB + grp * L::GROUP;
  int* I = sInt + grp * L::IGROUP;
  T* X = R + L::X;
  T* kapN = R + L::KAPN;
  T* tauL = R + L::TAUL;
  T* dV = R + L::DV;
  T* fq = R + L::FQ;
  T* fu = R + L::FU;
  T* dSt = R + L::DST;
  T* dSn = R + L::DSN;
  T* dSkn = R + L::DSKN;
  T* Mm = R + L::M;
  T* Cm = R + L::C;
  T* Km = R + L::KS;
  T* Tm = R + L::T;
  T* Em = R + L::E;
  T* Hm = R + L::H;
  T* G = R + L::BIG;                 // [NI][N][D] dV * J^{-1} grad phi
  T* KG = G + NI * N * D;            // [NI][N][D] dV * kappa J^{-1} grad phi
  T* Xl = R + L::BIG;                // [D][N][LL] (after G, KG die), later Q
  T* Xu = R + L::XU;                 // [D][N][N]
  T* invJ = R + L::XU;               // [NI][D][D] (before Xu)
  T* kq = invJ + NI * D * D;         // [NI][D][D]
  T* Am = R + L::AR;                 // [N][N] row-major
  T* Rhs = Am + N * N;               // [N][LL+1] row-major: Schur RHS columns then fu
  T* Aug = R + L::AR;                // Gauss-Jordan [N][2N] (before Am)
  T* Q0s = R + L::Q0;
  T* Wq = R + L::WQ;
  const bool rhsMode = p.rhsU != nullptr;
  int* piv = I;
  int* faceId = I + N;
  int* bnd = I + N + F;

  const int64_t nGroups = (int64_t)gridDim.x * EPC;
  // blocks precomputed on the tensor cores (FP32 path): loaded instead of integrated
  const bool tcMode = sizeof(T) == 4 && p.tcBlocks != nullptr;
  for (int64_t base = (int64_t)blockIdx.x * EPC; base < p.nCells; base += nGroups) {
    const int64_t e = base + grp;
    const bool active = e < p.nCells;
    const float* tcb = tcMode && active ? p.tcBlocks + e * p.tcStride : nullptr;
    // ---------------------------------------------------------- gather
    if (active && tcMode) {
      for (int i = t; i < F; i += TPE) {
        int f = p.cell2face[e * F + i];
        faceId[i] = f;
        bnd[i] = p.isBoundary[f];
      }
    }
    if (active && !tcMode) {
      const int* cell = p.cells + e * N;
      for (int i = t; i < N * D; i += TPE) X[i] = p.coords[(int64_t)cell[i / D] * D + (i % D)];
      for (int i = t; i < N * D * D; i += TPE) {
        int n = i / (D * D), a = i % (D * D);
        T v;
        if (p.kc == 0) v = (a % (D + 1) == 0) ? 1.0 : 0.0;
        else {
          int64_t base_k = p.kappaLayout == 0 ? (int64_t)cell[n] * p.kc : (e * N + n) * p.kc;
          if (p.kc == 1) v = (a % (D + 1) == 0) ? p.kappa[base_k] : 0.0;
          else v = p.kappa[base_k + a];
        }
        kapN[i] = v;
      }
      for (int i = t; i < F; i += TPE) {
        int f = p.cell2face[e * F + i];
        faceId[i] = f;
        bnd[i] = p.isBoundary[f];
      }
      for (int i = t; i < F * NF; i += TPE) {
        int f = p.cell2face[e * F + i / NF];
        int side = (p.face2cell[2 * (int64_t)f] == (int)e) ? 0 : 1;
        int q = p.perm[e * F * NF + i];
        tauL[i] = p.tau[((int64_t)f * NF + q) * p.tauVals + (p.tauVals == 2 ? side : 0)];
      }
    }
    __syncthreads();
    // ------------------------------------------------- volume geometry
    if (active && !tcMode) {
      for (int q = t; q < NI; q += TPE) {
        T J[D][D];
        for (int r = 0; r < D; ++r)
          for (int s = 0; s < D; ++s) {
            T acc = 0.0;
            for (int i = 0; i < N; ++i) acc += dphi[(q * N + i) * D + r] * X[i * D + s];
            J[r][s] = acc;
          }
        T det, iv[D][D];
        if (D == 2) {
          det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
          T id = 1.0 / det;
          iv[0][0] = J[1][1] * id;
          iv[0][1] = -J[0][1] * id;
          iv[1][0] = -J[1][0] * id;
          iv[1][1] = J[0][0] * id;
        } else {
          T c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
          T c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
          T c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
          det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
          T id = 1.0 / det;
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
        T dv = w[q] * det;
        dV[q] = dv;
        for (int a = 0; a < D; ++a)
          for (int b = 0; b < D; ++b) invJ[(q * D + a) * D + b] = iv[a][b];
        for (int a = 0; a < D * D; ++a) {
          T acc = 0.0;
          for (int i = 0; i < N; ++i) acc += phi[q * N + i] * kapN[i * D * D + a];
          kq[q * D * D + a] = acc;  // column-major d x d (HDGDiffusion.cpp:52-57)
        }
        T fval = 0.0;
        if (p.srcMode == 1) fval = p.src[e * NI + q];
        else if (p.srcMode == 2) {
          fval = p.srcParam;
          for (int k = 0; k < D; ++k) {
            T xk = 0.0;
            for (int i = 0; i < N; ++i) xk += phi[q * N + i] * X[i * D + k];
            fval *= sin(T(M_PI) * xk);
          }
        }
        fq[q] = fval * dv;
      }
      // face geometry
      for (int fk = t; fk < F * NIF; fk += TPE) {
        int f = fk / NIF, k = fk % NIF;
        T Jf[D - 1][D];
        for (int r = 0; r < DM; ++r)
          for (int s = 0; s < D; ++s) {
            T acc = 0.0;
            for (int i = 0; i < NF; ++i) acc += fdphi[(k * NF + i) * DM + r] * X[sFaceNodes[f * NF + i] * D + s];
            Jf[r][s] = acc;
          }
        T nv[D], ds;
        if (D == 2) {
          ds = sqrt(Jf[0][0] * Jf[0][0] + Jf[0][1] * Jf[0][1]);
          nv[0] = -Jf[0][1];
          nv[1] = Jf[0][0];
        } else {
          T g00 = Jf[0][0] * Jf[0][0] + Jf[0][1] * Jf[0][1] + Jf[0][2] * Jf[0][2];
          T g11 = Jf[1][0] * Jf[1][0] + Jf[1][1] * Jf[1][1] + Jf[1][2] * Jf[1][2];
          T g01 = Jf[0][0] * Jf[1][0] + Jf[0][1] * Jf[1][1] + Jf[0][2] * Jf[1][2];
          ds = sqrt(g00 * g11 - g01 * g01);
          nv[0] = Jf[0][1] * Jf[1][2] - Jf[0][2] * Jf[1][1];
          nv[1] = Jf[0][2] * Jf[1][0] - Jf[0][0] * Jf[1][2];
          nv[2] = Jf[0][0] * Jf[1][1] - Jf[0][1] * Jf[1][0];
        }
        T nn = 0.0;
        for (int a = 0; a < D; ++a) nn += nv[a] * nv[a];
        nn = 1.0 / sqrt(nn);
        T prod = 0.0;
        int v0 = sFaceNodes[f * NF], vn = sOpp[f];
        for (int a = 0; a < D; ++a) {
          nv[a] *= nn;
          prod += (X[vn * D + a] - X[v0 * D + a]) * nv[a];
        }
        if (prod > 0)
          for (int a = 0; a < D; ++a) nv[a] = -nv[a];
        ds *= fw[k];
        T tq = 0.0;
        for (int i = 0; i < NF; ++i) tq += fphi[k * NF + i] * tauL[f * NF + i];
        dSt[fk] = ds * tq;
        for (int a = 0; a < D; ++a) dSn[fk * D + a] = ds * nv[a];
        for (int a = 0; a < D; ++a) {
          T acc = 0.0;  // (kappa n)_a with kappa interpolated on the face
          for (int b = 0; b < D; ++b) {
            T kab = 0.0;
            for (int i = 0; i < NF; ++i) kab += fphi[k * NF + i] * kapN[sFaceNodes[f * NF + i] * D * D + a + b * D];
            acc += kab * nv[b];
          }
          dSkn[fk * D + a] = ds * acc;
        }
      }
    }
    __syncthreads();
    // scaled physical gradients G = dV J^{-1} grad phi and KG = kappa G
    if (active && tcMode) {
      const float* tfu = tcb + (2 * D * N + N) * N + F * NF * (1 + 2 * D) * NF;
      for (int i = t; i < N; i += TPE) fu[i] = rhsMode ? (T)p.rhsU[e * N + i] : (T)tfu[i];
    }
    if (active && !tcMode) {
      for (int qi = t; qi < NI * N; qi += TPE) {
        int q = qi / N, i = qi % N;
        T g[D];
        for (int a = 0; a < D; ++a) {
          T acc = 0.0;
          for (int b = 0; b < D; ++b) acc += invJ[(q * D + a) * D + b] * dphi[(q * N + i) * D + b];
          g[a] = acc * dV[q];
        }
        for (int a = 0; a < D; ++a) {
          G[qi * D + a] = g[a];
          if (p.kc == 0) continue;  // identity tensor: the kappa-weighted blocks equal the plain ones
          T acc = 0.0;
          for (int b = 0; b < D; ++b) acc += kq[q * D * D + a + b * D] * g[b];
          KG[qi * D + a] = acc;
        }
      }
      for (int i = t; i < N; i += TPE) {
        T acc = 0.0;
        if (rhsMode) acc = (T)p.rhsU[e * N + i];
        else
          for (int q = 0; q < NI; ++q) acc += phi[q * N + i] * fq[q];
        fu[i] = acc;
      }
    }
    __syncthreads();
    // ------------------------------------------ volume and face blocks
    if (active && tcMode) {
      // tensor-core blocks: [C | K | M] rows of N, then [T | E | H] rows of NF (same index order)
      for (int i = t; i < D * N * N; i += TPE) {
        Cm[i] = (T)tcb[i];
        Km[i] = (T)tcb[D * N * N + i];
      }
      for (int i = t; i < N * N; i += TPE) Mm[i] = (T)tcb[2 * D * N * N + i];
      const float* tf = tcb + (2 * D * N + N) * N;
      for (int i = t; i < F * NF * NF; i += TPE) Tm[i] = (T)tf[i];
      for (int i = t; i < F * D * NF * NF; i += TPE) {
        Em[i] = (T)tf[F * NF * NF + i];
        Hm[i] = (T)tf[F * NF * NF + F * D * NF * NF + i];
      }
    }
    if (active && !tcMode) {
      for (int ij = t; ij < N * N; ij += TPE) {
        int i = ij / N, j = ij % N;
        T m = 0.0;
        for (int q = 0; q < NI; ++q) m += dV[q] * phi[q * N + i] * phi[q * N + j];
        Mm[ij] = m;
      }
      for (int dij = t; dij < D * N * N; dij += TPE) {
        int d = dij / (N * N), i = (dij / N) % N, j = dij % N;
        T c = 0.0, k = 0.0;
        if (p.kc == 0) {
          for (int q = 0; q < NI; ++q) c += G[(q * N + i) * D + d] * phi[q * N + j];
          k = c;
        } else {
          for (int q = 0; q < NI; ++q) {
            T pj = phi[q * N + j];
            c += G[(q * N + i) * D + d] * pj;
            k += KG[(q * N + i) * D + d] * pj;
          }
        }
        Cm[dij] = c;  // Squ[(i,d)][j]
        Km[dij] = k;  // Suq[i][(j,d)] volume part
      }
      for (int fab = t; fab < F * NF * NF; fab += TPE) {
        int f = fab / (NF * NF), a = (fab / NF) % NF, b = fab % NF;
        T tt = 0.0, ee[D], hh[D];
        for (int d = 0; d < D; ++d) ee[d] = hh[d] = 0.0;
        for (int k = 0; k < NIF; ++k) {
          T ss = fphi[k * NF + a] * fphi[k * NF + b];
          int fk = f * NIF + k;
          tt += dSt[fk] * ss;
          for (int d = 0; d < D; ++d) ee[d] += dSn[fk * D + d] * ss;
          if (p.kc != 0)
            for (int d = 0; d < D; ++d) hh[d] += dSkn[fk * D + d] * ss;
        }
        if (p.kc == 0)
          for (int d = 0; d < D; ++d) hh[d] = ee[d];
        Tm[fab] = tt;
        for (int d = 0; d < D; ++d) {
          Em[((f * D + d) * NF + a) * NF + b] = ee[d];
          Hm[((f * D + d) * NF + a) * NF + b] = hh[d];
        }
      }
    }
    __syncthreads();
    // ----------------------------- M^{-1} by Gauss-Jordan ([M | I], no pivoting: M definite)
    if (active)
      for (int ij = t; ij < N * 2 * N; ij += TPE) {
        int i = ij / (2 * N), j = ij % (2 * N);
        Aug[ij] = j < N ? Mm[i * N + j] : (j - N == i ? 1.0 : 0.0);
      }
    __syncthreads();
    for (int k = 0; k < N; ++k) {
      T pinv = active ? 1.0 / Aug[k * 2 * N + k] : 0.0;
      __syncthreads();
      if (active)
        for (int ij = t; ij < N * 2 * N; ij += TPE) {
          int i = ij / (2 * N), j = ij % (2 * N);
          if (i == k || j <= k) continue;  // column k of row i is the factor: keep it
          T f = Aug[i * 2 * N + k] * pinv;
          Aug[ij] -= f * Aug[k * 2 * N + j];
        }
      __syncthreads();
      if (active)
        for (int j = t; j < 2 * N; j += TPE)
          if (j >= k) Aug[k * 2 * N + j] *= pinv;
      __syncthreads();
    }
    if (active)
      for (int ij = t; ij < N * N; ij += TPE) Mm[ij] = Aug[(ij / N) * 2 * N + N + (ij % N)];
    __syncthreads();
    // residual mode: w_d = M^{-1} r_q,d (r_q node-major (i, d))
    if (active)
      for (int di = t; di < D * N; di += TPE) {
        int d = di / N, i = di % N;
        T acc = 0.0;
        if (rhsMode)
          for (int m = 0; m < N; ++m) acc += Mm[i * N + m] * (T)p.rhsQ[e * N * D + m * D + d];
        Wq[di] = acc;
      }
    // ---- Xu_d = M^{-1} C_d ; Xl_d(:, (f,b)) = -sum_a M^{-1}(:, fn(f,a)) E_fd(a,b)
    if (active) {
      for (int dij = t; dij < D * N * N; dij += TPE) {
        int d = dij / (N * N), i = (dij / N) % N, j = dij % N;
        T acc = 0.0;
        for (int m = 0; m < N; ++m) acc += Mm[i * N + m] * Cm[(d * N + m) * N + j];
        Xu[dij] = acc;
      }
      for (int dic = t; dic < D * N * LL; dic += TPE) {
        int d = dic / (N * LL), i = (dic / LL) % N, c = dic % LL;
        int f = c / NF, b = c % NF;
        T acc = 0.0;
        for (int a = 0; a < NF; ++a)
          acc += Mm[i * N + sFaceNodes[f * NF + a]] * Em[((f * D + d) * NF + a) * NF + b];
        Xl[dic] = -acc;
      }
      // Suq_d(i,j) = K_d(i,j) - sum_f H_fd(pos_f(i), pos_f(j)) (in place, entry-wise)
      for (int dij = t; dij < D * N * N; dij += TPE) {
        int d = dij / (N * N), i = (dij / N) % N, j = dij % N;
        T acc = Km[dij];
        for (int f = 0; f < F; ++f) {
          int a = sPos[f * N + i], b = sPos[f * N + j];
          if (a >= 0 && b >= 0) acc -= Hm[((f * D + d) * NF + a) * NF + b];
        }
        Km[dij] = acc;
      }
    }
    __syncthreads();
    // ---- A = dt*(Suu - Suq Xu) + M_mass ; Rhs = [dt*(Sul - Suq Xl) | fu']
    // (without a time scheme dt_eff = 1 and no mass term)
    const T dts = p.dt > 0.0 ? p.dt : 1.0;
    const T cs = p.rkWu ? (T)p.cStiff : dts;  // scale of the U rows' stiffness (Runge-Kutta stage)
    if (active) {
      for (int ij = t; ij < N * N; ij += TPE) {
        int i = ij / N, j = ij % N;
        T suu = 0.0;
        for (int f = 0; f < F; ++f) {
          int a = sPos[f * N + i], b = sPos[f * N + j];
          if (a >= 0 && b >= 0) suu += Tm[(f * NF + a) * NF + b];
        }
        T acc = 0.0;
        for (int d = 0; d < D; ++d)
          for (int m = 0; m < N; ++m) acc += Km[(d * N + i) * N + m] * Xu[(d * N + m) * N + j];
        T v = suu - acc;
        if (p.dt > 0.0) {
          // mass of the time scheme: M = sum_q dV phi phi (Mass.cpp:5-38)
          T mm = 0.0;
          if (tcMode) mm = (T)tcb[2 * D * N * N + i * N + j];
          else
            for (int q = 0; q < NI; ++q) mm += dV[q] * phi[q * N + i] * phi[q * N + j];
          v = cs * v + mm;
        }
        Am[ij] = v;
      }
      for (int ic = t; ic < N * (LL + 1); ic += TPE) {
        int i = ic / (LL + 1), c = ic % (LL + 1);
        T v;
        if (c < LL) {
          int f = c / NF, b = c % NF;
          int a = sPos[f * N + i];
          T sul = (a >= 0) ? -Tm[(f * NF + a) * NF + b] : 0.0;
          T acc = 0.0;
          for (int d = 0; d < D; ++d)
            for (int m = 0; m < N; ++m) acc += Km[(d * N + i) * N + m] * Xl[(d * N + m) * LL + c];
          v = cs * (sul - acc);
        } else if (rhsMode) {
          // r_u - dt Suq M^{-1} r_q (the residual already carries the time scheme)
          T acc = 0.0;
          for (int d = 0; d < D; ++d)
            for (int m = 0; m < N; ++m) acc += Km[(d * N + i) * N + m] * Wq[d * N + m];
          v = fu[i] - dts * acc;
        } else {
          v = dts * fu[i];
          if (p.dt > 0.0) {
            T mu = 0.0;
            for (int j = 0; j < N; ++j) {
              T mm = 0.0;
              if (tcMode) mm = (T)tcb[2 * D * N * N + i * N + j];
              else
                for (int q = 0; q < NI; ++q) mm += dV[q] * phi[q * N + i] * phi[q * N + j];
              mu += mm * p.uOld[e * N + j];
            }
            v += mu;
          }
          if (p.rkWu) {
            // - (K w)_i over the unscaled U rows: [Suu | Suq | Sul] w
            T kw = 0.0;
            for (int f = 0; f < F; ++f) {
              const int a = sPos[f * N + i];
              if (a < 0) continue;
              const int64_t fc = p.cell2face[e * F + f];
              for (int b = 0; b < NF; ++b) {
                const T wl = (T)p.rkWl[fc * NF + p.perm[(e * F + f) * NF + b]];
                kw += Tm[(f * NF + a) * NF + b] * ((T)p.rkWu[e * N + sFaceNodes[f * NF + b]] - wl);
              }
            }
            for (int d = 0; d < D; ++d)
              for (int m = 0; m < N; ++m) kw += Km[(d * N + i) * N + m] * (T)p.rkWq[(e * N + m) * D + d];
            v -= kw;
          }
        }
        Rhs[ic] = v;
      }
    }
    __syncthreads();
    // ---- Gauss-Jordan with partial pivoting on [A | Rhs]: Rhs <- A^{-1} Rhs.
    // The pivot search is a warp argmax and every step updates all rows in
    // parallel, so no serial back substitution is left.
    bool singular = false;
    for (int k = 0; k < N; ++k) {
      if (active && t < 32) {
        T best = T(-1);
        int pr = k;
        for (int i = k + t; i < N; i += 32) {
          T v = fabs(Am[i * N + k]);
          if (v > best) {
            best = v;
            pr = i;
          }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          T ob = __shfl_xor_sync(0xffffffffu, best, o);
          int op = __shfl_xor_sync(0xffffffffu, pr, o);
          if (ob > best || (ob == best && op < pr)) {
            best = ob;
            pr = op;
          }
        }
        if (t == 0) piv[k] = pr;
      }
      __syncthreads();
      if (active) {
        int pr = piv[k];
        if (pr != k) {
          for (int j = t; j < N; j += TPE) {
            T tmp = Am[k * N + j];
            Am[k * N + j] = Am[pr * N + j];
            Am[pr * N + j] = tmp;
          }
          for (int j = t; j < LL + 1; j += TPE) {
            T tmp = Rhs[k * (LL + 1) + j];
            Rhs[k * (LL + 1) + j] = Rhs[pr * (LL + 1) + j];
            Rhs[pr * (LL + 1) + j] = tmp;
          }
        }
      }
      __syncthreads();
      if (active) {
        T akk = Am[k * N + k];
        if (akk == T(0)) singular = true;
        T inv = T(1) / akk;
        const int cols = (N - k - 1) + (LL + 1);
        for (int rc = t; rc < (N - 1) * cols; rc += TPE) {
          int i = rc / cols, c = rc % cols;
          if (i >= k) ++i;  // every row but the pivot row
          T l = Am[i * N + k] * inv;
          if (c < N - k - 1) {
            int j = k + 1 + c;
            Am[i * N + j] -= l * Am[k * N + j];
          } else {
            int j = c - (N - k - 1);
            Rhs[i * (LL + 1) + j] -= l * Rhs[k * (LL + 1) + j];
          }
        }
      }
      __syncthreads();
      if (active) {
        T inv = T(1) / Am[k * N + k];
        for (int j = t; j < (N - k - 1) + (LL + 1); j += TPE) {
          if (j < N - k - 1) Am[k * N + k + 1 + j] *= inv;
          else Rhs[k * (LL + 1) + (j - (N - k - 1))] *= inv;
        }
      }
      __syncthreads();
    }
    if (singular && t == 0) atomicCAS(p.status, 0, 1);
    __syncthreads();
    // U = -A^{-1}(...): negate the Schur solution columns in place
    if (active)
      for (int ic = t; ic < N * LL; ic += TPE) {
        int i = ic / LL, c = ic % LL;
        Rhs[i * (LL + 1) + c] = -Rhs[i * (LL + 1) + c];
      }
    __syncthreads();
    // ---- Q_d = -Xu_d U - Xl_d (in place over Xl) ; Q0_d = -Xu_d U0
    if (active) {
      for (int dic = t; dic < D * N * LL; dic += TPE) {
        int d = dic / (N * LL), i = (dic / LL) % N, c = dic % LL;
        T acc = 0.0;
        for (int m = 0; m < N; ++m) acc += Xu[(d * N + i) * N + m] * Rhs[m * (LL + 1) + c];
        Xl[dic] = -acc - Xl[dic];
      }
      for (int di = t; di < D * N; di += TPE) {
        int d = di / N, i = di % N;
        T acc = 0.0;
        for (int m = 0; m < N; ++m) acc += Xu[(d * N + i) * N + m] * Rhs[m * (LL + 1) + LL];
        Q0s[di] = Wq[di] - acc;
      }
    }
    __syncthreads();
    // ---- outputs: U, U0, Q, Q0 (column-major, HDGSolver.cpp:337-342)
    if (active) {
      T* Ug = (T*)p.U + e * LU * LL;
      for (int idx = t; p.writeOps && idx < LU * LL; idx += TPE) {
        int i = idx % LU, c = idx / LU;
        Ug[idx] = Rhs[i * (LL + 1) + c];
      }
      for (int i = t; i < LU; i += TPE) ((T*)p.U0)[e * LU + i] = Rhs[i * (LL + 1) + LL];
      T* Qg = (T*)p.Q + e * LQ * LL;
      for (int idx = t; p.writeOps && idx < LQ * LL; idx += TPE) {
        int r = idx % LQ, c = idx / LQ;
        int i = r / D, d = r % D;
        Qg[idx] = Xl[(d * N + i) * LL + c];
      }
      for (int r = t; r < LQ; r += TPE) ((T*)p.Q0)[e * LQ + r] = Q0s[(r % D) * N + r / D];
      // S = Sll + Slu U + Slq Q ; S0 = -Slu U0 - Slq Q0, then the Dirichlet Set rows
      T* Sg = (T*)p.S + e * LL * LL;
      for (int idx = t; p.writeOps && idx < LL * LL; idx += TPE) {
        int row = idx % LL, c = idx / LL;
        int f = row / NF, a = row % NF;
        T v;
        if (bnd[f]) {
          v = (row == c) ? 1.0 : 0.0;
        } else if (p.explicitMode) {
          v = (c / NF == f) ? -Tm[(f * NF + a) * NF + (c % NF)] : T(0);  // S = Sll
        } else {
          v = (c / NF == f) ? -Tm[(f * NF + a) * NF + (c % NF)] : 0.0;
          for (int b = 0; b < NF; ++b) {
            int nb = sFaceNodes[f * NF + b];
            v += Tm[(f * NF + a) * NF + b] * Rhs[nb * (LL + 1) + c];
            for (int d = 0; d < D; ++d) v -= Hm[((f * D + d) * NF + a) * NF + b] * Xl[(d * N + nb) * LL + c];
          }
        }
        Sg[idx] = v;
      }
      for (int row = t; row < LL; row += TPE) {
        int f = row / NF, a = row % NF;
        T v;
        if (bnd[f]) {
          v = rhsMode ? T(0) : (T)p.dirichlet[(int64_t)faceId[f] * NF + a];
        } else if (p.explicitMode) {
          // S0 = -Slu sol - Slq flux with the current state
          v = 0.0;
          for (int b = 0; b < NF; ++b) {
            int nb = sFaceNodes[f * NF + b];
            v -= Tm[(f * NF + a) * NF + b] * (T)p.solState[e * N + nb];
            for (int d = 0; d < D; ++d)
              v += Hm[((f * D + d) * NF + a) * NF + b] * (T)p.fluxState[e * N * D + nb * D + d];
          }
        } else {
          v = 0.0;
          for (int b = 0; b < NF; ++b) {
            int nb = sFaceNodes[f * NF + b];
            v -= Tm[(f * NF + a) * NF + b] * Rhs[nb * (LL + 1) + LL];
            for (int d = 0; d < D; ++d) v += Hm[((f * D + d) * NF + a) * NF + b] * Q0s[d * N + nb];
          }
        }
        ((T*)p.S0)[e * LL + row] = v;
      }
    }
    __syncthreads();
  }
}

template <typename T, int D, int P, int TPE, int EPC>
cudaError_t launch_t(const LocalParams& p, cudaStream_t s) {
  using L = Layout<T, D, P, TPE, EPC>;
  size_t smem = (size_t)L::TOTAL_DOUBLES * sizeof(T);
  auto kern = local_condense<T, D, P, TPE, EPC>;
  cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (err != cudaSuccess) return err;
  int dev = 0, nsm = 0, perSM = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, kern, TPE * EPC, smem);
  if (err != cudaSuccess) return err;
  if (perSM < 1) perSM = 1;
  int64_t need = (p.nCells + EPC - 1) / EPC;
  int64_t grid = (int64_t)nsm * perSM;
  if (grid > need) grid = need;
  if (grid < 1) grid = 1;
  kern<<<(unsigned)grid, TPE * EPC, smem, s>>>(p);
  return cudaGetLastError();
}

}  // namespace

bool local_condense_supported(int dim, int order) {
  return (dim == 2 && order >= 1 && order <= 5) || (dim == 3 && order >= 1 && order <= 3);
}

template <typename T>
cudaError_t launch_any(int dim, int order, const LocalParams& p, cudaStream_t s) {
  if (dim == 2) {
    switch (order) {
      case 1: return launch_t<T, 2, 1, 32, 8>(p, s);
      case 2: return launch_t<T, 2, 2, 32, 8>(p, s);
      case 3: return launch_t<T, 2, 3, 64, 4>(p, s);
      case 4: return launch_t<T, 2, 4, 64, 4>(p, s);
      case 5: return launch_t<T, 2, 5, 128, 2>(p, s);
    }
  } else if (dim == 3) {
    switch (order) {
      case 1: return launch_t<T, 3, 1, 64, 4>(p, s);
      case 2: return launch_t<T, 3, 2, 128, 2>(p, s);
      case 3: return launch_t<T, 3, 3, 256, 1>(p, s);
    }
  }
  return cudaErrorInvalidValue;
}

cudaError_t launch_local_condense(int dim, int order, const LocalParams& p, cudaStream_t s) {
  return p.fp32 ? launch_any<float>(dim, order, p, s) : launch_any<double>(dim, order, p, s);
}

}  // namespace hfx
