// HDG viscous Burgers element kernel (vector unknowns, nd = dim), FP64, sm_103a.
//
// One CTA of kBT threads owns one element at a time (grid-stride loop over the
// elements); the reference tables are staged once per CTA in shared memory.
// Restates, per element (HyperFox file:line):
//   Jacobians / measures / inverse   Operator.cpp:14-84, HDGModel.cpp:53-85
//   normals                          HDGBase.cpp:34-65
//   tau (nd x nd) at face IPs        HDGBase.cpp:18-32
//   HDGBase blocks, nd unknowns      HDGBase.cpp:67-158
//   HDGUNabU (u.grad u linearised)   HDGUNabU.cpp:27-193
//   HDGDiffusion blocks, nd unknowns HDGDiffusion.cpp:31-145
//   model composition                HDGBurgersModel.cpp:93-125 (one Source per component)
//   implicit Euler on the U rows     HDGModel.cpp:35-51, Euler.cpp:18-34, Operator.cpp:86-97
//   condensation U,Q,U0,Q0,S,S0      HDGSolver.cpp:331-348
//   Dirichlet Set on boundary faces  HDGSolver.cpp:361-529, DirichletModel.cpp:19-44
//
// Local layout (HDGBase.cpp:85-91): U row (i, c) = i*ND + c, Q row
// ((i*D + k)*ND + c), L row ((f*NF + a)*ND + c). The local matrix is never formed
// as a whole: the kernel builds the scalar blocks (mass M, C_k, the diffusion
// coupling K'_k, the face blocks E, H, the tau masses T and the convection face
// block) and condenses with Sqq = M (x) I, so Sqq^{-1} is one N x N inverse;
// the Schur block A = s (Suu - Suq Sqq^{-1} Squ) (+ M (x) I) couples the
// components and is solved by Gauss-Jordan with partial pivoting. Results equal
// the reference's dense QR condensation up to round-off.
//
// The blocks that depend only on geometry, tau and the diffusion field (M, M^-1 C_k,
// M^-1 E_k, the tau masses, H and the two Schur products) are stored per element by
// the first linearisation (cacheMode 1) and loaded by the later ones (cacheMode 2):
// a Newton iteration then recomputes only the convection terms, the Schur system,
// Q and S. The caller invalidates the cache when the mesh, tau or the diffusion
// field changes.
#include "hfx_device.h"

namespace hfx {
namespace {

constexpr int kBT = 128;  // threads per CTA = per element

template <int D, int P>
struct BL {
  using K = Dims<D, P>;
  static constexpr int N = K::N, NF = K::NF, F = K::F, NI = K::NI, NIF = K::NIF;
  static constexpr int ND = D, DM = D - 1, NT = ND * ND;
  static constexpr int NU = N * ND, NQ = D * N * ND, NLF = NF * ND, NL = F * NLF;
  static constexpr int W = NU + NL + 1;  // augmented row [A | -B | Fu]
  // tables, same packing as the quadrature kernel (phi, dphi, w, fphi, fdphi, fw)
  static constexpr int T_PHI = 0;
  static constexpr int T_DPHI = T_PHI + NI * N;
  static constexpr int T_W = T_DPHI + NI * N * D;
  static constexpr int T_FPHI = T_W + NI;
  static constexpr int T_FDPHI = T_FPHI + NIF * NF;
  static constexpr int T_FW = T_FDPHI + NIF * NF * DM;
  static constexpr int TAB = (T_FW + NIF + 1) & ~1;
  // element region (doubles, offsets from TAB)
  static constexpr int X = 0;                       // N*D coordinates
  static constexpr int UB = X + N * D;              // NU BufferSolution
  static constexpr int UO = UB + NU;                // NU old solution (implicit Euler)
  static constexpr int TR = UO + NU;                // NL local trace
  static constexpr int TAU = TR + NL;               // F*NF*NT local tau
  static constexpr int KAP = TAU + F * NF * NT;     // N*D*D nodal diffusion tensor
  static constexpr int IJ = KAP + N * D * D;        // NI*D*D inverse Jacobians
  static constexpr int DV = IJ + NI * D * D;        // NI
  static constexpr int DS = DV + NI;                // F*NIF
  static constexpr int NRM = DS + F * NIF;          // F*NIF*D
  static constexpr int SOL = NRM + F * NIF * D;     // NI*ND   u at the IPs
  static constexpr int DIV = SOL + NI * ND;         // NI      div u
  static constexpr int FSOL = DIV + NI;             // F*NIF*ND u (interior) at face IPs
  static constexpr int TN = FSOL + F * NIF * ND;    // F*NIF   (t.n) dS
  static constexpr int TAUQ = TN + F * NIF;         // F*NIF*NT dS tau
  static constexpr int DSKN = TAUQ + F * NIF * NT;  // F*NIF*D dS Ds n
  static constexpr int T1 = DSKN + F * NIF * D;     // N*N     sum_q AQ_qi phi_qj
  static constexpr int MM = T1 + N * N;             // N*N mass
  static constexpr int MI = MM + N * N;             // N*2N Gauss-Jordan [M | I] -> [I | M^-1]
  static constexpr int CK = MI + 2 * N * N;         // D*N*N  C_k
  static constexpr int MC = CK + D * N * N;         // D*N*N  M^-1 C_k
  static constexpr int KP = MC + D * N * N;         // D*N*N  K'_k
  static constexpr int EF = KP + D * N * N;         // F*D*NF*NF  E_fk
  static constexpr int ME = EF + F * D * NF * NF;   // D*N*F*NF   M^-1 E
  static constexpr int HF = ME + D * N * F * NF;    // F*D*NF*NF  H_fk
  static constexpr int TM = HF + F * D * NF * NF;   // F*NT*NF*NF tau masses [f][c][m][a][b]
  static constexpr int CLL = TM + F * NT * NF * NF; // F*NLF*NLF convection face blocks
  static constexpr int CUU = CLL + F * NLF * NLF;   // NU*NU convection volume block
  static constexpr int KM = CUU + NU * NU;          // N*N     sum_k K'_k M^-1 C_k
  static constexpr int KE = KM + N * N;             // N*F*NF  sum_k K'_k M^-1 E_k
  static constexpr int HMC = KE + N * F * NF;       // F*NF*N    sum_{b,k} H_fk[a][b] (M^-1 C_k)[fn(b)][j]
  static constexpr int HME = HMC + F * NF * N;      // F*NF*F*NF sum_{b,k} H_fk[a][b] (M^-1 E_k)[fn(b)][g]
  static constexpr int AUG = HME + F * NF * F * NF; // NU*W row-major (first holds X, NU*NU)
  static constexpr int QS = AUG + NU * W;           // per-IP arrays, then the right-hand-side parts
  // the per-IP arrays are dead before the right-hand-side parts are written
  static constexpr int G = QS;                      // NI*N*D  J^-1 grad phi
  static constexpr int KG = G + NI * N * D;         // NI*N*D  Ds J^-1 grad phi
  static constexpr int DSQ = KG + NI * N * D;       // NI*D*D  Ds at the volume IPs
  static constexpr int AQ = DSQ + NI * D * D;       // NI*N    (div u phi_i + u.grad phi_i) dV
  static constexpr int BQ = AQ + NI * N;            // NI*ND*N u_c dV phi_i
  static constexpr int QSZ = (BQ + NI * ND * N - QS) > NU * 4 ? (BQ + NI * ND * N - QS) : NU * 4;
  static constexpr int FL = QS + QSZ;               // NL
  static constexpr int TOTAL = TAB + FL + NL + 2;   // + pivot scalars
  // per-element cache of the parts that do not depend on the linearisation state
  // (geometry, tau, diffusion): M, M^-1 C_k, M^-1 E_k, tau masses, H_fk, the Schur products
  static constexpr int C_MM = 0;
  static constexpr int C_MC = C_MM + N * N;
  static constexpr int C_ME = C_MC + D * N * N;
  static constexpr int C_TM = C_ME + D * N * F * NF;
  static constexpr int C_HF = C_TM + F * NT * NF * NF;
  static constexpr int C_KM = C_HF + F * D * NF * NF;
  static constexpr int C_KE = C_KM + N * N;
  static constexpr int C_HMC = C_KE + N * F * NF;
  static constexpr int C_HME = C_HMC + F * NF * N;
  static constexpr int CL = C_HME + F * NF * F * NF;
  static_assert(TOTAL * 8 <= 227 * 1024, "element region exceeds the shared memory of one CTA");
};

template <int D, int P>
__global__ void __launch_bounds__(kBT) burgers_local(BurgersParams p) {
  using L = BL<D, P>;
  constexpr int N = L::N, NF = L::NF, F = L::F, NI = L::NI, NIF = L::NIF, DM = L::DM;
  constexpr int ND = L::ND, NT = L::NT, NU = L::NU, NLF = L::NLF, NL = L::NL, W = L::W;
  static_assert(D == 2, "the Burgers element kernel is built for 2D cells");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double* smem = reinterpret_cast<double*>(smem_raw);
  __shared__ int sFaceNodes[F * NF];
  __shared__ int sOpp[F];
  __shared__ int sPos[F * N];  // position of element node i on face f, -1 if not on it
  __shared__ int sFace[F], sBnd[F], sPiv;
  const int tid = threadIdx.x;
  {
    constexpr int nTab = L::T_FW + NIF;
    for (int i = tid; i < nTab; i += kBT) smem[i] = p.tab[i];
    for (int i = tid; i < F * NF; i += kBT) sFaceNodes[i] = p.itab[i];
    for (int i = tid; i < F; i += kBT) sOpp[i] = p.itab[F * NF + i];
    for (int i = tid; i < F * N; i += kBT) sPos[i] = -1;
    __syncthreads();
    for (int i = tid; i < F * NF; i += kBT) sPos[(i / NF) * N + sFaceNodes[i]] = i % NF;
    __syncthreads();
  }
  const double* phi = smem + L::T_PHI;
  const double* dphi = smem + L::T_DPHI;
  const double* w = smem + L::T_W;
  const double* fphi = smem + L::T_FPHI;
  const double* fdphi = smem + L::T_FDPHI;
  const double* fw = smem + L::T_FW;
  double* R = smem + L::TAB;
  double* X = R + L::X;
  double* ub = R + L::UB;
  double* uo = R + L::UO;
  double* tr = R + L::TR;
  double* tauL = R + L::TAU;
  double* kap = R + L::KAP;
  double* iJ = R + L::IJ;
  double* dV = R + L::DV;
  double* dS = R + L::DS;
  double* nrm = R + L::NRM;
  double* G = R + L::G;
  double* KG = R + L::KG;
  double* sol = R + L::SOL;
  double* divu = R + L::DIV;
  double* fsol = R + L::FSOL;
  double* tn = R + L::TN;
  double* tauq = R + L::TAUQ;
  double* dskn = R + L::DSKN;
  double* dsq = R + L::DSQ;
  double* aq = R + L::AQ;
  double* bq = R + L::BQ;
  double* t1 = R + L::T1;
  double* Mm = R + L::MM;
  double* MI = R + L::MI;
  double* Ck = R + L::CK;
  double* MC = R + L::MC;
  double* KP = R + L::KP;
  double* Ef = R + L::EF;
  double* ME = R + L::ME;
  double* Hf = R + L::HF;
  double* Tm = R + L::TM;
  double* Cll = R + L::CLL;
  double* Cuu = R + L::CUU;
  double* KMs = R + L::KM;
  double* KEs = R + L::KE;
  double* HMCs = R + L::HMC;
  double* HMEs = R + L::HME;
  double* Aug = R + L::AUG;
  double* Xc = R + L::AUG;  // X[(i,c),(j,m)] = sum_q u_qc dV_q phi_qi G_qjm, before the Schur system
  double* rhsPart = R + L::QS;  // NU*4 parts of the right-hand side column (after the per-IP arrays die)
  double* Fl = R + L::FL;
  double* pivInv = R + L::FL + NL;
  const bool diff = p.kc != 0;
  const bool euler = p.dt > 0.0;
  const bool load = p.cacheMode == 2, store = p.cacheMode == 1;
  const double s = euler ? p.dt : 1.0;

  for (int64_t e = blockIdx.x; e < p.nCells; e += gridDim.x) {
    // ------------------------------------------------------------ gather
    const int* cell = p.cells + e * N;
    for (int i = tid; i < N * D; i += kBT) X[i] = p.coords[(int64_t)cell[i / D] * D + (i % D)];
    for (int i = tid; i < NU; i += kBT) {
      ub[i] = p.buf[e * NU + i];
      uo[i] = euler ? p.uOld[e * NU + i] : 0.0;
    }
    for (int i = tid; i < F; i += kBT) {
      const int f = p.cell2face[e * F + i];
      sFace[i] = f;
      sBnd[i] = p.isBoundary[f];
    }
    for (int i = tid; i < F * NF; i += kBT) {
      const int f = p.cell2face[e * F + i / NF];
      const int side = (p.face2cell[2 * (int64_t)f] == (int)e) ? 0 : 1;
      const int q = p.perm[e * F * NF + i];
      for (int c = 0; c < ND; ++c) tr[i * ND + c] = p.trace[((int64_t)f * NF + q) * ND + c];
      const int64_t tb = (((int64_t)f * NF + q) * p.tauSides + (p.tauSides == 2 ? side : 0)) * NT;
      for (int v = 0; v < NT; ++v) tauL[i * NT + v] = p.tau[tb + v];
    }
    for (int i = tid; i < N * D * D; i += kBT) {
      const int n = i / (D * D), a = i % (D * D);
      double v = 0.0;
      if (diff) {
        const int64_t bk = p.nuLayout == 0 ? (int64_t)cell[n] * p.kc : (e * N + n) * p.kc;
        v = p.kc == 1 ? ((a % (D + 1) == 0) ? p.nu[bk] : 0.0) : p.nu[bk + a];
      }
      kap[i] = v;
    }
    if (load) {
      const double* ce = p.cache + e * L::CL;
      for (int i = tid; i < N * N; i += kBT) Mm[i] = ce[L::C_MM + i];
      for (int i = tid; i < D * N * N; i += kBT) MC[i] = ce[L::C_MC + i];
      for (int i = tid; i < D * N * F * NF; i += kBT) ME[i] = ce[L::C_ME + i];
      for (int i = tid; i < F * NT * NF * NF; i += kBT) Tm[i] = ce[L::C_TM + i];
      for (int i = tid; i < F * D * NF * NF; i += kBT) Hf[i] = ce[L::C_HF + i];
      for (int i = tid; i < N * N; i += kBT) KMs[i] = ce[L::C_KM + i];
      for (int i = tid; i < N * F * NF; i += kBT) KEs[i] = ce[L::C_KE + i];
      for (int i = tid; i < F * NF * N; i += kBT) HMCs[i] = ce[L::C_HMC + i];
      for (int i = tid; i < F * NF * F * NF; i += kBT) HMEs[i] = ce[L::C_HME + i];
    }
    __syncthreads();
    // ---------------------------------------------------------- geometry
    for (int q = tid; q < NI; q += kBT) {
      double J[D][D];
      for (int r = 0; r < D; ++r)
        for (int c = 0; c < D; ++c) {
          double acc = 0.0;
          for (int i = 0; i < N; ++i) acc += dphi[(q * N + i) * D + r] * X[i * D + c];
          J[r][c] = acc;
        }
      const double det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
      const double id = 1.0 / det;
      iJ[q * 4 + 0] = J[1][1] * id;   // (0,0)
      iJ[q * 4 + 1] = -J[0][1] * id;  // (0,1)
      iJ[q * 4 + 2] = -J[1][0] * id;  // (1,0)
      iJ[q * 4 + 3] = J[0][0] * id;   // (1,1)
      dV[q] = w[q] * det;
      if (!load)
        for (int a = 0; a < D * D; ++a) {  // Ds at q, column-major (HDGDiffusion.cpp:52-57)
          double acc = 0.0;
          if (diff)
            for (int n = 0; n < N; ++n) acc += phi[q * N + n] * kap[n * D * D + a];
          dsq[q * D * D + a] = acc;
        }
    }
    for (int fk = tid; fk < F * NIF; fk += kBT) {
      const int f = fk / NIF, k = fk % NIF;
      double j0 = 0.0, j1 = 0.0;
      for (int i = 0; i < NF; ++i) {
        const double g = fdphi[(k * NF + i) * DM];
        j0 += g * X[sFaceNodes[f * NF + i] * D + 0];
        j1 += g * X[sFaceNodes[f * NF + i] * D + 1];
      }
      const double ds = sqrt(j0 * j0 + j1 * j1);
      double n0 = -j1 / ds, n1 = j0 / ds;
      const int v0 = sFaceNodes[f * NF], vn = sOpp[f];
      const double prod = (X[vn * D] - X[v0 * D]) * n0 + (X[vn * D + 1] - X[v0 * D + 1]) * n1;
      if (prod > 0) {
        n0 = -n0;
        n1 = -n1;
      }
      dS[fk] = fw[k] * ds;
      nrm[fk * D] = n0;
      nrm[fk * D + 1] = n1;
    }
    __syncthreads();
    // ------------------------------------------- values at the integration points
    for (int qi = tid; qi < NI * N; qi += kBT) {
      const int q = qi / N, i = qi % N;
      double g[D];
      for (int a = 0; a < D; ++a) {
        double acc = 0.0;
        for (int b = 0; b < D; ++b) acc += iJ[q * 4 + a * 2 + b] * dphi[(q * N + i) * D + b];
        g[a] = acc;
        G[qi * D + a] = acc;
      }
      if (!load)
        for (int a = 0; a < D; ++a) {
          double acc = 0.0;
          for (int b = 0; b < D; ++b) acc += dsq[q * D * D + a + b * D] * g[b];
          KG[qi * D + a] = acc;
        }
    }
    for (int fq = tid; fq < F * NIF; fq += kBT) {
      const int f = fq / NIF, k = fq % NIF;
      const double ds = dS[fq];
      double trq[ND], dsf[D * D];
      for (int c = 0; c < ND; ++c) {
        double a1 = 0.0, a2 = 0.0;
        for (int a = 0; a < NF; ++a) {
          const double sh = fphi[k * NF + a];
          a1 += sh * ub[sFaceNodes[f * NF + a] * ND + c];
          a2 += sh * tr[(f * NF + a) * ND + c];
        }
        fsol[fq * ND + c] = a1;
        trq[c] = a2;
      }
      double t = 0.0;
      for (int c = 0; c < D; ++c) t += trq[c] * nrm[fq * D + c];
      tn[fq] = t * ds;
      if (load) continue;  // tau and the diffusion tensor at the face IPs feed cached blocks only
      for (int v = 0; v < NT; ++v) {
        double acc = 0.0;
        for (int a = 0; a < NF; ++a) acc += fphi[k * NF + a] * tauL[(f * NF + a) * NT + v];
        tauq[fq * NT + v] = ds * acc;
      }
      for (int v = 0; v < D * D; ++v) {
        double acc = 0.0;
        for (int a = 0; a < NF; ++a) acc += fphi[k * NF + a] * kap[sFaceNodes[f * NF + a] * D * D + v];
        dsf[v] = acc;
      }
      for (int a = 0; a < D; ++a) {
        double acc = 0.0;
        for (int b = 0; b < D; ++b) acc += dsf[a + b * D] * nrm[fq * D + b];
        dskn[fq * D + a] = ds * acc;
      }
    }
    for (int q = tid; q < NI; q += kBT) {
      for (int c = 0; c < ND; ++c) {
        double acc = 0.0;
        for (int i = 0; i < N; ++i) acc += phi[q * N + i] * ub[i * ND + c];
        sol[q * ND + c] = acc;
      }
    }
    __syncthreads();
    for (int q = tid; q < NI; q += kBT) {
      double acc = 0.0;  // trace of sum_i grad(phi_i) u_i^T (HDGUNabU.cpp:160-166)
      for (int i = 0; i < N; ++i)
        for (int k = 0; k < D; ++k) acc += G[(q * N + i) * D + k] * ub[i * ND + k];
      divu[q] = acc;
    }
    __syncthreads();
    for (int qi = tid; qi < NI * N; qi += kBT) {
      // factors of the volume convection block: AQ_qi = (div u phi_i + u.G_i) dV,
      // BQ_qci = u_c dV phi_i
      const int q = qi / N, i = qi % N;
      double sg = 0.0;
      for (int k = 0; k < D; ++k) sg += sol[q * ND + k] * G[qi * D + k];
      aq[qi] = (divu[q] * phi[qi] + sg) * dV[q];
      for (int c = 0; c < ND; ++c) bq[(q * ND + c) * N + i] = sol[q * ND + c] * dV[q] * phi[qi];
    }
    __syncthreads();
    // ------------------------------------------------------ scalar blocks
    if (load)
      for (int ij = tid; ij < N * N; ij += kBT) {
        const int i = ij / N, j = ij % N;
        double tt = 0.0;
        for (int q = 0; q < NI; ++q) tt += aq[q * N + i] * phi[q * N + j];
        t1[ij] = tt;
      }
    for (int ij = tid; ij < N * N && !load; ij += kBT) {
      const int i = ij / N, j = ij % N;
      double m = 0.0, c[D] = {}, kp[D] = {}, tt = 0.0;
      for (int q = 0; q < NI; ++q) {
        const double pj = phi[q * N + j] * dV[q];
        m += phi[q * N + i] * pj;
        tt += aq[q * N + i] * phi[q * N + j];
        for (int k = 0; k < D; ++k) {
          c[k] += G[(q * N + i) * D + k] * pj;
          kp[k] += KG[(q * N + i) * D + k] * pj;
        }
      }
      if (diff)
        for (int f = 0; f < F; ++f) {
          const int a = sPos[f * N + i], b = sPos[f * N + j];
          if (a < 0 || b < 0) continue;
          for (int k2 = 0; k2 < NIF; ++k2) {
            const double ss = fphi[k2 * NF + a] * fphi[k2 * NF + b];
            for (int k = 0; k < D; ++k) kp[k] -= dskn[(f * NIF + k2) * D + k] * ss;
          }
        }
      Mm[ij] = m;
      t1[ij] = tt;
      MI[i * 2 * N + j] = m;
      MI[i * 2 * N + N + j] = (i == j) ? 1.0 : 0.0;
      for (int k = 0; k < D; ++k) {
        Ck[k * N * N + ij] = c[k];
        KP[k * N * N + ij] = diff ? kp[k] : 0.0;
      }
    }
    for (int x = tid; x < F * D * NF * NF && !load; x += kBT) {
      // E_fk, H_fk: entry ((f*D + k)*NF + a)*NF + b
      const int f = x / (D * NF * NF), k = (x / (NF * NF)) % D, a = (x / NF) % NF, b = x % NF;
      double ev = 0.0, hv = 0.0;
      for (int k2 = 0; k2 < NIF; ++k2) {
        const int fq = f * NIF + k2;
        const double ss = fphi[k2 * NF + a] * fphi[k2 * NF + b];
        ev += dS[fq] * nrm[fq * D + k] * ss;
        hv += dskn[fq * D + k] * ss;
      }
      Ef[x] = ev;
      Hf[x] = diff ? hv : 0.0;
    }
    for (int x = tid; x < F * NT * NF * NF && !load; x += kBT) {
      // tau masses: entry (((f*ND + c)*ND + m)*NF + a)*NF + b, tau column-major ((c, m) at m*ND + c)
      const int f = x / (NT * NF * NF), c = (x / (ND * NF * NF)) % ND, m = (x / (NF * NF)) % ND;
      const int a = (x / NF) % NF, b = x % NF;
      double tv = 0.0;
      for (int k2 = 0; k2 < NIF; ++k2) {
        const int fq = f * NIF + k2;
        tv += tauq[fq * NT + m * ND + c] * (fphi[k2 * NF + a] * fphi[k2 * NF + b]);
      }
      Tm[x] = tv;
    }
    for (int x = tid; x < F * NLF * NLF; x += kBT) {
      // HDGUNabU face block (HDGUNabU.cpp:126-145): row (a, c), column (b, m)
      const int f = x / (NLF * NLF), r = (x / NLF) % NLF, cc = x % NLF;
      const int a = r / ND, c = r % ND, b = cc / ND, m = cc % ND;
      double acc = 0.0;
      for (int k2 = 0; k2 < NIF; ++k2) {
        const int fq = f * NIF + k2;
        const double ss = fphi[k2 * NF + a] * fphi[k2 * NF + b];
        acc += ((c == m ? tn[fq] : 0.0) + fsol[fq * ND + c] * nrm[fq * D + m] * dS[fq]) * ss;
      }
      Cll[x] = acc;
    }
    for (int x = tid; x < NU * NU; x += kBT) {
      // X[(i,c),(j,m)] = sum_q u_qc dV_q phi_qi G_qjm
      const int r = x / NU, cc = x % NU;
      const int i = r / ND, c = r % ND, j = cc / ND, m = cc % ND;
      double acc = 0.0;
      for (int q = 0; q < NI; ++q) acc += bq[(q * ND + c) * N + i] * G[(q * N + j) * D + m];
      Xc[x] = acc;
    }
    __syncthreads();
    for (int x = tid; x < NU * NU; x += kBT) {
      // HDGUNabU volume block (HDGUNabU.cpp:153-177), row (i, c), column (j, m):
      // -sum_q dV [d_cm (div u phi_i + u.G_i) phi_j + u_c (G_jm phi_i + G_im phi_j)]
      const int r = x / NU, cc = x % NU;
      const int i = r / ND, c = r % ND, j = cc / ND, m = cc % ND;
      Cuu[x] = -((c == m ? t1[i * N + j] : 0.0) + Xc[x] + Xc[(j * ND + c) * NU + i * ND + m]);
    }
    __syncthreads();
    if (!load) {
      // mass inverse: Gauss-Jordan on [M | I] (M is symmetric positive definite). Only
      // the columns right of the pivot are updated: the ones left of it are never read
      // again, and column k is read unchanged as the elimination factors.
      for (int k = 0; k < N; ++k) {
        const double pinv = 1.0 / MI[k * 2 * N + k];
        for (int j = k + 1 + tid; j < 2 * N; j += kBT) MI[k * 2 * N + j] *= pinv;
        __syncthreads();
        const int nc = 2 * N - k - 1;
        for (int x = tid; x < (N - 1) * nc; x += kBT) {
          int i = x / nc;
          const int j = k + 1 + x % nc;
          if (i >= k) ++i;
          MI[i * 2 * N + j] -= MI[i * 2 * N + k] * MI[k * 2 * N + j];
        }
        __syncthreads();
      }
      for (int x = tid; x < D * N * N; x += kBT) {
        const int k = x / (N * N), l = (x / N) % N, j = x % N;
        double acc = 0.0;
        for (int i = 0; i < N; ++i) acc += MI[l * 2 * N + N + i] * Ck[k * N * N + i * N + j];
        MC[x] = acc;
      }
      for (int x = tid; x < D * N * F * NF; x += kBT) {
        const int k = x / (N * F * NF), l = (x / (F * NF)) % N, fb = x % (F * NF);
        const int f = fb / NF, b = fb % NF;
        double acc = 0.0;
        for (int a = 0; a < NF; ++a)
          acc += MI[l * 2 * N + N + sFaceNodes[f * NF + a]] * Ef[((f * D + k) * NF + a) * NF + b];
        ME[x] = acc;
      }
      __syncthreads();
      if (diff) {
        // the Schur products sum_k K'_k M^-1 C_k and sum_k K'_k M^-1 E_k (shared by every
        // (c, m)), and the face products H M^-1 C, H M^-1 E that give S its Slq Q term
        constexpr int nKM = N * N, nKE = N * F * NF, nHC = F * NF * N, nHE = F * NF * F * NF;
        for (int x = tid; x < nKM + nKE + nHC + nHE; x += kBT) {
          double acc = 0.0;
          if (x >= nKM + nKE) {
            const int y = x - nKM - nKE;
            const bool hc = y < nHC;
            const int fa = hc ? y / N : (y - nHC) / (F * NF);
            const int col = hc ? y % N : (y - nHC) % (F * NF);
            const int f = fa / NF, a = fa % NF;
            for (int b = 0; b < NF; ++b) {
              const int jn = sFaceNodes[f * NF + b];
              for (int k = 0; k < D; ++k) {
                const double h = Hf[((f * D + k) * NF + a) * NF + b];
                acc += h * (hc ? MC[k * N * N + jn * N + col] : ME[(k * N + jn) * F * NF + col]);
              }
            }
            if (hc) HMCs[y] = acc;
            else HMEs[y - nHC] = acc;
          } else if (x < N * N) {
            const int i = x / N, j = x % N;
            for (int k = 0; k < D; ++k)
              for (int l = 0; l < N; ++l) acc += KP[k * N * N + i * N + l] * MC[k * N * N + l * N + j];
            KMs[x] = acc;
          } else {
            const int y = x - N * N, i = y / (F * NF), fb = y % (F * NF);
            for (int k = 0; k < D; ++k)
              for (int l = 0; l < N; ++l) acc += KP[k * N * N + i * N + l] * ME[(k * N + l) * F * NF + fb];
            KEs[y] = acc;
          }
        }
        __syncthreads();
      }
      if (store) {
        double* ce = p.cache + e * L::CL;
        for (int i = tid; i < N * N; i += kBT) ce[L::C_MM + i] = Mm[i];
        for (int i = tid; i < D * N * N; i += kBT) ce[L::C_MC + i] = MC[i];
        for (int i = tid; i < D * N * F * NF; i += kBT) ce[L::C_ME + i] = ME[i];
        for (int i = tid; i < F * NT * NF * NF; i += kBT) ce[L::C_TM + i] = Tm[i];
        for (int i = tid; i < F * D * NF * NF; i += kBT) ce[L::C_HF + i] = Hf[i];
        for (int i = tid; i < N * N; i += kBT) ce[L::C_KM + i] = diff ? KMs[i] : 0.0;
        for (int i = tid; i < N * F * NF; i += kBT) ce[L::C_KE + i] = diff ? KEs[i] : 0.0;
        for (int i = tid; i < F * NF * N; i += kBT) ce[L::C_HMC + i] = diff ? HMCs[i] : 0.0;
        for (int i = tid; i < F * NF * F * NF; i += kBT) ce[L::C_HME + i] = diff ? HMEs[i] : 0.0;
      }
    }
    // ------------------------------------- augmented Schur system [A | -B | Fu]
    for (int x = tid; x < NU * (W - 1); x += kBT) {
      const int r = x / (W - 1), col = x % (W - 1);
      const int i = r / ND, c = r % ND;
      double v;
      if (col < NU) {
        const int j = col / ND, m = col % ND;
        double base = 0.0;
        for (int f = 0; f < F; ++f) {
          const int a = sPos[f * N + i], b = sPos[f * N + j];
          if (a >= 0 && b >= 0) base += Tm[(((f * ND + c) * ND + m) * NF + a) * NF + b];
        }
        const double schur = (c == m && diff) ? KMs[i * N + j] : 0.0;
        v = s * (base + Cuu[r * NU + col] - schur) + ((euler && c == m) ? Mm[i * N + j] : 0.0);
      } else {
        const int cl = col - NU, f = cl / NLF, b = (cl % NLF) / ND, m = cl % ND;
        const int a = sPos[f * N + i];
        double sul = 0.0;
        if (a >= 0) sul = -Tm[(((f * ND + c) * ND + m) * NF + a) * NF + b] + Cll[(f * NLF + a * ND + c) * NLF + b * ND + m];
        const double schur = (c == m && diff) ? KEs[i * F * NF + f * NF + b] : 0.0;
        v = -s * (sul + schur);
      }
      Aug[r * W + col] = v;
    }
    // right-hand side column, four threads per U row: the HDGUNabU RHS (Cuu u + Cul t) / 2
    // (HDGUNabU.cpp:178-190) in two parts, the source, the implicit-Euler mass term
    for (int x = tid; x < NU * 4; x += kBT) {
      const int r = x / 4, part = x % 4;
      const int i = r / ND, c = r % ND;
      double acc = 0.0;
      if (part == 0) {
        for (int cc = 0; cc < NU; ++cc) acc += Cuu[r * NU + cc] * ub[cc];
      } else if (part == 1) {
        for (int f = 0; f < F; ++f) {
          const int a = sPos[f * N + i];
          if (a < 0) continue;
          for (int cc = 0; cc < NLF; ++cc) acc += Cll[(f * NLF + a * ND + c) * NLF + cc] * tr[f * NLF + cc];
        }
      } else if (part == 2) {
        if (p.src)
          for (int q = 0; q < NI; ++q) acc += phi[q * N + i] * p.src[(e * NI + q) * ND + c] * dV[q];
      } else if (euler) {
        for (int j = 0; j < N; ++j) acc += Mm[i * N + j] * uo[j * ND + c];
      }
      rhsPart[x] = acc;
    }
    for (int x = tid; x < NL; x += kBT) {
      // HDGUNabU RHS on the L rows: Cll t / 2 (the L-U convection block is zero)
      const int f = x / NLF, rr = x % NLF;
      double acc = 0.0;
      for (int cc = 0; cc < NLF; ++cc) acc += Cll[(f * NLF + rr) * NLF + cc] * tr[f * NLF + cc];
      Fl[x] = 0.5 * acc;
    }
    __syncthreads();
    for (int r = tid; r < NU; r += kBT) {
      const double* rp = rhsPart + 4 * r;
      Aug[r * W + W - 1] = s * (0.5 * (rp[0] + rp[1]) + rp[2]) + rp[3];
    }
    __syncthreads();
    // Gauss-Jordan with partial pivoting: [A | -B | Fu] -> [I | U | U0]. Columns left
    // of the pivot are never read again and are not updated; column k stays as the
    // elimination factors.
    bool singular = false;
    for (int k = 0; k < NU; ++k) {
      if (tid < 32) {
        // pivot: the first row r >= k of largest |A(r, k)| (the serial scan's choice)
        double best = -1.0;
        int br = NU;
        for (int r = k + tid; r < NU; r += 32) {
          const double v = fabs(Aug[r * W + k]);
          if (v > best) {
            best = v;
            br = r;
          }
        }
        for (int o = 16; o > 0; o >>= 1) {
          const double ob = __shfl_down_sync(0xffffffffu, best, o);
          const int orr = __shfl_down_sync(0xffffffffu, br, o);
          if (ob > best || (ob == best && orr < br)) {
            best = ob;
            br = orr;
          }
        }
        if (tid == 0) {
          sPiv = best > 0.0 ? br : -1;
          if (best > 0.0) pivInv[0] = 1.0 / Aug[br * W + k];
        }
      }
      __syncthreads();
      const int pr = sPiv;
      if (pr < 0) {
        singular = true;
        break;
      }
      const double pinv = pivInv[0];
      // swap rows k and pr (columns >= k), scale the new pivot row (columns > k)
      for (int j = k + tid; j < W; j += kBT) {
        const double a = Aug[k * W + j], b = Aug[pr * W + j];
        if (j == k) {
          Aug[pr * W + j] = a;  // the factor of row pr
        } else {
          Aug[k * W + j] = b * pinv;
          if (pr != k) Aug[pr * W + j] = a;
        }
      }
      __syncthreads();
      const int nc = W - k - 1;
      for (int x = tid; x < (NU - 1) * nc; x += kBT) {
        int i = x / nc;
        const int j = k + 1 + x % nc;
        if (i >= k) ++i;
        Aug[i * W + j] -= Aug[i * W + k] * Aug[k * W + j];
      }
      __syncthreads();
    }
    if (singular) {
      if (tid == 0) atomicCAS(p.status, 0, 1);
      __syncthreads();
      continue;
    }
    // ------------------------------------------------ U, U0 out; Q, Q0
    for (int x = tid; x < NU * (NL + 1); x += kBT) {
      const int r = x % NU, cl = x / NU;  // consecutive threads on consecutive rows
      const double v = Aug[r * W + NU + cl];
      if (cl < NL) p.U[e * NU * NL + (int64_t)cl * NU + r] = v;
      else p.U0[e * NU + r] = v;
    }
    __syncthreads();
    // ------------------------------------------- S, S0 (+ Dirichlet Set)
    for (int x = tid; x < NL * (NL + 1); x += kBT) {
      const int row = x % NL, cl = x / NL;
      const int f = row / NLF, a = (row % NLF) / ND, c = row % ND;
      double v;
      if (sBnd[f]) {
        // Set: identity rows, face-ordered Dirichlet values as they are
        v = cl < NL ? (cl == row ? 1.0 : 0.0) : p.dirichlet[(int64_t)sFace[f] * NLF + (row % NLF)];
      } else {
        double acc = 0.0;
        for (int b = 0; b < NF; ++b) {
          const int jn = sFaceNodes[f * NF + b];
          for (int m = 0; m < ND; ++m)
            acc += Tm[(((f * ND + c) * ND + m) * NF + a) * NF + b] * Aug[(jn * ND + m) * W + NU + cl];
        }
        if (diff) {
          // Slq Q with Q = -(M^-1 C (x) I) U + (M^-1 E (x) I): H M^-1 C U - H M^-1 E
          for (int j = 0; j < N; ++j) acc += HMCs[(f * NF + a) * N + j] * Aug[(j * ND + c) * W + NU + cl];
          if (cl < NL && cl % ND == c) acc -= HMEs[(f * NF + a) * F * NF + (cl / NLF) * NF + (cl % NLF) / ND];
        }
        if (cl < NL) {
          const int f2 = cl / NLF, b = (cl % NLF) / ND, m = cl % ND;
          if (f2 == f)
            acc += -Tm[(((f * ND + c) * ND + m) * NF + a) * NF + b] + Cll[(f * NLF + a * ND + c) * NLF + b * ND + m];
          v = acc;
        } else {
          v = Fl[row] - acc;
        }
      }
      if (cl < NL) p.S[e * NL * NL + (int64_t)cl * NL + row] = v;
      else p.S0[e * NL + row] = v;
    }
    __syncthreads();
  }
}

// Local recovery (HDGSolver.cpp:741-775), one CTA per element: Solution = U lambda + U0,
// and Flux = Q lambda + Q0 with Q = -(M^-1 C (x) I) U + (M^-1 E (x) I), Q0 = -(M^-1 C (x) I) U0,
// i.e. Flux = -(M^-1 C (x) I) Solution + (M^-1 E (x) I) lambda from the per-element cache.
template <int D, int P>
__global__ void __launch_bounds__(128) burgers_recover(BurgersRecoverParams p) {
  using L = BL<D, P>;
  constexpr int N = L::N, NF = L::NF, F = L::F, ND = L::ND, NU = L::NU, NQ = L::NQ, NLF = L::NLF, NL = L::NL;
  __shared__ double lam[NL], sol[NU];
  for (int64_t e = blockIdx.x; e < p.nCells; e += gridDim.x) {
    for (int j = threadIdx.x; j < NL; j += blockDim.x) {
      const int i = j / NLF;
      const int f = p.cell2face[e * F + i];
      lam[j] = p.trace[(int64_t)f * NLF + p.permx[(e * F + i) * NLF + (j % NLF)]];
    }
    __syncthreads();
    const double* U = p.U + e * NU * NL;
    for (int r = threadIdx.x; r < NU; r += blockDim.x) {
      double acc = p.U0[e * NU + r];
      for (int c2 = 0; c2 < NL; ++c2) acc += U[r + (int64_t)c2 * NU] * lam[c2];
      sol[r] = acc;
      p.sol[e * NU + r] = acc;
    }
    __syncthreads();
    const double* ce = p.cache + e * L::CL;
    for (int rq = threadIdx.x; rq < NQ; rq += blockDim.x) {
      const int l = rq / (D * ND), k = (rq / ND) % D, c = rq % ND;
      double acc = 0.0;
      for (int j = 0; j < N; ++j) acc -= ce[L::C_MC + k * N * N + l * N + j] * sol[j * ND + c];
      for (int g = 0; g < F * NF; ++g) acc += ce[L::C_ME + (k * N + l) * F * NF + g] * lam[g * ND + c];
      p.flux[e * NQ + rq] = acc;
    }
    __syncthreads();
  }
}

// Q and Q0 of every element from U, U0 and the cache, for the export of the condensed blocks:
// Q = -(M^-1 C (x) I) U + (M^-1 E (x) I), Q0 = -(M^-1 C (x) I) U0 (column-major per element).
template <int D, int P>
__global__ void burgers_q_from_u(int64_t nCells, const double* __restrict__ U, const double* __restrict__ U0,
                                 const double* __restrict__ cache, double* __restrict__ Q, double* __restrict__ Q0) {
  using L = BL<D, P>;
  constexpr int N = L::N, NF = L::NF, F = L::F, ND = L::ND, NU = L::NU, NQ = L::NQ, NLF = L::NLF, NL = L::NL;
  const int64_t total = nCells * NQ * (NL + 1);
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = idx / (NQ * (NL + 1));
    const int r = (int)(idx % (NQ * (NL + 1)));
    const int rq = r % NQ, cl = r / NQ;
    const int l = rq / (D * ND), k = (rq / ND) % D, c = rq % ND;
    const double* ce = cache + e * L::CL;
    double acc = 0.0;
    for (int j = 0; j < N; ++j)
      acc -= ce[L::C_MC + k * N * N + l * N + j] *
             (cl < NL ? U[e * NU * NL + (int64_t)cl * NU + j * ND + c] : U0[e * NU + j * ND + c]);
    if (cl < NL) {
      const int f = cl / NLF, b = (cl % NLF) / ND, m = cl % ND;
      if (m == c) acc += ce[L::C_ME + (k * N + l) * F * NF + f * NF + b];
      Q[e * NQ * NL + (int64_t)cl * NQ + rq] = acc;
    } else {
      Q0[e * NQ + rq] = acc;
    }
  }
}

template <int D, int P>
cudaError_t launch_t(const BurgersParams& p, cudaStream_t s) {
  using L = BL<D, P>;
  const size_t bytes = sizeof(double) * L::TOTAL;
  cudaError_t e = cudaFuncSetAttribute(burgers_local<D, P>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e != cudaSuccess) return e;
  int dev = 0, nsm = 0, perSM = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, burgers_local<D, P>, kBT, bytes);
  if (e != cudaSuccess) return e;
  if (perSM < 1) return cudaErrorInvalidConfiguration;
  int64_t grid = (int64_t)nsm * perSM;
  if (grid > p.nCells) grid = p.nCells;
  burgers_local<D, P><<<(unsigned)(grid < 1 ? 1 : grid), kBT, bytes, s>>>(p);
  return cudaGetLastError();
}

// Newton residual parts of NonLinearWrapper::vanillaResidualComputer
// (NonLinearWrapper.cpp:14-34): sum (sol - buf)^2 and sum buf^2 per block, the
// block sums added in block order by the last block (no atomics on the values).
constexpr int kRT = 256;
__global__ void __launch_bounds__(kRT) newton_residual(int64_t n, const double* __restrict__ sol,
                                                       const double* __restrict__ buf, double* __restrict__ partials,
                                                       unsigned* ticket, double* out) {
  __shared__ double rd[kRT / 32], rb[kRT / 32];
  __shared__ bool last;
  double d2 = 0.0, b2 = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * kRT + threadIdx.x; i < n; i += (int64_t)gridDim.x * kRT) {
    const double d = sol[i] - buf[i];
    d2 += d * d;
    b2 += buf[i] * buf[i];
  }
  for (int o = 16; o > 0; o >>= 1) {
    d2 += __shfl_down_sync(0xffffffffu, d2, o);
    b2 += __shfl_down_sync(0xffffffffu, b2, o);
  }
  if ((threadIdx.x & 31) == 0) {
    rd[threadIdx.x >> 5] = d2;
    rb[threadIdx.x >> 5] = b2;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int k = 0; k < kRT / 32; ++k) {
      a += rd[k];
      b += rb[k];
    }
    partials[2 * blockIdx.x] = a;
    partials[2 * blockIdx.x + 1] = b;
    __threadfence();
    last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (last && threadIdx.x == 0) {
    __threadfence();
    double a = 0.0, b = 0.0;
    for (unsigned k = 0; k < gridDim.x; ++k) {
      a += ((volatile double*)partials)[2 * k];
      b += ((volatile double*)partials)[2 * k + 1];
    }
    out[0] = a;
    out[1] = b;
    *ticket = 0u;
  }
}

// NonLinearWrapper::solve's update (NonLinearWrapper.cpp:64-70): both fields
// become (1 - d) sol + d buf.
__global__ void newton_update(int64_t n, double damp, double* __restrict__ sol, double* __restrict__ buf) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double v = (1.0 - damp) * sol[i] + damp * buf[i];
    sol[i] = v;
    buf[i] = v;
  }
}

}  // namespace

bool burgers_supported(int dim, int order) { return dim == 2 && order >= 1 && order <= 5; }

size_t burgers_smem_bytes(int dim, int order) {
  if (dim != 2) return 0;
  switch (order) {
    case 1: return sizeof(double) * BL<2, 1>::TOTAL;
    case 2: return sizeof(double) * BL<2, 2>::TOTAL;
    case 3: return sizeof(double) * BL<2, 3>::TOTAL;
    case 4: return sizeof(double) * BL<2, 4>::TOTAL;
    case 5: return sizeof(double) * BL<2, 5>::TOTAL;
  }
  return 0;
}

size_t burgers_cache_doubles(int dim, int order) {
  if (dim != 2) return 0;
  switch (order) {
    case 1: return BL<2, 1>::CL;
    case 2: return BL<2, 2>::CL;
    case 3: return BL<2, 3>::CL;
    case 4: return BL<2, 4>::CL;
    case 5: return BL<2, 5>::CL;
  }
  return 0;
}

cudaError_t launch_burgers_local(int dim, int order, const BurgersParams& p, cudaStream_t s) {
  if (dim == 2) switch (order) {
      case 1: return launch_t<2, 1>(p, s);
      case 2: return launch_t<2, 2>(p, s);
      case 3: return launch_t<2, 3>(p, s);
      case 4: return launch_t<2, 4>(p, s);
      case 5: return launch_t<2, 5>(p, s);
    }
  return cudaErrorInvalidValue;
}

cudaError_t launch_burgers_recover(int dim, int order, const BurgersRecoverParams& p, cudaStream_t s) {
  const int64_t g = p.nCells < 152 * 64 ? p.nCells : 152 * 64;
  const unsigned grid = (unsigned)(g < 1 ? 1 : g);
  if (dim == 2) switch (order) {
      case 1: burgers_recover<2, 1><<<grid, 128, 0, s>>>(p); return cudaGetLastError();
      case 2: burgers_recover<2, 2><<<grid, 128, 0, s>>>(p); return cudaGetLastError();
      case 3: burgers_recover<2, 3><<<grid, 128, 0, s>>>(p); return cudaGetLastError();
      case 4: burgers_recover<2, 4><<<grid, 128, 0, s>>>(p); return cudaGetLastError();
      case 5: burgers_recover<2, 5><<<grid, 128, 0, s>>>(p); return cudaGetLastError();
    }
  return cudaErrorInvalidValue;
}

cudaError_t launch_burgers_q(int dim, int order, int64_t nCells, const double* U, const double* U0,
                             const double* cache, double* Q, double* Q0, cudaStream_t s) {
  const unsigned grid = 152 * 16;
  if (dim == 2) switch (order) {
      case 1: burgers_q_from_u<2, 1><<<grid, 256, 0, s>>>(nCells, U, U0, cache, Q, Q0); return cudaGetLastError();
      case 2: burgers_q_from_u<2, 2><<<grid, 256, 0, s>>>(nCells, U, U0, cache, Q, Q0); return cudaGetLastError();
      case 3: burgers_q_from_u<2, 3><<<grid, 256, 0, s>>>(nCells, U, U0, cache, Q, Q0); return cudaGetLastError();
      case 4: burgers_q_from_u<2, 4><<<grid, 256, 0, s>>>(nCells, U, U0, cache, Q, Q0); return cudaGetLastError();
      case 5: burgers_q_from_u<2, 5><<<grid, 256, 0, s>>>(nCells, U, U0, cache, Q, Q0); return cudaGetLastError();
    }
  return cudaErrorInvalidValue;
}

constexpr int kResidualBlocks = 152 * 2;
size_t newton_partials_needed() { return 2 * kResidualBlocks; }

cudaError_t launch_newton_residual(int64_t n, const double* sol, const double* buf, double* partials,
                                   unsigned* ticket, double* out, cudaStream_t s) {
  int64_t g = (n + kRT - 1) / kRT;
  if (g > kResidualBlocks) g = kResidualBlocks;
  newton_residual<<<(unsigned)(g < 1 ? 1 : g), kRT, 0, s>>>(n, sol, buf, partials, ticket, out);
  return cudaGetLastError();
}

cudaError_t launch_newton_update(int64_t n, double damp, double* sol, double* buf, cudaStream_t s) {
  int64_t g = (n + 255) / 256;
  if (g > 152 * 16) g = 152 * 16;
  newton_update<<<(unsigned)(g < 1 ? 1 : g), 256, 0, s>>>(n, damp, sol, buf);
  return cudaGetLastError();
}

}  // namespace hfx
