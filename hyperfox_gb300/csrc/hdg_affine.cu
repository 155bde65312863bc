// Per-element HDG assembly + static condensation for straight-sided (affine)
// simplices with a diffusion tensor that is constant and symmetric inside each
// cell, FP64, sm_103a.
//
// Same blocks and the same condensed outputs as hdg_local.cu (which restates
// HDGBase.cpp:67-158, HDGDiffusion.cpp:74-145, Source.cpp:24-48, Euler.cpp:18-34
// and the condensation of HDGSolver.cpp:331-348), computed from reference
// operators instead of quadrature per element. With J the constant Jacobian,
// G = J^{-1}, K the cell tensor, |F_f| and n_f the face measure and unit outward
// normal, the reference tables M, C_r (C_r[i][j] = int d_r phi_i phi_j),
// R_rs = C_r^T M^{-1} C_s, L_f = M^{-1} E_f (E_f the face-mass coupling),
// P_rf = C_r^T L_f, T_ff' = E_f^T L_f' and T_f[a][b][c] = int_f mu_a mu_b mu_c give
//   Tm_f = |F_f| sum_c tau_c T_f[.,.,c]                        (tau face mass)
//   A    = dt (sum_f Tm_f + |J| sum_rs (G^T K G)_sr R_rs) + |J| M [time scheme]
//   B    = -Tm_f - |F_f| sum_r (n_f^T K G)_r P_rf                (N x LL)
//   C    = -Tm_f delta_ff' - |F_f||F_f'|/|J| (n_f'^T K n_f) T_ff'
//   U = -dt A^{-1} B, U0 = A^{-1} f_u, S = C + dt B^T A^{-1} B, S0 = B^T U0
// (B' = Slu - Slq Xu equals -B^T because K is symmetric: the local system is
// symmetric after eliminating Q = -Xu U - Xl Lambda). A is symmetric positive
// definite; with its Cholesky factor L and W = L^{-1} B, S = C + dt W^T W.
// About 47k FP64 FMAs per p=3 tetrahedron instead of about 0.5M by quadrature.
//
// Q and Q0 are not stored: the recovery forms the flux from U and Lambda,
// Q = -Xu (U Lambda + U0) - Xl Lambda with Xu = G . M^{-1} C and
// Xl = -(|F_f|/|J|) n_f L_f, from the per-element factors in geo[] =
// [G (D x D) | (|F_f|/|J|) n_f (F x D)].
#include <cmath>
#include <vector>

#include "hfx_device.h"
#include "hfx_host.h"

namespace hfx {

// ------------------------------------------------------------------ host tables

static bool small_inverse(int n, const std::vector<double>& A, std::vector<double>* inv) {
  std::vector<double> a(A);
  inv->assign((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i) (*inv)[(size_t)i * n + i] = 1.0;
  for (int k = 0; k < n; ++k) {
    int piv = k;
    for (int i = k + 1; i < n; ++i)
      if (std::fabs(a[(size_t)i * n + k]) > std::fabs(a[(size_t)piv * n + k])) piv = i;
    if (a[(size_t)piv * n + k] == 0.0) return false;
    for (int j = 0; j < n; ++j) {
      std::swap(a[(size_t)k * n + j], a[(size_t)piv * n + j]);
      std::swap((*inv)[(size_t)k * n + j], (*inv)[(size_t)piv * n + j]);
    }
    double d = 1.0 / a[(size_t)k * n + k];
    for (int j = 0; j < n; ++j) {
      a[(size_t)k * n + j] *= d;
      (*inv)[(size_t)k * n + j] *= d;
    }
    for (int i = 0; i < n; ++i) {
      if (i == k) continue;
      double l = a[(size_t)i * n + k];
      if (l == 0.0) continue;
      for (int j = 0; j < n; ++j) {
        a[(size_t)i * n + j] -= l * a[(size_t)k * n + j];
        (*inv)[(size_t)i * n + j] -= l * (*inv)[(size_t)k * n + j];
      }
    }
  }
  return true;
}

bool affine_tables(const RefEl& re, std::vector<double>* out) {
  const int D = re.dim, N = re.nNodes, NF = re.nNodesFace, F = D + 1, NI = re.nIP, NIF = re.nIPFace;
  const double *phi = re.phi.data(), *dphi = re.dphi.data(), *w = re.ipW.data(), *fphi = re.fPhi.data(),
               *fw = re.fIpW.data();
  std::vector<double> M((size_t)N * N, 0.0), Mi;
  for (int q = 0; q < NI; ++q)
    for (int i = 0; i < N; ++i)
      for (int j = 0; j < N; ++j) M[(size_t)i * N + j] += w[q] * phi[q * N + i] * phi[q * N + j];
  if (!small_inverse(N, M, &Mi)) return false;
  std::vector<double> C((size_t)D * N * N, 0.0);  // C[r][i][j] = sum_q w d_r phi_i phi_j
  for (int q = 0; q < NI; ++q)
    for (int r = 0; r < D; ++r)
      for (int i = 0; i < N; ++i)
        for (int j = 0; j < N; ++j)
          C[((size_t)r * N + i) * N + j] += w[q] * dphi[(q * N + i) * D + r] * phi[q * N + j];
  std::vector<double> Dr((size_t)D * N * N, 0.0);  // M^{-1} C_r
  for (int r = 0; r < D; ++r)
    for (int i = 0; i < N; ++i)
      for (int j = 0; j < N; ++j) {
        double s = 0.0;
        for (int k = 0; k < N; ++k) s += Mi[(size_t)i * N + k] * C[((size_t)r * N + k) * N + j];
        Dr[((size_t)r * N + i) * N + j] = s;
      }
  std::vector<double> R((size_t)D * D * N * N, 0.0);  // R[r][s][i][j] = sum_m C_r[m][i] Dr_s[m][j]
  for (int r = 0; r < D; ++r)
    for (int s = 0; s < D; ++s)
      for (int i = 0; i < N; ++i)
        for (int j = 0; j < N; ++j) {
          double v = 0.0;
          for (int m = 0; m < N; ++m) v += C[((size_t)r * N + m) * N + i] * Dr[((size_t)s * N + m) * N + j];
          R[(((size_t)r * D + s) * N + i) * N + j] = v;
        }
  std::vector<double> Mf((size_t)NF * NF, 0.0), Tf((size_t)NF * NF * NF, 0.0);
  for (int k = 0; k < NIF; ++k)
    for (int a = 0; a < NF; ++a)
      for (int b = 0; b < NF; ++b) {
        double ab = fw[k] * fphi[k * NF + a] * fphi[k * NF + b];
        Mf[(size_t)a * NF + b] += ab;
        for (int c = 0; c < NF; ++c) Tf[((size_t)a * NF + b) * NF + c] += ab * fphi[k * NF + c];
      }
  std::vector<double> L((size_t)F * N * NF, 0.0);  // L_f = M^{-1} E_f
  for (int f = 0; f < F; ++f)
    for (int i = 0; i < N; ++i)
      for (int b = 0; b < NF; ++b) {
        double s = 0.0;
        for (int a = 0; a < NF; ++a) s += Mi[(size_t)i * N + re.faceNodes[f * NF + a]] * Mf[(size_t)a * NF + b];
        L[((size_t)f * N + i) * NF + b] = s;
      }
  std::vector<double> P((size_t)D * F * N * NF, 0.0);  // P[r][f][i][b] = sum_m C_r[m][i] L_f[m][b]
  for (int r = 0; r < D; ++r)
    for (int f = 0; f < F; ++f)
      for (int i = 0; i < N; ++i)
        for (int b = 0; b < NF; ++b) {
          double s = 0.0;
          for (int m = 0; m < N; ++m) s += C[((size_t)r * N + m) * N + i] * L[((size_t)f * N + m) * NF + b];
          P[(((size_t)r * F + f) * N + i) * NF + b] = s;
        }
  std::vector<double> T((size_t)F * F * NF * NF, 0.0);  // T[f][g][a][b] = sum_a' Mf[a][a'] L_g[fn(f,a')][b]
  for (int f = 0; f < F; ++f)
    for (int g = 0; g < F; ++g)
      for (int a = 0; a < NF; ++a)
        for (int b = 0; b < NF; ++b) {
          double s = 0.0;
          for (int a2 = 0; a2 < NF; ++a2)
            s += Mf[(size_t)a * NF + a2] * L[((size_t)g * N + re.faceNodes[f * NF + a2]) * NF + b];
          T[(((size_t)f * F + g) * NF + a) * NF + b] = s;
        }
  out->clear();
  for (auto* v : {&M, &R, &Tf, &P, &T, &Dr, &L}) out->insert(out->end(), v->begin(), v->end());
  out->insert(out->end(), re.ipX.begin(), re.ipX.end());  // volume IPs, for the source
  out->insert(out->end(), C.begin(), C.end());            // C_r, for Runge-Kutta stages
  out->insert(out->end(), Mf.begin(), Mf.end());          // face mass
  return true;
}

// ------------------------------------------------------------------ device

namespace {

// W^T W in double-float arithmetic on the FP32 pipe (GB300's FP32 pipe is
// about 64x its FP64 one): every W entry is a pair hi + lo of floats, products
// are split exactly with an FMA (two-product) and sums carried with Knuth's
// two-sum, the double-float scheme of Dekker (1971) and of the QD library
// (Hida, Li, Bailey 2001); about 44 significant bits per accumulated term.
// The _rn intrinsics keep the compiler from contracting the error terms.
__device__ __forceinline__ void ds_mac(float& sh, float& sl, float2 a, float2 b) {
  const float p = __fmul_rn(a.x, b.x);
  float e = fmaf(a.x, b.x, -p);
  e = fmaf(a.x, b.y, e);
  e = fmaf(a.y, b.x, e);
  const float s = __fadd_rn(sh, p);
  const float bb = __fsub_rn(s, sh);
  float t = __fadd_rn(__fsub_rn(sh, __fsub_rn(s, bb)), __fsub_rn(p, bb));
  t = __fadd_rn(t, __fadd_rn(sl, e));
  sh = __fadd_rn(s, t);
  sl = __fsub_rn(t, __fsub_rn(sh, s));
}

template <int D, int P>
struct AffLayout {
  using K = Dims<D, P>;
  static constexpr int N = K::N, NF = K::NF, F = K::F, NI = K::NI, NIF = K::NIF, LL = K::LL;
  // table offsets in the affine table block
  static constexpr int A_M = 0;
  static constexpr int A_R = A_M + N * N;
  static constexpr int A_TF = A_R + D * D * N * N;
  static constexpr int A_P = A_TF + NF * NF * NF;
  static constexpr int A_T = A_P + D * F * N * NF;
  static constexpr int A_D = A_T + F * F * NF * NF;
  static constexpr int A_L = A_D + D * N * N;
  static constexpr int A_X = A_L + F * N * NF;  // [NI][D] reference IP coordinates
  static constexpr int A_C = A_X + NI * D;      // [D][N][N] C_r[i][j] = sum_q w d_r phi_i phi_j
  static constexpr int A_MF = A_C + D * N * N;  // [NF][NF] reference face mass
  static constexpr int A_END = A_MF + NF * NF;
  // per-element precomputed factors (affine_prep): G, |J|, |F_f|, n_f, Gamma,
  // g_f, c_ff', f(x_q) w_q |J|, K
  static constexpr int P_IV = 0, P_DET = P_IV + D * D, P_AR = P_DET + 1, P_NRM = P_AR + F, P_GAM = P_NRM + F * D;
  static constexpr int P_GV = P_GAM + D * D, P_CFF = P_GV + F * D, P_KS = P_CFF + F * F, P_FQ = P_KS + D * D;
  static constexpr int PREP = P_FQ + NI;
  static constexpr int P_SMEM = P_FQ;  // the part of the record staged in shared memory
  // offsets in the packed quadrature table (phi, dphi, w, fphi, fdphi, fw)
  static constexpr int T_PHI = 0;
  static constexpr int T_DPHI = T_PHI + NI * N;
  static constexpr int T_W = T_DPHI + NI * N * D;
  static constexpr int T_FPHI = T_W + NI;
  static constexpr int T_FDPHI = T_FPHI + NIF * NF;
  // per-warp shared region (doubles)
  static constexpr int LW = LL + 1;              // columns of [B | f_u]
  static constexpr int H0 = LL / 2;              // columns of B in the first pass
  static constexpr int LWH = LL - H0 + 1;        // widest pass: the second, with f_u
  static constexpr int NT = NF * (NF + 1) / 2;
  static constexpr int PR = 0;                   // P_SMEM  the element's affine_prep record
  static constexpr int TM = PR + P_SMEM;         // F*NT  tau face masses, symmetric, packed
  static constexpr int AM = TM + F * NT;         // N(N+1)/2  lower triangle of A by rows, then L
                                                 //   with 1 / L[k][k] on the diagonal
  static constexpr int BW = AM + N * (N + 1) / 2; // N*LWH  the columns of one pass, row-major
  static constexpr int FU = BW + N * LWH;        // N     f_u
  static constexpr int Y0P = FU + N;             // N     y0 = L^{-1} f_u as float pairs
  static constexpr int WDS = (Y0P + N + 1) & ~1; // N*LL  W as float pairs (hi, lo)
  // before W exists its region holds the Runge-Kutta stage vector w (u, q,
  // lambda parts), y_r = (K G)^T w_q, K n_f, K G, and the face tau values
  static constexpr int RKU = WDS;                // N
  static constexpr int RKQ = RKU + N;            // N*D
  static constexpr int RKL = RKQ + N * D;        // F*NF
  static constexpr int RKY = RKL + F * NF;       // D*N
  static constexpr int RKN = RKY + D * N;        // F*D
  static constexpr int RKG = RKN + F * D;        // D*D
  static constexpr int TAU = RKG + D * D;        // F*NF
  static constexpr int WARP = (WDS + N * LL > TAU + F * NF) ? WDS + N * LL : TAU + F * NF;
};

// Per-element geometry and source, one thread per element (full warps): the
// affine Jacobian from the vertices (J[r][s] = (x_{r+1} - x_0)_s / 2 on the
// reference simplex with vertices (-1,..), e_r), its inverse G, the face
// measures and outward unit normals (face vertices first in every face-node
// list), Gamma = G^T K G, g_f = n_f^T K G, c_ff', the source at the IPs
// (affine map of the reference IPs), the cell tensor K, and the recovery factors.
template <int D, int P>
__global__ void affine_prep(LocalParams p, const double* __restrict__ atab, double* __restrict__ prep,
                            double* __restrict__ geo) {
  using L = AffLayout<D, P>;
  constexpr int N = L::N, NF = L::NF, F = L::F, NI = L::NI;
  const int* fnAll = p.itab;          // faceNodes [F][NF]
  const int* opp = p.itab + F * NF;   // faceOpposite [F]
  const double* ipx = atab + L::A_X;
  const double* wq = p.tab + L::T_W;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < p.nCells; e += (int64_t)gridDim.x * blockDim.x) {
    const int* cell = p.cells + e * N;
    double* out = prep + e * L::PREP;
    double X[D + 1][D];
    for (int m = 0; m <= D; ++m)
      for (int c = 0; c < D; ++c) X[m][c] = p.coords[(int64_t)cell[m] * D + c];
    double K[D][D];  // K[d][b] from the column-major cell tensor
    for (int a = 0; a < D * D; ++a) {
      double v;
      if (p.kc == 0) v = (a % (D + 1) == 0) ? 1.0 : 0.0;
      else {
        int64_t bk = p.kappaLayout == 0 ? (int64_t)cell[0] * p.kc : (e * N) * p.kc;
        v = p.kc == 1 ? ((a % (D + 1) == 0) ? p.kappa[bk] : 0.0) : p.kappa[bk + a];
      }
      K[a % D][a / D] = v;
      out[L::P_KS + a] = v;
    }
    double J[D][D], iv[D][D], det;
    for (int r = 0; r < D; ++r)
      for (int c = 0; c < D; ++c) J[r][c] = 0.5 * (X[r + 1][c] - X[0][c]);
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
    for (int a = 0; a < D; ++a)
      for (int b = 0; b < D; ++b) out[L::P_IV + a * D + b] = iv[a][b];
    out[L::P_DET] = det;
    double area[F], nrm[F][D];
    for (int f = 0; f < F; ++f) {
      const int* fv = fnAll + f * NF;  // the face's vertices are its first D nodes
      double Jf[D - 1][D];
      for (int r = 0; r < D - 1; ++r)
        for (int c = 0; c < D; ++c) Jf[r][c] = 0.5 * (X[fv[r + 1]][c] - X[fv[0]][c]);
      double nv[D], ds;
      if (D == 2) {
        ds = sqrt(Jf[0][0] * Jf[0][0] + Jf[0][1] * Jf[0][1]);
        nv[0] = -Jf[0][1];
        nv[1] = Jf[0][0];
      } else {
        const double g00 = Jf[0][0] * Jf[0][0] + Jf[0][1] * Jf[0][1] + Jf[0][2] * Jf[0][2];
        const double g11 = Jf[1][0] * Jf[1][0] + Jf[1][1] * Jf[1][1] + Jf[1][2] * Jf[1][2];
        const double g01 = Jf[0][0] * Jf[1][0] + Jf[0][1] * Jf[1][1] + Jf[0][2] * Jf[1][2];
        ds = sqrt(g00 * g11 - g01 * g01);
        nv[0] = Jf[0][1] * Jf[1][2] - Jf[0][2] * Jf[1][1];
        nv[1] = Jf[0][2] * Jf[1][0] - Jf[0][0] * Jf[1][2];
        nv[2] = Jf[0][0] * Jf[1][1] - Jf[0][1] * Jf[1][0];
      }
      double nn = 0.0;
      for (int a = 0; a < D; ++a) nn += nv[a] * nv[a];
      nn = rsqrt(nn);
      double prod = 0.0;
      for (int a = 0; a < D; ++a) {
        nv[a] *= nn;
        prod += (X[opp[f]][a] - X[fv[0]][a]) * nv[a];
      }
      if (prod > 0)
        for (int a = 0; a < D; ++a) nv[a] = -nv[a];
      area[f] = ds;
      out[L::P_AR + f] = ds;
      for (int a = 0; a < D; ++a) {
        nrm[f][a] = nv[a];
        out[L::P_NRM + f * D + a] = nv[a];
      }
    }
    for (int r = 0; r < D; ++r)
      for (int c = 0; c < D; ++c) {
        double acc = 0.0;
        for (int d = 0; d < D; ++d)
          for (int b = 0; b < D; ++b) acc += K[d][b] * iv[b][r] * iv[d][c];
        out[L::P_GAM + r * D + c] = acc;
      }
    double kn[F][D];
    for (int f = 0; f < F; ++f) {
      for (int r = 0; r < D; ++r) {
        double acc = 0.0;
        for (int d = 0; d < D; ++d)
          for (int b = 0; b < D; ++b) acc += nrm[f][d] * K[d][b] * iv[b][r];
        out[L::P_GV + f * D + r] = acc;
      }
      for (int d = 0; d < D; ++d) {
        double acc = 0.0;
        for (int b = 0; b < D; ++b) acc += K[d][b] * nrm[f][b];
        kn[f][d] = acc;
      }
    }
    for (int f = 0; f < F; ++f)
      for (int g = 0; g < F; ++g) {
        double acc = 0.0;
        for (int d = 0; d < D; ++d) acc += nrm[g][d] * kn[f][d];
        out[L::P_CFF + f * F + g] = area[f] * area[g] / det * acc;
      }
    for (int q = 0; q < NI; ++q) {
      double fval = 0.0;
      if (p.srcMode == 1) fval = p.src[e * NI + q];
      else if (p.srcMode == 2) {
        fval = p.srcParam;
        for (int c = 0; c < D; ++c) {
          double xc = X[0][c];
          for (int r = 0; r < D; ++r) xc += 0.5 * (ipx[q * D + r] + 1.0) * (X[r + 1][c] - X[0][c]);
          fval *= sinpi(xc);  // sin(pi x) without the product's rounding
        }
      }
      out[L::P_FQ + q] = fval * wq[q] * det;
    }
    if (geo) {
      double* ge = geo + e * (D * D + F * D);
      for (int a = 0; a < D; ++a)
        for (int b = 0; b < D; ++b) ge[a * D + b] = iv[a][b];
      for (int f = 0; f < F; ++f)
        for (int a = 0; a < D; ++a) ge[D * D + f * D + a] = area[f] / det * nrm[f][a];
    }
  }
}

// packed symmetric face block (a, b) of face f, rows a <= b of length NF - a
template <int NF>
__device__ __forceinline__ int tm_index(int f, int a, int b) {
  const int lo = a < b ? a : b, hi = a < b ? b : a;
  return f * (NF * (NF + 1) / 2) + lo * NF - lo * (lo - 1) / 2 + (hi - lo);
}
// packed lower triangle by rows, (i, j) with j <= i
__device__ __forceinline__ int pl_index(int i, int j) { return i * (i + 1) / 2 + j; }

template <int D, int P, int EPC>
__global__ void __launch_bounds__(32 * EPC) local_affine(LocalParams p, const double* __restrict__ atab,
                                                         const double* __restrict__ prep) {
  using L = AffLayout<D, P>;
  constexpr int N = L::N, NF = L::NF, F = L::F, NI = L::NI, LL = L::LL;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double* sm = reinterpret_cast<double*>(smem_raw);
  __shared__ int sFN[F * NF];
  __shared__ int sOpp[F];
  __shared__ int sPos[F * N];
  for (int i = threadIdx.x; i < F * NF; i += blockDim.x) sFN[i] = p.itab[i];
  for (int i = threadIdx.x; i < F; i += blockDim.x) sOpp[i] = p.itab[F * NF + i];
  for (int i = threadIdx.x; i < F * N; i += blockDim.x) sPos[i] = -1;
  __syncthreads();
  for (int i = threadIdx.x; i < F * NF; i += blockDim.x) sPos[(i / NF) * N + sFN[i]] = i % NF;
  __syncthreads();

  const int warp = threadIdx.x >> 5, t = threadIdx.x & 31;
  double* W = sm + warp * L::WARP;
  double* pr = W + L::PR;
  double* tau = W + L::TAU;
  const double* Ks = pr + L::P_KS;
  const double* gam = pr + L::P_GAM;
  const double* gv = pr + L::P_GV;
  const double* nrm = pr + L::P_NRM;
  const double* cff = pr + L::P_CFF;
  const double* area = pr + L::P_AR;
  double* Tm = W + L::TM;
  double* Am = W + L::AM;
  double* BW = W + L::BW;
  double* FUv = W + L::FU;
  float2* y0p = reinterpret_cast<float2*>(W + L::Y0P);
  float2* wds = reinterpret_cast<float2*>(W + L::WDS);
  double* rku = W + L::RKU;
  double* rkq = W + L::RKQ;
  double* rkl = W + L::RKL;
  double* rky = W + L::RKY;
  double* rkn = W + L::RKN;
  double* rkg = W + L::RKG;
  const bool rk = p.rkWu != nullptr;
  const double* phi = p.tab + L::T_PHI;
  const double* tM = atab + L::A_M;
  const double* tR = atab + L::A_R;
  const double* tTf = atab + L::A_TF;
  const double* tP = atab + L::A_P;
  const double* tT = atab + L::A_T;
  const double dts = p.dt > 0.0 ? p.dt : 1.0;
  const double cs = rk ? p.cStiff : dts;  // scale of the U rows' stiffness
  const int64_t nWarps = (int64_t)gridDim.x * EPC;
  for (int64_t e = (int64_t)blockIdx.x * EPC + warp; e < p.nCells; e += nWarps) {
    // ------------------------------------- gather: prep record and face tau
    for (int i = t; i < L::P_SMEM; i += 32) pr[i] = prep[e * L::PREP + i];
    const double* fq = prep + e * L::PREP + L::P_FQ;  // read once, from global
    for (int i = t; i < F * NF; i += 32) {
      int f = p.cell2face[e * F + i / NF];
      int side = (p.face2cell[2 * (int64_t)f] == (int)e) ? 0 : 1;
      int q = p.perm[e * F * NF + i];
      tau[i] = p.tau[((int64_t)f * NF + q) * p.tauVals + (p.tauVals == 2 ? side : 0)];
    }
    if (rk) {
      for (int i = t; i < N; i += 32) rku[i] = p.rkWu[e * N + i];
      for (int i = t; i < N * D; i += 32) rkq[i] = p.rkWq[e * N * D + i];
      for (int i = t; i < F * NF; i += 32)
        rkl[i] = p.rkWl[(int64_t)p.cell2face[e * F + i / NF] * NF + p.perm[e * F * NF + i]];
    }
    __syncwarp();
    const double detJ = pr[L::P_DET];
    if (rk) {
      // (K G)[k][r] and K n_f, then y_r[j] = sum_k (K G)[k][r] w_q[j][k]
      const double* iv = pr + L::P_IV;
      if (t < D * D) {
        const int k = t / D, r = t % D;
        double acc = 0.0;
        for (int b = 0; b < D; ++b) acc += Ks[k + b * D] * iv[b * D + r];
        rkg[t] = acc;
      } else if (t >= 16 && t < 16 + F * D) {
        const int f = (t - 16) / D, k = (t - 16) % D;
        double acc = 0.0;
        for (int b = 0; b < D; ++b) acc += Ks[k + b * D] * nrm[f * D + b];
        rkn[t - 16] = acc;
      }
      __syncwarp();
      for (int rj = t; rj < D * N; rj += 32) {
        const int r = rj / N, j = rj % N;
        double acc = 0.0;
        for (int k = 0; k < D; ++k) acc += rkg[k * D + r] * rkq[j * D + k];
        rky[rj] = acc;
      }
    }
    // ----------------------------------------------- tau face mass Tm_f
    // symmetric in (a, b): the upper triangle, mirrored
    constexpr int NT = NF * (NF + 1) / 2;
    for (int idx = t; idx < F * NT; idx += 32) {
      const int f = idx / NT;
      int q = idx % NT, a = 0;
      while (q >= NF - a) {
        q -= NF - a;
        ++a;
      }
      const int b = a + q;
      const double* tf = tTf + (a * NF + b) * NF;
      double acc = 0.0;
#pragma unroll
      for (int c = 0; c < NF; ++c) acc += tau[f * NF + c] * __ldg(tf + c);
      acc *= area[f];
      Tm[f * L::NT + idx % NT] = acc;
    }
    __syncwarp();
    // ------------------------------------------------- A, B and f_u
    for (int lij = t; lij < N * (N + 1) / 2; lij += 32) {
      // lower triangle i >= j, mirrored (A is symmetric)
      int i = (int)((sqrtf(8.0f * lij + 1.0f) - 1.0f) * 0.5f);
      while (i * (i + 1) / 2 > lij) --i;
      while ((i + 1) * (i + 2) / 2 <= lij) ++i;
      const int j = lij - i * (i + 1) / 2;
      const int ij = i * N + j;
      double ts = 0.0;
      for (int f = 0; f < F; ++f) {
        const int a = sPos[f * N + i], b = sPos[f * N + j];
        if (a >= 0 && b >= 0) ts += Tm[tm_index<NF>(f, a, b)];
      }
      double st = 0.0;
#pragma unroll
      for (int rs = 0; rs < D * D; ++rs) st += gam[rs] * __ldg(tR + rs * N * N + ij);
      double v = cs * (ts + detJ * st);
      if (p.dt > 0.0) v += detJ * __ldg(tM + ij);
      Am[pl_index(i, j)] = v;
    }
    for (int i = t; i < N; i += 32) {
      double acc = 0.0;
      for (int q = 0; q < NI; ++q) acc += phi[q * N + i] * fq[q];
      double v = dts * acc;
      if (p.dt > 0.0) {
        double mu = 0.0;
        for (int j = 0; j < N; ++j) mu += __ldg(tM + i * N + j) * p.uOld[e * N + j];
        v += detJ * mu;
      }
      if (rk) {
        // - (K w)_i: tau face masses on (w_u - w_lambda), the flux coupling on w_q
        double kw = 0.0;
        const double* tC = atab + L::A_C;
        const double* tMf = atab + L::A_MF;
        for (int f = 0; f < F; ++f) {
          const int a = sPos[f * N + i];
          if (a < 0) continue;
          for (int b = 0; b < NF; ++b) {
            const int nb = sFN[f * NF + b];
            double qn = 0.0;
            for (int k = 0; k < D; ++k) qn += rkn[f * D + k] * rkq[nb * D + k];
            kw += Tm[tm_index<NF>(f, a, b)] * (rku[nb] - rkl[f * NF + b]) - area[f] * __ldg(tMf + a * NF + b) * qn;
          }
        }
        double vol = 0.0;
        for (int r = 0; r < D; ++r)
          for (int j = 0; j < N; ++j) vol += __ldg(tC + (r * N + i) * N + j) * rky[r * N + j];
        v -= kw + detJ * vol;
      }
      FUv[i] = v;
    }
    __syncwarp();
    // ------------------------------------- Cholesky A = L L^T (lower, in place)
    bool bad = false;
    for (int k = 0; k < N; ++k) {
      const double akk = Am[pl_index(k, k)];
      if (!(akk > 0.0)) bad = true;
      const double il = rsqrt(akk > 0.0 ? akk : 1.0);  // 1 / L[k][k]
      __syncwarp();
      if (t == 0) Am[pl_index(k, k)] = il;  // only 1 / L[k][k] is used from here on
      for (int i = k + 1 + t; i < N; i += 32) Am[pl_index(i, k)] *= il;
      __syncwarp();
      const int m = N - k - 1;
      for (int idx = t; idx < m * (m + 1) / 2; idx += 32) {
        // packed lower triangle of the trailing block: row ii >= column jj
        int ii = (int)((sqrtf(8.0f * idx + 1.0f) - 1.0f) * 0.5f);
        while (ii * (ii + 1) / 2 > idx) --ii;
        while ((ii + 1) * (ii + 2) / 2 <= idx) ++ii;
        const int i = k + 1 + ii, j = k + 1 + (idx - ii * (ii + 1) / 2);
        Am[pl_index(i, j)] -= Am[pl_index(i, k)] * Am[pl_index(j, k)];
      }
      __syncwarp();
    }
    if (bad && t == 0) atomicCAS(p.status, 0, 1);
    // ---------------- two passes over the columns of B ([0, H0), then the rest
    // with f_u): each forms its columns of B, forward- and back-substitutes them
    // in FP64 ([W | y0] = L^{-1} [B | f_u], then L^{-T}), keeps W as double-float
    // pairs for S and writes its columns of U = -dt L^{-T} W (and U0).
    double* Ug = (double*)p.U + e * N * LL;
    constexpr int LWH = L::LWH;
    for (int h = 0; h < 2; ++h) {
      const int c0 = h ? L::H0 : 0, nc = h ? LL - L::H0 : L::H0, wc = nc + h;
      for (int ic = t; ic < N * nc; ic += 32) {
        const int i = ic / nc, cl = ic % nc, c = c0 + cl;
        const int f = c / NF, b = c % NF;
        double acc = 0.0;
#pragma unroll
        for (int r = 0; r < D; ++r) acc += gv[f * D + r] * __ldg(tP + ((r * F + f) * N + i) * NF + b);
        double v = -area[f] * acc;
        const int a = sPos[f * N + i];
        if (a >= 0) v -= Tm[tm_index<NF>(f, a, b)];
        BW[i * LWH + cl] = v;
      }
      if (h)
        for (int i = t; i < N; i += 32) BW[i * LWH + nc] = FUv[i];
      __syncwarp();
      // forward, row-oriented: after row k is final every lane updates (row, column)
      // pairs below it, so all 32 lanes stay busy whatever the column count
      for (int k = 0; k < N; ++k) {
        const double ik = Am[pl_index(k, k)];
        for (int c = t; c < wc; c += 32) BW[k * LWH + c] *= ik;
        __syncwarp();
        const int rows = N - k - 1;
        for (int ic = t; ic < rows * wc; ic += 32) {
          const int i = k + 1 + ic / wc, c = ic % wc;
          BW[i * LWH + c] -= Am[pl_index(i, k)] * BW[k * LWH + c];
        }
        __syncwarp();
      }
      if (!p.explicitMode) {
        for (int idx = t; idx < N * nc; idx += 32) {
          const int m = idx / nc, cl = idx % nc;
          const double w = BW[m * LWH + cl];
          const float hi = __double2float_rn(w);
          wds[m * LL + c0 + cl] = make_float2(hi, __double2float_rn(w - (double)hi));
        }
        if (h)
          for (int m = t; m < N; m += 32) {
            const double y = BW[m * LWH + nc];
            const float hi = __double2float_rn(y);
            y0p[m] = make_float2(hi, __double2float_rn(y - (double)hi));
          }
      }
      __syncwarp();
      // back substitution in place: rows above k get BW[i] -= L[k][i] x_k
      for (int k = N - 1; k >= 0; --k) {
        const double ik = Am[pl_index(k, k)];
        for (int c = t; c < wc; c += 32) BW[k * LWH + c] *= ik;
        __syncwarp();
        for (int ic = t; ic < k * wc; ic += 32) {
          const int i = ic / wc, c = ic % wc;
          BW[i * LWH + c] -= Am[pl_index(k, i)] * BW[k * LWH + c];
        }
        __syncwarp();
      }
      for (int idx = t; idx < N * nc; idx += 32) {
        const int i = idx % N, cl = idx / N;
        Ug[(c0 + cl) * N + i] = -cs * BW[i * LWH + cl];
      }
      if (h)
        for (int i = t; i < N; i += 32) ((double*)p.U0)[e * N + i] = BW[i * LWH + nc];
      __syncwarp();
    }
    // ------------------ S = C + dt W^T W (upper triangle, mirrored), S0 = W^T y0
    {
      double* Sg = (double*)p.S + e * LL * LL;
      unsigned bmask = 0;  // bit f: face f of the cell is a Dirichlet face
      for (int f = 0; f < F; ++f)
        if (p.isBoundary[p.cell2face[e * F + f]]) bmask |= 1u << f;
      if (p.explicitMode) {
        // explicit modes: S = Sll (block diagonal), S0 = -Slu sol + Hm flux
        for (int idx = t; idx < LL * LL; idx += 32) {
          const int r = idx % LL, c = idx / LL, fr = r / NF;
          double v;
          if ((bmask >> fr) & 1u) v = r == c ? 1.0 : 0.0;
          else v = (c / NF == fr) ? -Tm[tm_index<NF>(fr, r % NF, c % NF)] : 0.0;
          Sg[idx] = v;
        }
        const double* sol = p.solState + e * N;
        const double* flx = p.fluxState + e * N * D;
        for (int c = t; c < LL; c += 32) {
          const int f = c / NF, a = c % NF;
          double v;
          if ((bmask >> f) & 1u) {
            v = p.dirichlet[(int64_t)p.cell2face[e * F + f] * NF + a];
          } else {
            double kn[D];
            for (int dd = 0; dd < D; ++dd) {
              double acc = 0.0;
              for (int b2 = 0; b2 < D; ++b2) acc += Ks[dd + b2 * D] * nrm[f * D + b2];
              kn[dd] = acc;
            }
            v = 0.0;
            for (int b = 0; b < NF; ++b) {
              const int nb = sFN[f * NF + b];
              double mf = 0.0;  // face mass: sum_c T_f[a][b][c] (the face shapes sum to 1)
              for (int cc = 0; cc < NF; ++cc) mf += __ldg(tTf + (a * NF + b) * NF + cc);
              double qn = 0.0;
              for (int dd = 0; dd < D; ++dd) qn += kn[dd] * flx[nb * D + dd];
              v += -Tm[tm_index<NF>(f, a, b)] * sol[nb] + area[f] * mf * qn;
            }
          }
          ((double*)p.S0)[e * LL + c] = v;
        }
      }
      for (int idx = t; !p.explicitMode && idx < LL * (LL + 1) / 2; idx += 32) {
        // column c, row r <= c, column-major packing of the upper triangle
        int c = (int)((sqrtf(8.0f * idx + 1.0f) - 1.0f) * 0.5f);
        while (c * (c + 1) / 2 > idx) --c;
        while ((c + 1) * (c + 2) / 2 <= idx) ++c;
        const int r = idx - c * (c + 1) / 2;
        const int fr = r / NF, fc = c / NF;
        float sh = 0.f, sl = 0.f;
#pragma unroll 4
        for (int m = 0; m < N; ++m) ds_mac(sh, sl, wds[m * LL + r], wds[m * LL + c]);
        double v = ((double)sh + (double)sl) * cs;
        v -= cff[fr * F + fc] * __ldg(tT + ((fr * F + fc) * NF + (r % NF)) * NF + (c % NF));
        if (fr == fc) v -= Tm[tm_index<NF>(fr, r % NF, c % NF)];
        const bool br = (bmask >> fr) & 1u;
        const bool bc = (bmask >> fc) & 1u;
        // Dirichlet Set: boundary rows become identity rows (columns are kept)
        Sg[r + c * LL] = br ? (r == c ? 1.0 : 0.0) : v;
        if (r != c) Sg[c + r * LL] = bc ? 0.0 : v;
      }
      for (int c = t; !p.explicitMode && c < LL; c += 32) {
        const int f = c / NF;
        double v;
        if ((bmask >> f) & 1u) {
          v = p.dirichlet[(int64_t)p.cell2face[e * F + f] * NF + c % NF];
        } else {
          float sh = 0.f, sl = 0.f;  // S0 = W^T y0
          for (int m = 0; m < N; ++m) ds_mac(sh, sl, wds[m * LL + c], y0p[m]);
          v = (double)sh + (double)sl;
        }
        ((double*)p.S0)[e * LL + c] = v;
      }
    }
    __syncwarp();
    __syncwarp();
  }
}

// Recovery for the affine path: sol = U lambda + U0, flux = -Xu sol - Xl lambda,
// with the products shared: t_s = M^{-1} C_s sol and l_f = L_f lambda_f once
// per element, then flux(i, d) = -sum_s G[d][s] t_s[i] + sum_f g_f[d] l_f[i].
template <int D, int P>
__global__ void recover_affine(RecoverParams p, const double* __restrict__ atab, const double* __restrict__ geo) {
  using L = AffLayout<D, P>;
  constexpr int N = L::N, NF = L::NF, F = L::F, LL = L::LL;
  __shared__ double lam[LL];
  __shared__ double sol[N];
  __shared__ double ts[D * N];
  __shared__ double lf[F * N];
  __shared__ double ge[D * D + F * D];
  const double* tD = atab + L::A_D;
  const double* tL = atab + L::A_L;
  for (int64_t e = blockIdx.x; e < p.nCells; e += gridDim.x) {
    for (int j = threadIdx.x; j < LL; j += blockDim.x) {
      int i = j / NF;
      int f = p.cell2face[e * F + i];
      lam[j] = p.trace[(int64_t)f * NF + p.perm[(e * F + i) * NF + (j % NF)]];
    }
    for (int j = threadIdx.x; j < D * D + F * D; j += blockDim.x) ge[j] = geo[e * (D * D + F * D) + j];
    __syncthreads();
    for (int r = threadIdx.x; r < N; r += blockDim.x) {
      const double* U = p.U + e * N * LL;
      double acc = p.U0[e * N + r];
      for (int c = 0; c < LL; ++c) acc += U[r + (int64_t)c * N] * lam[c];
      sol[r] = acc;
      p.sol[e * N + r] = acc;
    }
    for (int fi = threadIdx.x; fi < F * N; fi += blockDim.x) {
      const int f = fi / N, i = fi % N;
      double acc = 0.0;
      for (int b = 0; b < NF; ++b) acc += __ldg(tL + (f * N + i) * NF + b) * lam[f * NF + b];
      lf[fi] = acc;
    }
    __syncthreads();
    for (int si = threadIdx.x; si < D * N; si += blockDim.x) {
      const int sd = si / N, i = si % N;
      double acc = 0.0;
      for (int j = 0; j < N; ++j) acc += __ldg(tD + (sd * N + i) * N + j) * sol[j];
      ts[si] = acc;
    }
    __syncthreads();
    for (int r = threadIdx.x; r < N * D; r += blockDim.x) {
      const int i = r / D, d = r % D;  // flux node-major (i, d)
      double acc = 0.0;
      for (int sd = 0; sd < D; ++sd) acc -= ge[d * D + sd] * ts[sd * N + i];
      for (int f = 0; f < F; ++f) acc += ge[D * D + f * D + d] * lf[f * N + i];
      p.flux[e * N * D + r] = acc;
    }
    __syncthreads();
  }
}

// Q = -Xu U - Xl, Q0 = -Xu U0 (column-major LQ x LL, rows node-major (i, d)), for exports.
template <int D, int P>
__global__ void q_from_u(int nCells, const double* __restrict__ U, const double* __restrict__ U0,
                         const double* __restrict__ atab, const double* __restrict__ geo, double* Q, double* Q0) {
  using L = AffLayout<D, P>;
  constexpr int N = L::N, NF = L::NF, F = L::F, LL = L::LL, LQ = D * N;
  const double* tD = atab + L::A_D;
  const double* tL = atab + L::A_L;
  const int64_t total = (int64_t)nCells * LQ * (LL + 1);
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = idx / (LQ * (LL + 1));
    const int rc = (int)(idx % (LQ * (LL + 1)));
    const int c = rc / LQ, row = rc % LQ;
    const int i = row / D, d = row % D;
    const double* ge = geo + e * (D * D + F * D);
    const double* u = c < LL ? U + e * N * LL + (int64_t)c * N : U0 + e * N;
    double acc = 0.0;
    for (int s = 0; s < D; ++s) {
      double ds = 0.0;
      for (int j = 0; j < N; ++j) ds += tD[(s * N + i) * N + j] * u[j];
      acc -= ge[d * D + s] * ds;
    }
    if (c < LL) {
      const int f = c / NF, b = c % NF;
      acc += ge[D * D + f * D + d] * tL[(f * N + i) * NF + b];
      Q[e * LQ * LL + (int64_t)c * LQ + row] = acc;
    } else {
      Q0[e * LQ + row] = acc;
    }
  }
}

unsigned grid_cap(int64_t n, int threads) {
  int64_t g = (n + threads - 1) / threads;
  if (g > 152 * 64) g = 152 * 64;
  return (unsigned)(g < 1 ? 1 : g);
}

template <int D, int P>
cudaError_t launch_affine_t(const LocalParams& p, const double* atab, double* geo, double* prep, cudaStream_t s) {
  using L = AffLayout<D, P>;
  // warps (elements) per block: 4 when a warp's region is large, so that the
  // shared memory of an SM is used by several blocks without a remainder
  constexpr int EPC = L::WARP * 8 * 8 > 96 * 1024 ? 4 : 8;
  affine_prep<D, P><<<grid_cap(p.nCells, 128), 128, 0, s>>>(p, atab, prep, geo);
  size_t smem = (size_t)EPC * L::WARP * sizeof(double);
  auto kern = local_affine<D, P, EPC>;
  cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (err != cudaSuccess) return err;
  int dev = 0, nsm = 0, perSM = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, kern, 32 * EPC, smem);
  if (err != cudaSuccess) return err;
  if (perSM < 1) perSM = 1;
  int64_t need = (p.nCells + EPC - 1) / EPC;
  int64_t grid = (int64_t)nsm * perSM;
  if (grid > need) grid = need;
  if (grid < 1) grid = 1;
  kern<<<(unsigned)grid, 32 * EPC, smem, s>>>(p, atab, prep);
  return cudaGetLastError();
}

}  // namespace

#define HFX_AFFINE_DISPATCH(FN, ...)                          \
  if (dim == 2) {                                             \
    switch (order) {                                          \
      case 1: return FN<2, 1>(__VA_ARGS__);                   \
      case 2: return FN<2, 2>(__VA_ARGS__);                   \
      case 3: return FN<2, 3>(__VA_ARGS__);                   \
      case 4: return FN<2, 4>(__VA_ARGS__);                   \
      case 5: return FN<2, 5>(__VA_ARGS__);                   \
    }                                                         \
  } else if (dim == 3) {                                      \
    switch (order) {                                          \
      case 1: return FN<3, 1>(__VA_ARGS__);                   \
      case 2: return FN<3, 2>(__VA_ARGS__);                   \
      case 3: return FN<3, 3>(__VA_ARGS__);                   \
    }                                                         \
  }                                                           \
  return cudaErrorInvalidValue;

cudaError_t launch_local_affine(int dim, int order, const LocalParams& p, const double* atab, double* geo,
                                double* prep, cudaStream_t s) {
  HFX_AFFINE_DISPATCH(launch_affine_t, p, atab, geo, prep, s)
}

namespace {
template <int D, int P>
int64_t affine_prep_doubles_t() {
  return AffLayout<D, P>::PREP;
}
}  // namespace

int64_t affine_prep_doubles(int dim, int order) {
  if (dim == 2 && order >= 1 && order <= 5) {
    const int64_t v[] = {affine_prep_doubles_t<2, 1>(), affine_prep_doubles_t<2, 2>(), affine_prep_doubles_t<2, 3>(),
                         affine_prep_doubles_t<2, 4>(), affine_prep_doubles_t<2, 5>()};
    return v[order - 1];
  }
  if (dim == 3 && order >= 1 && order <= 3) {
    const int64_t v[] = {affine_prep_doubles_t<3, 1>(), affine_prep_doubles_t<3, 2>(), affine_prep_doubles_t<3, 3>()};
    return v[order - 1];
  }
  return 0;
}

namespace {
template <int D, int P>
cudaError_t launch_recover_affine_t(const RecoverParams& p, const double* atab, const double* geo, cudaStream_t s) {
  int64_t grid = p.nCells < 152 * 64 ? p.nCells : 152 * 64;
  recover_affine<D, P><<<(unsigned)(grid < 1 ? 1 : grid), 64, 0, s>>>(p, atab, geo);
  return cudaGetLastError();
}
template <int D, int P>
cudaError_t launch_q_from_u_t(int nCells, const double* U, const double* U0, const double* atab, const double* geo,
                              double* Q, double* Q0, cudaStream_t s) {
  using L = AffLayout<D, P>;
  const int64_t total = (int64_t)nCells * D * L::N * (L::LL + 1);
  q_from_u<D, P><<<grid_cap(total, 256), 256, 0, s>>>(nCells, U, U0, atab, geo, Q, Q0);
  return cudaGetLastError();
}
}  // namespace

cudaError_t launch_recover_affine(int dim, int order, const RecoverParams& p, const double* atab, const double* geo,
                                  cudaStream_t s) {
  HFX_AFFINE_DISPATCH(launch_recover_affine_t, p, atab, geo, s)
}

cudaError_t launch_q_from_u(int dim, int order, int nCells, const double* U, const double* U0, const double* atab,
                            const double* geo, double* Q, double* Q0, cudaStream_t s) {
  HFX_AFFINE_DISPATCH(launch_q_from_u_t, nCells, U, U0, atab, geo, Q, Q0, s)
}

}  // namespace hfx
