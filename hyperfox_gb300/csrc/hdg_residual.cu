// FP64 residual of the full (uncondensed) HDG system, matrix free.
//
// For every element, r = b - A_loc [u; q; lambda] with A_loc the element
// matrix HyperFox assembles (HDGBase.cpp:67-158 + HDGDiffusion.cpp:74-145,
// Source.cpp:24-48, implicit Euler on the U rows Euler.cpp:18-34), applied
// through the integration points instead of being formed: values and
// gradients of u and q at the volume IPs, traces of u, q and lambda at the face
// IPs, then the transposed evaluations. Costs O(nIP * N * d) per element
// instead of O(n_loc^2), in FP64.
//
// Outputs the element rows (r_u, r_q) and the element's contribution to the
// face rows (r_l, local face-node order), which face_residual() assembles per
// face (Dirichlet faces: g - lambda, the Set rows of HDGSolver.cpp:493-501).
// This is the FP64 "refinement residual" of the mixed-precision solve and the
// final residual check.
#include "hfx_device.h"
#include "hdg_mixed.h"

namespace hfx {
namespace {

template <int D, int P, int TPE, int EPC>
struct RLayout {
  using K = Dims<D, P>;
  static constexpr int N = K::N, NF = K::NF, F = K::F, NI = K::NI, NIF = K::NIF, LL = K::LL, DM = D - 1;
  static constexpr int T_PHI = 0, T_DPHI = NI * N, T_W = T_DPHI + NI * N * D, T_FPHI = T_W + NI;
  static constexpr int T_FDPHI = T_FPHI + NIF * NF, T_FW = T_FDPHI + NIF * NF * DM;
  static constexpr int TAB = (T_FW + NIF + 1) & ~1;
  // group region
  static constexpr int X = 0;
  static constexpr int KAPN = X + N * D;
  static constexpr int U = KAPN + N * D * D;       // u (N)
  static constexpr int Q = U + N;                  // q (N*D), node-major
  static constexpr int L = Q + N * D;              // lambda local (LL)
  static constexpr int UQ = L + LL;                // u at IPs, q at IPs: NI*(1+D)
  static constexpr int GV = UQ + NI * (1 + D);     // per IP: dV, invJ (D*D), kappa (D*D), f
  static constexpr int GVSZ = 2 + 2 * D * D;
  static constexpr int FV = GV + NI * GVSZ;        // per face IP: dS*tau, dS*n (D), dS*kappa*n (D), uhat, lhat, qhat(D)
  static constexpr int FVSZ = 3 + 3 * D;
  static constexpr int GROUP = (FV + F * NIF * FVSZ + 1) & ~1;
  static constexpr int TOTAL = TAB + EPC * GROUP;
};

template <int D, int P, int TPE, int EPC>
__global__ void __launch_bounds__(TPE * EPC) residual_f64(ResidualParams p) {
  using L = RLayout<D, P, TPE, EPC>;
  constexpr int N = L::N, NF = L::NF, F = L::F, NI = L::NI, NIF = L::NIF, LL = L::LL, DM = L::DM;
  extern __shared__ double smem[];
  __shared__ int sFaceNodes[F * NF];
  __shared__ int sOpp[F];
  const int nthr = TPE * EPC;
  for (int i = threadIdx.x; i < L::T_FW + NIF; i += nthr) smem[i] = p.tab[i];
  for (int i = threadIdx.x; i < F * NF; i += nthr) sFaceNodes[i] = p.itab[i];
  for (int i = threadIdx.x; i < F; i += nthr) sOpp[i] = p.itab[F * NF + i];
  __syncthreads();
  const double* phi = smem + L::T_PHI;
  const double* dphi = smem + L::T_DPHI;
  const double* w = smem + L::T_W;
  const double* fphi = smem + L::T_FPHI;
  const double* fdphi = smem + L::T_FDPHI;
  const double* fw = smem + L::T_FW;
  const int grp = threadIdx.x / TPE, t = threadIdx.x % TPE;
  double* R = smem + L::TAB + grp * L::GROUP;
  double* X = R + L::X;
  double* kapN = R + L::KAPN;
  double* u = R + L::U;
  double* q = R + L::Q;
  double* lam = R + L::L;
  double* uq = R + L::UQ;   // [NI][1+D]
  double* gv = R + L::GV;   // [NI][GVSZ]
  double* fv = R + L::FV;   // [F*NIF][FVSZ]
  const double dts = p.dt > 0.0 ? p.dt : 1.0;
  const int64_t nGroups = (int64_t)gridDim.x * EPC;
  for (int64_t base = (int64_t)blockIdx.x * EPC; base < p.nCells; base += nGroups) {
    const int64_t e = base + grp;
    const bool active = e < p.nCells;
    if (active) {
      const int* cell = p.cells + e * N;
      for (int i = t; i < N * D; i += TPE) X[i] = p.coords[(int64_t)cell[i / D] * D + (i % D)];
      for (int i = t; i < N * D * D; i += TPE) {
        int n = i / (D * D), a = i % (D * D);
        double v;
        if (p.kc == 0) v = (a % (D + 1) == 0) ? 1.0 : 0.0;
        else {
          int64_t bk = p.kappaLayout == 0 ? (int64_t)cell[n] * p.kc : (e * N + n) * p.kc;
          v = p.kc == 1 ? ((a % (D + 1) == 0) ? p.kappa[bk] : 0.0) : p.kappa[bk + a];
        }
        kapN[i] = v;
      }
      for (int i = t; i < N; i += TPE) u[i] = p.sol[e * N + i];
      for (int i = t; i < N * D; i += TPE) q[i] = p.flux[e * N * D + i];
      for (int i = t; i < LL; i += TPE) {
        int f = p.cell2face[e * F + i / NF];
        lam[i] = p.trace[(int64_t)f * NF + p.perm[e * F * NF + i]];
      }
    }
    __syncthreads();
    if (active) {
      // volume IPs: geometry, kappa, source; u and q values
      for (int qi = t; qi < NI; qi += TPE) {
        double J[D][D];
        for (int r = 0; r < D; ++r)
          for (int s = 0; s < D; ++s) {
            double acc = 0.0;
            for (int i = 0; i < N; ++i) acc += dphi[(qi * N + i) * D + r] * X[i * D + s];
            J[r][s] = acc;
          }
        double det, iv[D][D];
        if (D == 2) {
          det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
          double id = 1.0 / det;
          iv[0][0] = J[1][1] * id;
          iv[0][1] = -J[0][1] * id;
          iv[1][0] = -J[1][0] * id;
          iv[1][1] = J[0][0] * id;
        } else {
          double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
          double c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
          double c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
          det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
          double id = 1.0 / det;
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
        double* g = gv + qi * L::GVSZ;
        g[0] = w[qi] * det;
        for (int a = 0; a < D; ++a)
          for (int b = 0; b < D; ++b) g[1 + a * D + b] = iv[a][b];
        for (int a = 0; a < D * D; ++a) {
          double acc = 0.0;
          for (int i = 0; i < N; ++i) acc += phi[qi * N + i] * kapN[i * D * D + a];
          g[1 + D * D + a] = acc;
        }
        double fval = 0.0;
        if (p.srcMode == 1) fval = p.src[e * NI + qi];
        else if (p.srcMode == 2) {
          fval = p.srcParam;
          for (int k = 0; k < D; ++k) {
            double xk = 0.0;
            for (int i = 0; i < N; ++i) xk += phi[qi * N + i] * X[i * D + k];
            fval *= sin(M_PI * xk);
          }
        }
        g[1 + 2 * D * D] = fval;
        double uv = 0.0;
        for (int i = 0; i < N; ++i) uv += phi[qi * N + i] * u[i];
        uq[qi * (1 + D)] = uv;
        for (int d = 0; d < D; ++d) {
          double qv = 0.0;
          for (int i = 0; i < N; ++i) qv += phi[qi * N + i] * q[i * D + d];
          uq[qi * (1 + D) + 1 + d] = qv;
        }
      }
      // face IPs: measure, normal, tau, kappa*n and the traces of u, q, lambda
      for (int fk = t; fk < F * NIF; fk += TPE) {
        int f = fk / NIF, k = fk % NIF;
        double Jf[D - 1][D];
        for (int r = 0; r < DM; ++r)
          for (int s = 0; s < D; ++s) {
            double acc = 0.0;
            for (int i = 0; i < NF; ++i) acc += fdphi[(k * NF + i) * DM + r] * X[sFaceNodes[f * NF + i] * D + s];
            Jf[r][s] = acc;
          }
        double nv[D], ds;
        if (D == 2) {
          ds = sqrt(Jf[0][0] * Jf[0][0] + Jf[0][1] * Jf[0][1]);
          nv[0] = -Jf[0][1];
          nv[1] = Jf[0][0];
        } else {
          double g00 = Jf[0][0] * Jf[0][0] + Jf[0][1] * Jf[0][1] + Jf[0][2] * Jf[0][2];
          double g11 = Jf[1][0] * Jf[1][0] + Jf[1][1] * Jf[1][1] + Jf[1][2] * Jf[1][2];
          double g01 = Jf[0][0] * Jf[1][0] + Jf[0][1] * Jf[1][1] + Jf[0][2] * Jf[1][2];
          ds = sqrt(g00 * g11 - g01 * g01);
          nv[0] = Jf[0][1] * Jf[1][2] - Jf[0][2] * Jf[1][1];
          nv[1] = Jf[0][2] * Jf[1][0] - Jf[0][0] * Jf[1][2];
          nv[2] = Jf[0][0] * Jf[1][1] - Jf[0][1] * Jf[1][0];
        }
        double nn = 0.0;
        for (int a = 0; a < D; ++a) nn += nv[a] * nv[a];
        nn = 1.0 / sqrt(nn);
        double prod = 0.0;
        int v0 = sFaceNodes[f * NF], vn = sOpp[f];
        for (int a = 0; a < D; ++a) {
          nv[a] *= nn;
          prod += (X[vn * D + a] - X[v0 * D + a]) * nv[a];
        }
        if (prod > 0)
          for (int a = 0; a < D; ++a) nv[a] = -nv[a];
        ds *= fw[k];
        // tau at the face IP, from the local tau (double valued side and face order)
        double tq = 0.0;
        {
          int fid = p.cell2face[e * F + f];
          int side = (p.face2cell[2 * (int64_t)fid] == (int)e) ? 0 : 1;
          for (int i = 0; i < NF; ++i) {
            int qpos = p.perm[e * F * NF + f * NF + i];
            double ti = p.tau[((int64_t)fid * NF + qpos) * p.tauVals + (p.tauVals == 2 ? side : 0)];
            tq += fphi[k * NF + i] * ti;
          }
        }
        double* fr = fv + fk * L::FVSZ;
        fr[0] = ds * tq;
        for (int a = 0; a < D; ++a) fr[1 + a] = ds * nv[a];
        for (int a = 0; a < D; ++a) {
          double acc = 0.0;
          for (int b = 0; b < D; ++b) {
            double kab = 0.0;
            for (int i = 0; i < NF; ++i) kab += fphi[k * NF + i] * kapN[sFaceNodes[f * NF + i] * D * D + a + b * D];
            acc += kab * nv[b];
          }
          fr[1 + D + a] = ds * acc;
        }
        double uh = 0.0, lh = 0.0, qh[D];
        for (int d = 0; d < D; ++d) qh[d] = 0.0;
        for (int i = 0; i < NF; ++i) {
          double ps = fphi[k * NF + i];
          int n = sFaceNodes[f * NF + i];
          uh += ps * u[n];
          lh += ps * lam[f * NF + i];
          for (int d = 0; d < D; ++d) qh[d] += ps * q[n * D + d];
        }
        fr[1 + 2 * D] = uh;
        fr[2 + 2 * D] = lh;
        for (int d = 0; d < D; ++d) fr[3 + 2 * D + d] = qh[d];
      }
    }
    __syncthreads();
    if (active) {
      // U rows: r_u = dt f_u (+ M uOld) - [dt (Suu u + Suq q + Sul lam) (+ M u)]
      for (int i = t; i < N; i += TPE) {
        double fu = 0.0, mass = 0.0, vol = 0.0;
        for (int qi = 0; qi < NI; ++qi) {
          const double* g = gv + qi * L::GVSZ;
          double dv = g[0];
          fu += phi[qi * N + i] * g[1 + 2 * D * D] * dv;
          // Suq volume: sum_d (kappa J^{-1} grad phi_i)_d dV q_d(ip)
          double gi[D];
          for (int a = 0; a < D; ++a) {
            double acc = 0.0;
            for (int b = 0; b < D; ++b) acc += g[1 + a * D + b] * dphi[(qi * N + i) * D + b];
            gi[a] = acc;
          }
          for (int a = 0; a < D; ++a) {
            double kg = 0.0;
            for (int b = 0; b < D; ++b) kg += g[1 + D * D + a + b * D] * gi[b];
            vol += kg * dv * uq[qi * (1 + D) + 1 + a];
          }
          mass += dv * phi[qi * N + i] * uq[qi * (1 + D)];
        }
        double face = 0.0;
        for (int f = 0; f < F; ++f) {
          int a = -1;
          for (int j = 0; j < NF; ++j)
            if (sFaceNodes[f * NF + j] == i) a = j;
          if (a < 0) continue;
          for (int k = 0; k < NIF; ++k) {
            const double* fr = fv + (f * NIF + k) * L::FVSZ;
            double ps = fphi[k * NF + a];
            double kq = 0.0;
            for (int d = 0; d < D; ++d) kq += fr[1 + D + d] * fr[3 + 2 * D + d];
            // Suu u - Sul lam = tau (u - lam); Suq face = -kappa n . q
            face += ps * (fr[0] * (fr[1 + 2 * D] - fr[2 + 2 * D]) - kq);
          }
        }
        double Au = vol + face;
        double r;
        if (p.dt > 0.0) {
          double mo = 0.0;  // M uOld
          for (int qi = 0; qi < NI; ++qi) {
            double uo = 0.0;
            for (int j = 0; j < N; ++j) uo += phi[qi * N + j] * p.uOld[e * N + j];
            mo += gv[qi * L::GVSZ] * phi[qi * N + i] * uo;
          }
          r = dts * fu + mo - (dts * Au + mass);
        } else {
          r = fu - Au;
        }
        p.ru[e * N + i] = r;
      }
      // Q rows: r_q = -(Squ u + Sqq q + Sql lam)
      for (int id = t; id < N * D; id += TPE) {
        int i = id / D, d = id % D;
        double acc = 0.0;
        for (int qi = 0; qi < NI; ++qi) {
          const double* g = gv + qi * L::GVSZ;
          double gid = 0.0;
          for (int b = 0; b < D; ++b) gid += g[1 + d * D + b] * dphi[(qi * N + i) * D + b];
          acc += g[0] * (gid * uq[qi * (1 + D)] + phi[qi * N + i] * uq[qi * (1 + D) + 1 + d]);
        }
        for (int f = 0; f < F; ++f) {
          int a = -1;
          for (int j = 0; j < NF; ++j)
            if (sFaceNodes[f * NF + j] == i) a = j;
          if (a < 0) continue;
          for (int k = 0; k < NIF; ++k) {
            const double* fr = fv + (f * NIF + k) * L::FVSZ;
            acc -= fphi[k * NF + a] * fr[1 + d] * fr[2 + 2 * D];  // Sql = -n phi phi
          }
        }
        p.rq[e * N * D + id] = -acc;
      }
      // face rows (element contribution): r_l = -(Slu u + Slq q + Sll lam)
      for (int row = t; row < LL; row += TPE) {
        int f = row / NF, a = row % NF;
        double acc = 0.0;
        for (int k = 0; k < NIF; ++k) {
          const double* fr = fv + (f * NIF + k) * L::FVSZ;
          double kq = 0.0;
          for (int d = 0; d < D; ++d) kq += fr[1 + D + d] * fr[3 + 2 * D + d];
          acc += fphi[k * NF + a] * (fr[0] * (fr[1 + 2 * D] - fr[2 + 2 * D]) - kq);
        }
        p.rl[e * LL + row] = -acc;
      }
    }
    __syncthreads();
  }
}

// Face rows: interior faces sum their two element contributions (lower cell
// first); Dirichlet faces give g - lambda.
__global__ void face_residual(FaceResidualParams p) {
  const int NF = p.NF, F = p.F, LL = p.LL;
  const int64_t total = (int64_t)p.nFaces * NF;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    int f = (int)(idx / NF), a = (int)(idx % NF);
    double v = 0.0;
    if (p.isBnd[f]) {
      v = p.dirichlet[idx] - p.trace[idx];
    } else {
      for (int s = 0; s < 2; ++s) {
        int c = p.face2cell[2 * (int64_t)f + s];
        if (c < 0) continue;
        int li = 0;
        for (int i = 0; i < F; ++i)
          if (p.cell2face[(int64_t)c * F + i] == f) li = i;
        const uint8_t* pi = p.perm + ((int64_t)c * F + li) * NF;
        int ja = 0;
        for (int j = 0; j < NF; ++j)
          if (pi[j] == a) ja = j;
        v += p.rl[(int64_t)c * LL + li * NF + ja];
      }
    }
    p.rtrace[idx] = v;
  }
}

template <int D, int P, int TPE, int EPC>
cudaError_t launch_r(const ResidualParams& p, cudaStream_t s) {
  using L = RLayout<D, P, TPE, EPC>;
  size_t smem = (size_t)L::TOTAL * sizeof(double);
  auto kern = residual_f64<D, P, TPE, EPC>;
  cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (err != cudaSuccess) return err;
  int dev = 0, nsm = 0, perSM = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, kern, TPE * EPC, smem);
  if (perSM < 1) perSM = 1;
  int64_t need = (p.nCells + EPC - 1) / EPC, grid = (int64_t)nsm * perSM;
  if (grid > need) grid = need;
  kern<<<(unsigned)(grid < 1 ? 1 : grid), TPE * EPC, smem, s>>>(p);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_residual(int dim, int order, const ResidualParams& p, const FaceResidualParams& fp,
                            cudaStream_t s) {
  cudaError_t e = cudaErrorInvalidValue;
  if (dim == 2) {
    switch (order) {
      case 1: e = launch_r<2, 1, 32, 8>(p, s); break;
      case 2: e = launch_r<2, 2, 32, 8>(p, s); break;
      case 3: e = launch_r<2, 3, 32, 8>(p, s); break;
      case 4: e = launch_r<2, 4, 64, 4>(p, s); break;
      case 5: e = launch_r<2, 5, 64, 4>(p, s); break;
    }
  } else if (dim == 3) {
    switch (order) {
      case 1: e = launch_r<3, 1, 32, 8>(p, s); break;
      case 2: e = launch_r<3, 2, 64, 4>(p, s); break;
      case 3: e = launch_r<3, 3, 64, 4>(p, s); break;
    }
  }
  if (e != cudaSuccess) return e;
  int64_t total = (int64_t)fp.nFaces * fp.NF;
  unsigned g = (unsigned)((total + 255) / 256);
  if (g > 152 * 64) g = 152 * 64;
  face_residual<<<g < 1 ? 1 : g, 256, 0, s>>>(fp);
  return cudaGetLastError();
}

}  // namespace hfx
